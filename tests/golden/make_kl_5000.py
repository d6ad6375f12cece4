"""Golden KL curves of the compiled reference (oracle/_ref, the unmodified sources) on a
5,000-point problem, for the final-KL-within-1% test.  The data are regenerated from the
seed by the test itself (numpy's default_rng is the same on every platform), so only the
costs are stored.

    python tests/golden/make_kl_5000.py   (needs the reference tree: make -C oracle ref)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))

N, D, SEED = 5000, 20, 21
CASES = {"df1": dict(perplexity=30.0), "df05_late": dict(perplexity=20.0, df=0.5, start_late_exag_iter=300,
                                                         late_exag_coeff=2.0)}
COMMON = dict(no_dims=2, max_iter=500, stop_lying_iter=250, mom_switch_iter=250, learning_rate=N / 12.0)


def data():
    rng = np.random.default_rng(SEED)
    c = rng.standard_normal((8, D)) * 3.0
    X = c[rng.integers(0, 8, N)] + rng.standard_normal((N, D))
    Y0 = rng.standard_normal((N, 2)) * 1e-4
    return X, Y0


def main():
    import oracle
    oracle.build_reference()
    ref = oracle.Reference()
    X, Y0 = data()
    out = {}
    for name, kw in CASES.items():
        _, costs = ref.run(X, Y0, nthreads=os.cpu_count() or 1, **COMMON, **kw)
        out[name] = costs
        print(name, costs[49], costs[249], costs[499])
    np.savez_compressed(os.path.join(HERE, "kl_5000.npz"), **out)


if __name__ == "__main__":
    main()
