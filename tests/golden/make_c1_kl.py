"""Golden KL curves of the compiled reference (oracle/_ref, the unmodified sources) on the
10,000-point configuration: N = 10,000 x D = 50, ten equal Gaussian clusters (centres
N(0, 16 I), within-cluster N(0, I), data seed 42); perplexity 30, K = 90, the exact VP-tree
kNN, 2-D, df = 1, 1000 iterations, early exaggeration 12 until iteration 250, learning rate
N / 12, momentum 0.5 -> 0.8 at 250, nterms 3, min_num_intervals 50, intervals_per_integer 1.

Three runs that differ in the initial embedding (N(0, 1e-4^2) from default_rng(seed), seeds
1, 2, 3), each with nthreads = 1: the reference's KL sum races under threads.  The data and
the initial embeddings are regenerated by the test (numpy's default_rng is the same on every
platform; the file stores checksums to prove it), so only the costs are stored.

    python tests/golden/make_c1_kl.py   (needs the reference tree: make -C oracle ref)
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))

N, D, K_CLUSTERS, DATA_SEED = 10000, 50, 10, 42
INIT_SEEDS = (1, 2, 3)
SETTINGS = dict(no_dims=2, perplexity=30.0, max_iter=1000, stop_lying_iter=250, mom_switch_iter=250,
                momentum=0.5, final_momentum=0.8, learning_rate=N / 12.0, early_exag_coeff=12.0, nterms=3,
                ipi=1.0, min_num_intervals=50, df=1.0, knn_algo=2)


def data():
    """Ten equal clusters: centres N(0, 16 I), within-cluster N(0, I)."""
    rng = np.random.default_rng(DATA_SEED)
    centres = rng.standard_normal((K_CLUSTERS, D)) * 4.0
    labels = np.repeat(np.arange(K_CLUSTERS), N // K_CLUSTERS)
    return centres[labels] + rng.standard_normal((N, D))


def initial(seed):
    return np.random.default_rng(seed).standard_normal((N, 2)) * 1e-4


def checksum(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()


def main():
    import oracle
    oracle.build_reference()
    ref = oracle.Reference()
    X = data()
    out = {"X_sha256": np.array(checksum(X))}
    for s in INIT_SEEDS:
        Y0 = initial(s)
        _, costs = ref.run(X, Y0, nthreads=1, **SETTINGS)
        out["costs_seed%d" % s] = costs
        out["Y0_sha256_seed%d" % s] = np.array(checksum(Y0))
        print("seed", s, costs[49], costs[249], costs[999], flush=True)
    np.savez_compressed(os.path.join(HERE, "c1_kl.npz"), **out)


if __name__ == "__main__":
    main()
