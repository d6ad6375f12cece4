"""Generates tests/golden/*.npz from the reference itself.

Runs the UNMODIFIED FIt-SNE reference sources compiled by ``make -C oracle ref`` (against
the project FFT shim; the reference has no tests or fixtures of its own) on small seeded
inputs and stores inputs and outputs.  The GPU machine has no copy of the reference, so the
GPU parity tests read these files.  Re-run with ``python tests/golden/make_golden.py``.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402


def mixture(rng, N, D, C, spread, within=1.0):
    centres = rng.standard_normal((C, D)) * spread
    lab = rng.integers(0, C, N)
    return centres[lab] + rng.standard_normal((N, D)) * within, lab


def normalise(X):
    """zeroMean + division by max|X| as TSNE::run does before the kNN (tsne.cpp:153-164)."""
    X = X - X.mean(0)
    return X / np.abs(X).max()


def main():
    path = oracle.build_reference()
    if path is None:
        raise SystemExit("the reference tree is needed to generate fixtures")
    ref = oracle.Reference(path)
    rng = np.random.default_rng(20261203)
    out = {}

    # --- similarities: kNN + calibration + symmetrisation --------------------------
    N, D, perp = 2000, 10, 10.0
    K = int(3 * perp)
    X, _ = mixture(rng, N, D, 6, 4.0)
    Xn = normalise(X)
    row, col, val = ref.gaussian_perplexity(Xn, perp, K, -1.0, 1)
    out.update(sim_X=Xn, sim_perp=perp, sim_K=K, knn_row=row, knn_col=col, knn_val=val)
    srow, scol, sval = ref.symmetrize(row, col, val, N)
    out.update(sym_row=srow, sym_col=scol, sym_val=sval)
    Pn = sval / sval.sum()
    # perplexity list and fixed sigma on the same data
    lrow, lcol, lval = ref.gaussian_perplexity(Xn, 0.0, int(3 * 15), -1.0, 1, perplexity_list=[5.0, 15.0])
    out.update(list_perps=np.array([5.0, 15.0]), list_col=lcol, list_val=lval)
    frow, fcol, fval = ref.gaussian_perplexity(Xn, -1.0, 20, 0.1, 1)
    out.update(sigma_K=20, sigma=0.1, sigma_col=fcol, sigma_val=fval)

    # --- gradients on a spread-out embedding and on the initial one -----------------
    Y2, lab = mixture(rng, N, 2, 8, 12.0, 1.5)
    Y2 -= Y2.mean(0)
    Y1 = Y2[:, :1] * 2.0
    Y0 = rng.standard_normal((N, 2)) * 1e-4
    out.update(Y2=Y2, Y1=Y1, Y0=Y0)
    cases = {"g2_df1": (Y2, 1.0), "g2_df05": (Y2, 0.5), "g1_df1": (Y1, 1.0), "g1_df05": (Y1, 0.5),
             "g0_df1": (Y0, 1.0), "g2_df3": (Y2, 3.0)}
    for name, (Y, df) in cases.items():
        dC, z = ref.fft_gradient(srow, scol, Pn, Y, 3, 1.0, 50, 1, df)
        kl = ref.evaluate_error_fft(srow, scol, Pn, Y, df, z)
        out[name + "_dC"] = dC
        out[name + "_Z"] = z
        out[name + "_KL"] = kl
    # nterms = 5 and a finer grid
    dC, z = ref.fft_gradient(srow, scol, Pn, Y2, 5, 2.0, 30, 1, 1.0)
    out.update(g2_nt5_dC=dC, g2_nt5_Z=z)

    # --- a short end-to-end run with a given initialisation -------------------------
    Ne = 1000
    Xe, _ = mixture(rng, Ne, 10, 5, 5.0)
    Ye0 = rng.standard_normal((Ne, 2)) * 1e-4
    kw = dict(no_dims=2, perplexity=15.0, max_iter=300, stop_lying_iter=100, mom_switch_iter=100,
              learning_rate=200.0, early_exag_coeff=12.0, nthreads=1)
    Ye, costs = ref.run(Xe, Ye0, **kw)
    out.update(e2e_X=Xe, e2e_Y0=Ye0, e2e_Y=Ye, e2e_costs=costs)

    dst = os.path.join(HERE, "fitsne_golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
