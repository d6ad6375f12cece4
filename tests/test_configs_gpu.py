"""The parity configurations at their full sizes, through size-independent properties.

* 70,000-point precision form: the FP32 gradient against the FP64 gradient on the identical
  state every 50 iterations of a 750-iteration run, relative L2 <= 1e-4.
* 250,000-point 1-D heavy-tail path (df = 0.5, perplexity 50, K = 150, late exaggeration 4
  from iteration 250): the FP32 form's final KL within 1 % of the FP64 form's.
* 2,000,000-point run with the learned calibration (100 Zipf-sized clusters, late
  exaggeration 2): every row's entropy within 1e-5 of log(perplexity), the network trained on
  the first 200,000 rows, and the final KL within 1 % of the FP64 form with the reference's
  bisection.

The data are seeded synthetic stand-ins with the configurations' shapes and distributions
(no public dataset is named)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def mixture_unequal(N, D=50, k=10, seed=42):
    """k clusters, Dirichlet(2) weights, isotropic std U(0.5, 2), centres N(0, 25 I)."""
    rng = np.random.default_rng(seed)
    sizes = rng.multinomial(N, rng.dirichlet(np.full(k, 2.0)))
    lab = np.repeat(np.arange(k), sizes)
    centres = rng.standard_normal((k, D)) * 5.0
    std = rng.uniform(0.5, 2.0, k)
    return centres[lab] + rng.standard_normal((N, D)) * std[lab, None]


def subspace_mixture(N, D=50, k=20, dim=5, seed=7):
    """k equal clusters in a random dim-dimensional subspace (centres N(0, 16 I), unit
    within-cluster spread there) plus N(0, 0.1^2) isotropic noise in all D dimensions."""
    rng = np.random.default_rng(seed)
    basis = np.linalg.qr(rng.standard_normal((D, dim)))[0].T  # dim x D, orthonormal rows
    lab = rng.integers(0, k, N)
    z = rng.standard_normal((k, dim))[lab] * 4.0 + rng.standard_normal((N, dim))
    return z @ basis + rng.standard_normal((N, D)) * 0.1


def zipf_mixture(N, D=50, k=100, s=1.1, seed=11):
    """k clusters with Zipf(s) sizes, centres N(0, 9 I), unit within-cluster spread."""
    rng = np.random.default_rng(seed)
    w = 1.0 / np.arange(1, k + 1) ** s
    sizes = np.floor(N * w / w.sum()).astype(int)
    sizes[0] += N - sizes.sum()
    lab = np.repeat(np.arange(k), sizes)
    rng.shuffle(lab)
    centres = rng.standard_normal((k, D)) * 3.0
    return centres[lab] + rng.standard_normal((N, D))


def test_precision_form_gradient_every_50_iterations(gpu_lib):
    N = 70000
    X = mixture_unequal(N)
    Y0 = np.random.default_rng(1).standard_normal((N, 2)) * 1e-4
    # P as TSNE::run builds it (X centred and scaled by its largest magnitude), shared by the
    # FP32 session and the FP64 reference gradients
    Xn = X - X.mean(0)
    Xn /= np.abs(Xn).max()
    row, col, val = gpu_lib.gaussian_perplexity(Xn, 30.0, 90)
    row, col, val = gpu_lib.symmetrize(row, col, val, N)
    val = np.asarray(val) / np.sum(val)
    s = gpu_lib.Session(row, col, val, Y0, precision=32)
    worst = 0.0
    try:
        for it in range(0, 750, 50):
            s.run(it, it + 50, max_iter=750, learning_rate=N / 12.0)
            Y = s.get_y()
            d32, _ = s.gradient()
            gpu_lib.set_precision(64)
            try:
                d64, _ = gpu_lib.fft_gradient(row, col, val, Y)
            finally:
                gpu_lib.set_precision(32)
            err = rel_l2(d32, d64)
            worst = max(worst, err)
            assert err <= 1e-4, (it + 50, err)
    finally:
        s.close()
    assert worst > 0.0


def test_one_dimensional_heavy_tail_kl_matches_fp64(gpu_lib):
    N = 250000
    X = subspace_mixture(N)
    Y0 = np.random.default_rng(2).standard_normal((N, 1)) * 1e-4
    kw = dict(no_dims=1, perplexity=50.0, K=150, df=0.5, max_iter=1000, learning_rate=N / 12.0, Y0=Y0,
              start_late_exag_iter=250, late_exag_coeff=4.0)
    Y32, c32 = gpu_lib.run(X, **kw)
    gpu_lib.set_precision(64)
    try:
        Y64, c64 = gpu_lib.run(X, **kw)
    finally:
        gpu_lib.set_precision(32)
    assert Y32.shape == (N, 1) and np.isfinite(Y32).all()
    assert abs(c32[-1] - c64[-1]) / c64[-1] < 0.01, (c32[-1], c64[-1])


def test_learned_calibration_two_million_points(gpu_lib):
    N = 2000000
    X = zipf_mixture(N)
    perp = 30.0
    gpu_lib.set_calibration("learned")
    try:
        row, col, val = gpu_lib.gaussian_perplexity(X, perp, 90)
        st = gpu_lib.calibration_stats()
        P = np.asarray(val).reshape(N, 90)
        H = -(P * np.log(np.maximum(P, 1e-300))).sum(1)
        assert np.abs(H - np.log(perp)).max() < 1e-5
        assert st["rows"] == N and st["rows_harvest"] == 200000
        assert st["evals_warm"] < st["evals_plain"] / 3
        del P, H, row, col, val
        Y0 = np.random.default_rng(3).standard_normal((N, 2)) * 1e-4
        kw = dict(perplexity=perp, K=90, max_iter=1000, learning_rate=N / 12.0, Y0=Y0, start_late_exag_iter=250,
                  late_exag_coeff=2.0)
        _, c32 = gpu_lib.run(X, **kw)
    finally:
        gpu_lib.set_calibration("bisection")
    gpu_lib.set_precision(64)
    try:
        _, c64 = gpu_lib.run(X, **kw)
    finally:
        gpu_lib.set_precision(32)
    assert abs(c32[-1] - c64[-1]) / c64[-1] < 0.01, (c32[-1], c64[-1])
