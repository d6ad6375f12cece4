"""The parity configurations at their full sizes, against the reference's own path on the
same inputs (the compiled reference's golden KL curves, and the C restatement in oracle/,
which reproduces the compiled reference bit for bit on every golden fixture).

* 10,000 x 50, ten equal clusters, VP-tree kNN, 1000 iterations: the final KL of both GPU
  forms within 1 % of the compiled reference's, for three initial embeddings
  (tests/golden/c1_kl.npz, made by tests/golden/make_c1_kl.py with nthreads = 1).
* 70,000-point precision form (Dirichlet(2) weights, std U(0.5, 2), centres N(0, 25 I)):
  every 50 iterations of a 750-iteration run, the FP32 gradient against the restated
  computeFftGradient (FP64) on the identical Y and P, relative L2 <= 1e-4 and Z within
  1e-5; the FP64 form on the same states within 1e-9.  The exact kNN lists against the
  restated VP-tree's (src/tsne.cpp:1643-1726), ties excepted, and P within 1e-12.
* 250,000-point 1-D heavy-tail path (df = 0.5, perplexity 50, K = 150, late exaggeration 4
  from iteration 250): the FP32 gradient against the restated
  computeFftGradientOneDVariableDf at iterations 250, 500 and 1000 (relative L2 <= 1e-4),
  and the final KL within 1 % of the restated loop's on the same P from the same start.
* 2,000,000-point run with the learned calibration (100 Zipf-sized clusters, late
  exaggeration 2): every row's entropy within 1e-5 of log(perplexity), the network trained
  on the first 200,000 rows; the final KL within 1 % of the FP64 form with the reference's
  bisection; the FP32 gradient at the final embedding against the restated one on the
  reference's P.

The data are seeded synthetic stand-ins with the configurations' shapes and distributions
(no public dataset is named)."""
import hashlib
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def orc():
    oracle.build_restated()
    return oracle.Restated()


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


def prepared(X):
    """X as TSNE::run prepares it (src/tsne.cpp:153-164): centred by zeroMean's sequential
    column sums, then divided by its largest magnitude."""
    X = X - np.cumsum(X, axis=0)[-1] / len(X)
    return X / np.abs(X).max()


def reference_P(gpu_lib, X, perplexity, K):
    """P as TSNE::run builds it (src/tsne.cpp:153-330) from the prepared X: exact kNN and
    calibration (the GPU's; identical to the reference's, tested elsewhere), symmetrisation,
    normalisation by the sequential sum."""
    row, col, val = gpu_lib.gaussian_perplexity(prepared(X), perplexity, K)
    row, col, val = gpu_lib.symmetrize(row, col, val, len(X))
    return row, col, val / np.cumsum(val)[-1]


def _fp64_gradient(gpu_lib, row, col, val, Y, **kw):
    gpu_lib.set_precision(64)
    try:
        return gpu_lib.fft_gradient(row, col, val, Y, **kw)
    finally:
        gpu_lib.set_precision(32)


# ---------------------------------------------------------------------------------------
# 10,000 x 50: final KL against the compiled reference, three initial embeddings

def c1_data():
    import make_c1_kl
    return make_c1_kl


@pytest.mark.parametrize("bits", [32, 64])
def test_c1_final_kl_within_one_percent_of_the_reference_for_three_seeds(gpu_lib, bits):
    g = np.load(os.path.join(GOLDEN, "c1_kl.npz"))
    c1 = c1_data()
    X = c1.data()
    assert c1.checksum(X) == str(g["X_sha256"]), "numpy's generator stream differs from the fixture's"
    s = c1.SETTINGS
    gpu_lib.set_precision(bits)
    try:
        for seed in c1.INIT_SEEDS:
            Y0 = c1.initial(seed)
            assert c1.checksum(Y0) == str(g["Y0_sha256_seed%d" % seed])
            Y, costs = gpu_lib.run(X, Y0=Y0, no_dims=2, perplexity=s["perplexity"], max_iter=s["max_iter"],
                                   stop_lying_iter=s["stop_lying_iter"], mom_switch_iter=s["mom_switch_iter"],
                                   momentum=s["momentum"], final_momentum=s["final_momentum"],
                                   learning_rate=s["learning_rate"], early_exag_coeff=s["early_exag_coeff"],
                                   nterms=s["nterms"], intervals_per_integer=s["ipi"],
                                   min_num_intervals=s["min_num_intervals"], df=s["df"], knn_algo=s["knn_algo"])
            ref = g["costs_seed%d" % seed]
            assert np.isfinite(Y).all()
            # the first checkpoint is still close to rounding level; the last one is held
            # to the 1 % criterion (the optimiser amplifies rounding differences)
            assert abs(costs[49] - ref[49]) <= 5e-3 * ref[49], (seed, costs[49], ref[49])
            assert abs(costs[999] - ref[999]) <= 0.01 * ref[999], (seed, costs[999], ref[999])
    finally:
        gpu_lib.set_precision(32)


# ---------------------------------------------------------------------------------------
# 70,000-point precision form

@pytest.fixture(scope="module")
def c2(gpu_lib):
    X = mixture_unequal(70000)
    return X, reference_P(gpu_lib, X, 30.0, 90)


def test_c2_gradient_every_50_iterations_against_the_oracle(gpu_lib, orc, c2):
    X, (row, col, val) = c2
    N = len(X)
    Y0 = np.random.default_rng(1).standard_normal((N, 2)) * 1e-4
    s = gpu_lib.Session(row, col, val, Y0, precision=32)
    worst = 0.0
    try:
        for it in range(0, 750, 50):
            s.run(it, it + 50, max_iter=750, learning_rate=N / 12.0)
            Y = s.get_y()
            d32, z32 = s.gradient()
            dref, zref = orc.fft_gradient(row, col, val, Y, 3, 1.0, 50, NT, 1.0)
            err = rel_l2(d32, dref)
            worst = max(worst, err)
            assert err <= 1e-4, (it + 50, err)
            assert abs(z32 - zref) <= 1e-5 * zref, (it + 50, z32, zref)
            if it + 50 in (50, 300, 750):  # the plain FP64 form on the same state
                d64, z64 = _fp64_gradient(gpu_lib, row, col, val, Y)
                assert rel_l2(d64, dref) <= 1e-9, (it + 50, rel_l2(d64, dref))
                assert abs(z64 - zref) <= 1e-11 * zref
    finally:
        s.close()
    assert worst > 0.0


def test_c2_session_from_data_in_the_data_order_against_the_oracle(gpu_lib, orc, c2):
    """The same configuration through Session.from_data: the library builds P itself and, the
    data being 50-D and the embedding large enough to be renumbered, numbers the points in the
    data's locality order from the start.  Every 150 iterations its gradient, returned in the
    caller's order, matches the restated reference gradient on the same Y and on P built in the
    caller's order."""
    X, (row, col, val) = c2
    N = len(X)
    Y0 = np.random.default_rng(1).standard_normal((N, 2)) * 1e-4
    s = gpu_lib.Session.from_data(X, Y0, perplexity=30.0, precision=32)
    try:
        assert s.nnz == len(col)
        for it in range(0, 750, 150):
            s.run(it, it + 150, max_iter=750, learning_rate=N / 12.0)
            Y = s.get_y()
            d32, z32 = s.gradient()
            dref, zref = orc.fft_gradient(row, col, val, Y, 3, 1.0, 50, NT, 1.0)
            assert rel_l2(d32, dref) <= 1e-4, (it + 150, rel_l2(d32, dref))
            assert abs(z32 - zref) <= 1e-5 * zref, (it + 150, z32, zref)
    finally:
        s.close()


def test_c2_knn_lists_match_the_restated_vptree(gpu_lib, orc, c2):
    """Neighbour lists of the 70,000-point data (K = 90) against the restated VP-tree search
    (src/tsne.cpp:1643-1726, vptree.h): the same index sets except within groups of equal
    distances, and P within 1e-12 where the lists agree."""
    X, _ = c2
    Xp = prepared(X)
    row, col, val = gpu_lib.gaussian_perplexity(Xp, 30.0, 90)
    orow, ocol, oval = orc.gaussian_perplexity(Xp, 30.0, 90, nthreads=NT)
    assert np.array_equal(row, orow)
    K = 90
    col, ocol = col.reshape(-1, K), ocol.reshape(-1, K)
    val, oval = val.reshape(-1, K), oval.reshape(-1, K)
    same = (col == ocol).all(axis=1)
    for r in np.nonzero(~same)[0]:
        # a different set is allowed only through a tie at the K-th distance: compare the
        # FP64 distances of both lists
        d = np.sqrt(((Xp[col[r]] - Xp[r]) ** 2).sum(1))
        od = np.sqrt(((Xp[ocol[r]] - Xp[r]) ** 2).sum(1))
        assert np.allclose(np.sort(d), np.sort(od), rtol=1e-12, atol=0), r
    assert same.mean() > 0.999
    assert np.allclose(val[same], oval[same], rtol=1e-12, atol=1e-300)


# ---------------------------------------------------------------------------------------
# 250,000-point 1-D heavy-tail path

def test_c3_one_dimensional_heavy_tail_against_the_oracle(gpu_lib, orc):
    N = 250000
    X = subspace_mixture(N)
    row, col, val = reference_P(gpu_lib, X, 50.0, 150)
    Y0 = np.random.default_rng(2).standard_normal((N, 1)) * 1e-4
    sched = dict(max_iter=1000, learning_rate=N / 12.0, start_late_exag_iter=250, late_exag_coeff=4.0)
    costs = np.zeros(1000)
    s = gpu_lib.Session(row, col, val, Y0, df=0.5, precision=32)
    try:
        for it0, it1 in ((0, 250), (250, 500), (500, 1000)):
            s.run(it0, it1, costs=costs, **sched)
            Y = s.get_y()
            d32, z32 = s.gradient()
            dref, zref = orc.fft_gradient(row, col, val, Y, 3, 1.0, 50, NT, 0.5)
            assert rel_l2(d32, dref) <= 1e-4, (it1, rel_l2(d32, dref))
            assert abs(z32 - zref) <= 1e-5 * zref, (it1, z32, zref)
    finally:
        s.close()
    Yref, cref = orc.run_from_P(row, col, val, Y0, nthreads=NT, df=0.5, **sched)
    assert np.isfinite(Y).all() and np.isfinite(Yref).all()
    assert abs(costs[999] - cref[999]) <= 0.01 * cref[999], (costs[999], cref[999])


# ---------------------------------------------------------------------------------------
# 2,000,000 points with the learned calibration

def test_c5_learned_calibration_two_million_points(gpu_lib, orc):
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
        Y32, c32 = gpu_lib.run(X, **kw)
    finally:
        gpu_lib.set_calibration("bisection")
    gpu_lib.set_precision(64)
    try:
        _, c64 = gpu_lib.run(X, **kw)
    finally:
        gpu_lib.set_precision(32)
    assert abs(c32[-1] - c64[-1]) / c64[-1] < 0.01, (c32[-1], c64[-1])
    # the gradient at the final embedding, FP32 form against the restated reference, on the
    # reference's P (bisection calibration)
    row, col, val = reference_P(gpu_lib, X, perp, 90)
    d32, z32 = gpu_lib.fft_gradient(row, col, val, Y32)
    dref, zref = orc.fft_gradient(row, col, val, Y32, 3, 1.0, 50, NT, 1.0)
    assert rel_l2(d32, dref) <= 1e-4, rel_l2(d32, dref)
    assert abs(z32 - zref) <= 1e-5 * zref
