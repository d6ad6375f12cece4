"""Whole pipeline (fitsne_run, the TSNE::run replacement) against the reference and the
C restatement.  Final-KL criterion: within 1% of the reference."""
import ctypes
import math
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
IDX = [49, 99, 149, 199, 249, 299]


@pytest.fixture(scope="module")
def orc():
    oracle.build_restated()
    return oracle.Restated()


@pytest.mark.parametrize("bits,early_rtol,final_rtol", [(32, 5e-3, 3e-2), (64, 1e-8, 3e-2)])
def test_run_final_kl_matches_reference(gpu_lib, golden, bits, early_rtol, final_rtol):
    """KL of a 1,000-point run against the reference.  The optimiser (sign-based gains,
    momentum) amplifies rounding differences chaotically: the FP64 form stays at rounding
    level through the first checkpoint; FP32 runs (not bitwise repeatable: float atomics)
    spread by up to 3e-3 at iteration 49 and 1.4e-2 at iteration 299 over 15 repeats on a
    GB300 (the same spread before and after the warp-aggregated spread); FP64 runs, whose
    last bits depend on the twiddle source and the attraction's launch shape, reach 1.9e-2
    at iteration 299.  The 1% criterion is tested at 5,000 points, where the final KL
    averages out the chaos."""
    gpu_lib.set_precision(bits)
    try:
        Y, costs = gpu_lib.run(golden["e2e_X"], Y0=golden["e2e_Y0"], perplexity=15.0, max_iter=300,
                               stop_lying_iter=100, mom_switch_iter=100, learning_rate=200.0, knn_algo=2)
    finally:
        gpu_lib.set_precision(32)
    ref = golden["e2e_costs"]
    assert abs(costs[49] - ref[49]) <= early_rtol * ref[49]
    assert abs(costs[299] - ref[299]) <= final_rtol * ref[299]
    assert np.isfinite(Y).all() and np.abs(Y.mean(0)).max() < 1e-6


def test_run_random_init_uses_the_reference_generator(gpu_lib):
    """With no initial Y the solution starts from srand(seed) + the polar method * 1e-4."""
    X = np.random.default_rng(0).standard_normal((300, 5))
    Y, _ = gpu_lib.run(X, perplexity=10.0, rand_seed=17, max_iter=0)
    libc = ctypes.CDLL(None)
    libc.srand(17)
    RAND_MAX = 2147483647
    out = []
    while len(out) < 600:
        while True:
            x = 2 * (libc.rand() / (RAND_MAX + 1.0)) - 1
            y = 2 * (libc.rand() / (RAND_MAX + 1.0)) - 1
            r = x * x + y * y
            if r < 1.0 and r != 0.0:
                break
        out.append(x * math.sqrt(-2 * math.log(r) / r) * 1e-4)
    assert np.allclose(Y.ravel(), out, rtol=1e-14, atol=0)


def test_run_leaves_the_data_unmodified(gpu_lib):
    """fitsne_run reads X without centring or rescaling it in place (the reference does both to
    its own copy): called through the C ABI on the caller's array, which must come back as it
    went in."""
    X = np.random.default_rng(1).standard_normal((500, 6)) * 3.0 + 1.0
    X0 = X.copy()
    Y = np.zeros((500, 2))
    c = np.zeros(5)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = gpu_lib.lib().fitsne_run(X.ctypes.data_as(dp), 500, 6, Y.ctypes.data_as(dp), 2, 10.0, 0.5, 3, 0, 5, 250,
                                  250, .5, .8, 200.0, -1, -1.0, 2, 2, 12.0, c.ctypes.data_as(dp), 0, -1, -1.0, 50,
                                  -1, 3, 1.0, 50, 0, 0, 0, None, 1.0, 5.0)
    assert rc == 0 and np.isfinite(Y).all()
    assert np.array_equal(X, X0)


@pytest.mark.parametrize("case", ["late_exag_1d_df05", "no_momentum_2d", "auto_exag", "perp_list_df3"])
def test_run_options_match_restatement(gpu_lib, orc, case):
    rng = np.random.default_rng(11)
    # 4,000 points: large enough for the final KL to average out the optimiser's chaos
    X = np.concatenate([rng.standard_normal((1000, 8)) + c for c in (0, 4, 8, 12)])
    kw = dict(perplexity=12.0, max_iter=600, stop_lying_iter=100, mom_switch_iter=100, learning_rate=4000 / 12.0)
    nd = 2
    if case == "late_exag_1d_df05":
        kw.update(start_late_exag_iter=150, late_exag_coeff=4.0, df=0.5)
        nd = 1
    elif case == "no_momentum_2d":
        kw.update(no_momentum_during_exag=1, max_step_norm=-1.0)
    elif case == "auto_exag":
        kw.update(early_exag_coeff=0.0)
    else:
        kw.update(perplexity=0.0, perplexity_list=[5.0, 20.0], df=3.0)
    Y0 = rng.standard_normal((len(X), nd)) * 1e-4
    gkw = dict(kw)
    # df = 3 with a perplexity list: a single FP32 run's final KL varies by about +-1.2 % from
    # run to run (float-atomic order; six repeats 2.623 - 2.664, FP64 form 2.640, restatement
    # 2.645), so that case holds the mean of five runs to the 1 % criterion
    reps = 5 if case == "perp_list_df3" else 1
    runs = [gpu_lib.run(X, no_dims=nd, Y0=Y0, **gkw)[1] for _ in range(reps)]
    costs = np.mean(runs, axis=0)
    okw = dict(kw)
    Yo, co = orc.run(X, Y0, no_dims=nd, nthreads=os.cpu_count() or 4, **okw)
    assert abs(costs[99] - co[99]) <= 1e-2 * co[99]
    assert abs(costs[599] - co[599]) <= 1e-2 * co[599]


def test_affinity_files_save_and_load(gpu_lib, golden, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    X, Y0 = golden["e2e_X"], golden["e2e_Y0"]
    kw = dict(Y0=Y0, perplexity=15.0, max_iter=100, stop_lying_iter=50, mom_switch_iter=50, learning_rate=200.0)
    Ya, ca = gpu_lib.run(X, load_affinities=2, **kw)
    for f in ("P_row.dat", "P_col.dat", "P_val.dat"):
        assert os.path.getsize(f) > 0
    row = np.fromfile("P_row.dat", np.uint32)
    val = np.fromfile("P_val.dat", np.float64)
    assert len(row) == len(X) + 1 and abs(val.sum() - 1.0) < 1e-12
    col = np.fromfile("P_col.dat", np.uint32)
    Yb, cb = gpu_lib.run(X, load_affinities=1, **kw)
    # the loaded P is the saved one; FP32 runs are not bitwise repeatable (float atomics)
    gpu_lib.set_precision(64)
    try:
        dC1, z1 = gpu_lib.fft_gradient(row, col, val, Y0, 3, 1.0, 50, 1.0)
    finally:
        gpu_lib.set_precision(32)
    assert np.isfinite(dC1).all() and z1 > 0
    assert abs(ca[49] - cb[49]) <= 1e-2 * ca[49]


def test_p_files_interchange_with_the_reference(gpu_lib, golden, tmp_path, monkeypatch):
    """P files of the compiled reference (load_affinities = 2, src/tsne.cpp:333-366;
    tests/golden/pfiles_e2e.npz) against fitsne_run's.  The files fitsne_run writes have the
    reference's rows and columns byte for byte, and its values within 1e-13 relative: the
    GPU's exp and the host's may differ in the last bit, and the normalisation divides by the
    sum of P, which the reference adds up sequentially and the GPU by a parallel reduction
    (measured: within 3e-14).  The reference's files load with load_affinities = 1
    (src/tsne.cpp:236-281) and the FP64 form then follows the reference's run on that P to
    rounding level at the first checkpoint."""
    pf = np.load(os.path.join(os.path.dirname(__file__), "golden", "pfiles_e2e.npz"))
    monkeypatch.chdir(tmp_path)
    X, Y0 = golden["e2e_X"], golden["e2e_Y0"]
    kw = dict(Y0=Y0, perplexity=15.0, stop_lying_iter=100, mom_switch_iter=100, learning_rate=200.0, knn_algo=2)
    gpu_lib.run(X, load_affinities=2, max_iter=1, **kw)
    row = np.fromfile("P_row.dat", np.uint32)
    col = np.fromfile("P_col.dat", np.uint32)
    val = np.fromfile("P_val.dat", np.float64)
    assert np.array_equal(row, pf["P_row"]) and np.array_equal(col, pf["P_col"])
    assert np.allclose(val, pf["P_val"], rtol=1e-13, atol=0)
    # the reference's files, loaded
    pf["P_row"].tofile("P_row.dat")
    pf["P_col"].tofile("P_col.dat")
    pf["P_val"].tofile("P_val.dat")
    gpu_lib.set_precision(64)
    try:
        Y, costs = gpu_lib.run(X, load_affinities=1, max_iter=300, **kw)
    finally:
        gpu_lib.set_precision(32)
    ref = golden["e2e_costs"]
    assert abs(costs[49] - ref[49]) <= 1e-8 * ref[49], (costs[49], ref[49])
    assert abs(costs[299] - ref[299]) <= 3e-2 * ref[299]
    assert np.isfinite(Y).all()


def _kl5000():
    import make_kl_5000 as m
    return m, np.load(os.path.join(os.path.dirname(__file__), "golden", "kl_5000.npz"))


@pytest.mark.parametrize("case", ["df1", "df05_late"])
@pytest.mark.parametrize("bits,graphs", [(32, "1"), (32, "0"), (64, "1")])
def test_final_kl_within_one_percent_of_reference_5000(gpu_lib, monkeypatch, case, bits, graphs):
    """Final KL of a 5,000-point, 500-iteration run within 1% of the compiled reference's
    (golden curve), in both forms, with and without the graph-captured iteration."""
    m, g = _kl5000()
    X, Y0 = m.data()
    monkeypatch.setenv("FITSNE_GRAPH", graphs)
    gpu_lib.set_precision(bits)
    try:
        _, costs = gpu_lib.run(X, Y0=Y0, knn_algo=2, **m.COMMON, **m.CASES[case])
    finally:
        gpu_lib.set_precision(32)
    ref = g[case]
    assert abs(costs[499] - ref[499]) <= 1e-2 * ref[499]
    assert abs(costs[49] - ref[49]) <= 1e-2 * ref[49]


def test_graph_iteration_matches_host_iteration_fp64(gpu_lib, monkeypatch, golden):
    """The graph path (grid sized on the device, chunks of iterations replayed) computes the
    same iterations as the host path: FP64 runs agree to rounding through iteration 49."""
    kw = dict(Y0=golden["e2e_Y0"], perplexity=15.0, max_iter=100, stop_lying_iter=50, mom_switch_iter=50,
              learning_rate=200.0, knn_algo=2)
    gpu_lib.set_precision(64)
    try:
        monkeypatch.setenv("FITSNE_GRAPH", "0")
        Ya, ca = gpu_lib.run(golden["e2e_X"], **kw)
        monkeypatch.setenv("FITSNE_GRAPH", "1")
        Yb, cb = gpu_lib.run(golden["e2e_X"], **kw)
    finally:
        gpu_lib.set_precision(32)
    assert abs(ca[49] - cb[49]) <= 1e-9 * ca[49]
    assert np.abs(Ya - Yb).max() <= 1e-6 * np.abs(Ya).max()


@pytest.mark.parametrize("mode", ["pipeline", "streams"])
def test_batched_jobs_match_single_runs(gpu_lib, monkeypatch, mode):
    """fitsne_batch_run advances several embeddings together; each job ends where its own
    fitsne_run ends (final KL within 1% of the mean of 3 single runs), the 5,000-point job
    within 1% of the reference.
    "pipeline": all jobs in the same launches (the default for 2-D, nterms 3, df 1);
    "streams": one graph per job on its own stream (FITSNE_BATCH=streams).
    (FP32 runs differ by the optimiser's chaos alone, seeded by the order of the spread's atomic
    additions.  Measured on the 2,500-point job: 6 single runs 1.525 - 1.535, 3 batched runs
    1.524 - 1.537, so two single runs can be 1.2% apart; on structureless data, 1.2% on 1,200
    isotropic Gaussian points.)"""
    if mode == "streams":
        monkeypatch.setenv("FITSNE_BATCH", "streams")
    m, g = _kl5000()
    X5, Y5 = m.data()
    rng = np.random.default_rng(3)
    c3 = rng.standard_normal((6, 30)) * 4.0
    Xs = [X5, rng.standard_normal((2500, 10)) + np.repeat(np.eye(10) * 6, 250, axis=0),
          c3[rng.integers(0, 6, 1200)] + rng.standard_normal((1200, 30))]
    perps = [30.0, 20.0, 10.0]
    Y0s = [Y5] + [rng.standard_normal((len(X), 2)) * 1e-4 for X in Xs[1:]]
    lrs = [len(X) / 12.0 for X in Xs]
    Ys, costs, st = gpu_lib.batch_run(Xs, perps, learning_rates=lrs, Y0s=Y0s, max_iter=500)
    assert st["graph_launches"] >= 9 and st["graph_instantiations"] >= 1
    for j, X in enumerate(Xs):
        ref = np.mean([gpu_lib.run(X, Y0=Y0s[j], perplexity=perps[j], learning_rate=lrs[j], max_iter=500,
                                   knn_algo=2)[1][499] for _ in range(3)])
        assert abs(costs[j][499] - ref) <= 1e-2 * ref, j
        assert np.isfinite(Ys[j]).all()
    assert abs(costs[0][499] - g["df1"][499]) <= 1e-2 * g["df1"][499]


def test_sixteen_batched_jobs_of_uneven_size(gpu_lib, orc):
    """16 jobs, N log-uniform in [1,500, 12,000], 5 - 15 clusters each, perplexity 10 / 30 / 50
    cycled (K = 3 perplexity), advanced together by the all-jobs pipeline: each job's final KL
    within 1.5 % of the mean of two single runs of the same job, and the smallest job's within
    1 % of the restated reference loop run on the reference's P from the same start."""
    rng = np.random.default_rng(16)
    Xs, perps = [], []
    for j in range(16):
        N = int(round(np.exp(rng.uniform(np.log(1500), np.log(12000)))))
        k = int(rng.integers(5, 16))
        c = rng.standard_normal((k, 20)) * 5.0
        Xs.append(c[rng.integers(0, k, N)] + rng.standard_normal((N, 20)))
        perps.append((10.0, 30.0, 50.0)[j % 3])
    Y0s = [rng.standard_normal((len(X), 2)) * 1e-4 for X in Xs]
    lrs = [max(200.0, len(X) / 12.0) for X in Xs]
    Ys, costs, st = gpu_lib.batch_run(Xs, perps, learning_rates=lrs, Y0s=Y0s, max_iter=500)
    assert st["graph_launches"] >= 9
    for j, X in enumerate(Xs):
        ref = np.mean([gpu_lib.run(X, Y0=Y0s[j], perplexity=perps[j], learning_rate=lrs[j], max_iter=500,
                                   knn_algo=2)[1][499] for _ in range(2)])
        assert np.isfinite(Ys[j]).all()
        assert abs(costs[j][499] - ref) <= 1.5e-2 * ref, (j, len(X), costs[j][499], ref)
    j = int(np.argmin([len(X) for X in Xs]))
    X = Xs[j] - np.cumsum(Xs[j], axis=0)[-1] / len(Xs[j])
    X /= np.abs(X).max()
    r, c, v = gpu_lib.gaussian_perplexity(X, perps[j], int(3 * perps[j]))
    r, c, v = gpu_lib.symmetrize(r, c, v, len(X))
    _, cref = orc.run_from_P(r, c, v / np.cumsum(v)[-1], Y0s[j], max_iter=500, learning_rate=lrs[j], nthreads=4)
    assert abs(costs[j][499] - cref[499]) <= 1e-2 * cref[499], (costs[j][499], cref[499])


def test_batched_one_dimensional_jobs(gpu_lib):
    """1-D batches (outside the all-jobs pipeline: one graph per job) end where the jobs' own
    runs end (final KL within 2 %: 800-point FP32 runs)."""
    rng = np.random.default_rng(8)
    Xs = [rng.standard_normal((800, 6)) + np.repeat(np.eye(6)[:4] * 5, 200, axis=0),
          rng.standard_normal((600, 6)) + np.repeat(np.eye(6)[:3] * 5, 200, axis=0)]
    Y0s = [rng.standard_normal((len(X), 1)) * 1e-4 for X in Xs]
    lrs = [200.0, 200.0]
    Ys, costs, st = gpu_lib.batch_run(Xs, [20.0, 20.0], learning_rates=lrs, Y0s=Y0s, no_dims=1, max_iter=300)
    for j, X in enumerate(Xs):
        _, c = gpu_lib.run(X, no_dims=1, Y0=Y0s[j], perplexity=20.0, learning_rate=lrs[j], max_iter=300)
        assert Ys[j].shape == (len(X), 1) and np.isfinite(Ys[j]).all()
        assert abs(costs[j][299] - c[299]) <= 2e-2 * c[299], j
