"""GPU input-similarity stage vs the reference (fixtures) and the C restatement."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc():
    oracle.build_restated()
    return oracle.Restated()


def test_knn_matches_reference_neighbour_lists(gpu_lib, golden):
    X = golden["sim_X"]
    K = int(golden["sim_K"])
    idx, dist = gpu_lib.knn(X, K + 1)
    assert np.array_equal(idx[:, 0], np.arange(len(X)))
    # the reference's VP-tree lists, nearest first (this data has no distance ties)
    assert np.array_equal(idx[:, 1:], golden["knn_col"].reshape(-1, K))
    assert np.all(np.diff(dist, axis=1) >= 0)


@pytest.mark.parametrize("N,D,K", [(3000, 100, 31), (2500, 7, 15), (700, 50, 200)])
def test_knn_is_exact_against_bruteforce(gpu_lib, orc, N, D, K):
    rng = np.random.default_rng(N + D)
    X = rng.standard_normal((N, D)) * rng.uniform(0.1, 2.0, D)
    X[5] = X[7]  # a duplicate pair: a distance tie at zero
    idx, dist = gpu_lib.knn(X, K)
    oidx, odist = orc.knn(X, K, 4)
    assert np.allclose(dist, odist, rtol=1e-13, atol=1e-15)
    # index lists agree except within groups of equal distances
    diff = np.nonzero((idx != oidx).any(axis=1))[0]
    for r in diff:
        assert np.allclose(np.sort(dist[r]), np.sort(odist[r]), rtol=1e-13)
        assert set(idx[r][dist[r] < odist[r][-1]]) == set(oidx[r][odist[r] < odist[r][-1]])


@pytest.mark.parametrize("N,D,K,spread,path,order", [(3001, 50, 91, 4.0, "tcgen05", "random"),
                                                      (4096, 62, 31, 0.3, "tcgen05", "random"),
                                                      (1500, 20, 100, 2.0, "FP32", "random"),
                                                      (2000, 63, 20, 1.0, "FP32", "random"),
                                                      (70001, 50, 91, 3.0, "tcgen05", "random"),
                                                      (70001, 50, 91, 3.0, "tcgen05", "input"),
                                                      (50001, 40, 91, 3.0, "tcgen05", "clusters"),
                                                      (30000, 50, 31, 0.6, "tcgen05", "clusters")])
def test_tensor_core_candidates_give_the_exact_lists(gpu_lib, monkeypatch, capfd, N, D, K, spread, path, order):
    """The tcgen05 candidate search (BF16 hi/lo split, folded norms, tile skipping, locality
    order) and the FP32 scan must end in the same exact neighbour lists after the FP64
    re-rank; tight clusters exercise the rescans, N = 70001 a ragged last tile of a multi-tile
    grid, well separated clusters the skipping of reference tiles, whether the rows come in
    random order (put in locality order first) or grouped by cluster; "input" keeps the
    caller's random order (FITSNE_KNN_ORDER=input).  K + 29 > 120 candidates or D > 62 take
    the FP32 scan."""
    rng = np.random.default_rng(N + D)
    centres = rng.standard_normal((8, D)) * spread
    lab = rng.integers(0, 8, N)
    if order == "clusters":
        lab = np.sort(lab)
    if order == "input":
        monkeypatch.setenv("FITSNE_KNN_ORDER", "input")
    X = centres[lab] + rng.standard_normal((N, D)) * 0.05
    X = (X - X.mean(0)) / np.abs(X - X.mean(0)).max()
    monkeypatch.setenv("FITSNE_TIMING", "1")
    capfd.readouterr()
    idx_tc, d_tc = gpu_lib.knn(X, K)
    log = capfd.readouterr().err
    assert path + " candidates" in log
    if N >= 16384 and path == "tcgen05":  # 8 separated clusters: most reference tiles skipped
        computed = float(log.split("tile pairs computed ")[1].split("%")[0])
        assert (computed > 90.0) if order == "input" else (computed < 50.0), log
    monkeypatch.setenv("FITSNE_KNN", "simt")
    idx_s, d_s = gpu_lib.knn(X, K)
    assert np.allclose(d_tc, d_s, rtol=0, atol=0)
    diff = np.nonzero((idx_tc != idx_s).any(axis=1))[0]
    for r in diff:  # only permutations within equal distances
        for a in np.unique(d_tc[r]):
            assert set(idx_tc[r][d_tc[r] == a]) == set(idx_s[r][d_s[r] == a])


def test_calibration_matches_reference(gpu_lib, golden):
    X = golden["sim_X"]
    K = int(golden["sim_K"])
    _, dist = gpu_lib.knn(X, K + 1)
    P, betas = gpu_lib.distances2similarities(dist[:, 1:], float(golden["sim_perp"]))
    assert np.allclose(P.ravel(), golden["knn_val"], rtol=1e-12, atol=1e-300)
    H = -(P * np.log(P)).sum(1)
    assert np.abs(H - np.log(float(golden["sim_perp"]))).max() < 1e-5 + 1e-12


def test_gaussian_perplexity_matches_reference(gpu_lib, golden):
    X = golden["sim_X"]
    row, col, val = gpu_lib.gaussian_perplexity(X, float(golden["sim_perp"]), int(golden["sim_K"]))
    assert np.array_equal(row, golden["knn_row"]) and np.array_equal(col, golden["knn_col"])
    assert np.allclose(val, golden["knn_val"], rtol=1e-12)
    _, lcol, lval = gpu_lib.gaussian_perplexity(X, 0.0, 45, perplexity_list=list(golden["list_perps"]))
    assert np.array_equal(lcol, golden["list_col"]) and np.allclose(lval, golden["list_val"], rtol=1e-12)
    _, fcol, fval = gpu_lib.gaussian_perplexity(X, -1.0, int(golden["sigma_K"]), sigma=float(golden["sigma"]))
    assert np.array_equal(fcol, golden["sigma_col"]) and np.allclose(fval, golden["sigma_val"], rtol=1e-12)


def test_symmetrize_matches_reference_exactly(gpu_lib, golden):
    r, c, v = gpu_lib.symmetrize(golden["knn_row"], golden["knn_col"], golden["knn_val"], 2000)
    assert np.array_equal(r, golden["sym_row"]) and np.array_equal(c, golden["sym_col"])
    assert np.array_equal(v, golden["sym_val"])


@pytest.mark.parametrize("N,kmax,seed,hub", [(500, 9, 0, False), (20000, 30, 1, False), (3000, 20, 2, True)])
def test_symmetrize_general_csr_matches_oracle(gpu_lib, orc, N, kmax, seed, hub):
    """Entry-for-entry equality with the restated symmetrizeMatrix on random CSR patterns
    (empty rows, self loops); "hub": one row lists 400 points and 300 rows list point 7, so that
    rows longer than a warp's 256 entries take the thread-per-row kernels."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, kmax + 1, N)
    if hub:
        lens[3] = 400
    row = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint32)
    cols = []
    for i in range(N):
        c = rng.choice(N, lens[i], replace=False)
        if i % 97 == 0 and lens[i] > 0 and i not in c:
            c[0] = i  # self loops appear with duplicate points
        if hub and 100 <= i < 400 and lens[i] > 0 and 7 not in c:
            c[0] = 7  # many incoming edges of point 7
        cols.append(c)
    col = np.concatenate(cols).astype(np.uint32)
    val = rng.random(len(col))
    a = gpu_lib.symmetrize(row, col, val, N)
    b = orc.symmetrize(row, col, val, N)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
