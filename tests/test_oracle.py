"""The CPU oracle itself: project FFT vs numpy, the C restatement vs the golden fixtures
made by the reference, and (where the reference tree is present) vs the compiled
reference on fresh inputs.  These tests pin the checker before it judges the GPU."""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import rel_l2

GRAD_CASES = [("g2_df1", "Y2", 1.0), ("g2_df05", "Y2", 0.5), ("g2_df3", "Y2", 3.0), ("g1_df1", "Y1", 1.0),
              ("g1_df05", "Y1", 0.5), ("g0_df1", "Y0", 1.0)]


@pytest.fixture(scope="module")
def orc():
    oracle.build_restated()
    return oracle.Restated()


def _fft(lib):
    dp = ctypes.POINTER(ctypes.c_double)
    lib.fft64_plan_c2c.restype = ctypes.c_void_p
    lib.fft64_plan_c2c.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.fft64_exec_c2c.argtypes = [ctypes.c_void_p, dp, dp]
    lib.fft64_destroy.argtypes = [ctypes.c_void_p]
    lib.fft64_r2c_2d.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
    lib.fft64_c2r_2d.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
    return dp


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 12, 30, 150, 330, 1050, 1278, 97, 1999])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft64_c2c_matches_numpy(orc, n, sign):
    dp = _fft(orc.lib)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = np.zeros(n, complex)
    p = orc.lib.fft64_plan_c2c(n, sign)
    orc.lib.fft64_exec_c2c(p, x.ctypes.data_as(dp), y.ctypes.data_as(dp))
    orc.lib.fft64_destroy(p)
    ref = np.fft.fft(x) if sign == -1 else np.fft.ifft(x) * n
    assert np.abs(y - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("shape", [(6, 6), (7, 9), (300, 300), (330, 330)])
def test_fft64_r2c_c2r_2d_match_numpy(orc, shape):
    dp = _fft(orc.lib)
    n0, n1 = shape
    a = np.random.default_rng(1).standard_normal(shape)
    out = np.zeros((n0, n1 // 2 + 1), complex)
    orc.lib.fft64_r2c_2d(n0, n1, a.ctypes.data_as(dp), out.ctypes.data_as(dp))
    ref = np.fft.rfft2(a)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()
    back = np.zeros(shape)
    orc.lib.fft64_c2r_2d(n0, n1, out.ctypes.data_as(dp), back.ctypes.data_as(dp))
    assert np.abs(back / (n0 * n1) - a).max() <= 1e-12


@pytest.mark.parametrize("name,yk,df", GRAD_CASES)
def test_restated_gradient_matches_reference_fixture(orc, golden, name, yk, df):
    val = golden["sym_val"] / golden["sym_val"].sum()
    dC, z = orc.fft_gradient(golden["sym_row"], golden["sym_col"], val, golden[yk], 3, 1.0, 50, 2, df)
    assert rel_l2(dC, golden[name + "_dC"]) < 1e-12
    assert abs(z - float(golden[name + "_Z"])) <= 1e-12 * abs(float(golden[name + "_Z"]))
    kl = orc.evaluate_error_fft(golden["sym_row"], golden["sym_col"], val, golden[yk], df, float(golden[name + "_Z"]))
    assert abs(kl - float(golden[name + "_KL"])) <= 1e-12 * abs(float(golden[name + "_KL"]))


def test_restated_similarities_match_reference_fixture(orc, golden):
    X = golden["sim_X"]
    row, col, val = orc.gaussian_perplexity(X, float(golden["sim_perp"]), int(golden["sim_K"]), -1.0, 2)
    assert np.array_equal(row, golden["knn_row"]) and np.array_equal(col, golden["knn_col"])
    assert np.abs(val - golden["knn_val"]).max() <= 1e-15
    _, lcol, lval = orc.gaussian_perplexity(X, 0.0, 45, -1.0, 2, perplexity_list=list(golden["list_perps"]))
    assert np.array_equal(lcol, golden["list_col"]) and np.abs(lval - golden["list_val"]).max() <= 1e-15
    _, fcol, fval = orc.gaussian_perplexity(X, -1.0, int(golden["sigma_K"]), float(golden["sigma"]), 2)
    assert np.array_equal(fcol, golden["sigma_col"]) and np.abs(fval - golden["sigma_val"]).max() <= 1e-15


def test_restated_symmetrize_matches_reference_fixture(orc, golden):
    r, c, v = orc.symmetrize(golden["knn_row"], golden["knn_col"], golden["knn_val"], 2000)
    assert np.array_equal(r, golden["sym_row"]) and np.array_equal(c, golden["sym_col"])
    assert np.array_equal(v, golden["sym_val"])


def test_restated_run_matches_reference_fixture(orc, golden):
    Y, costs = orc.run(golden["e2e_X"], golden["e2e_Y0"], no_dims=2, perplexity=15.0, max_iter=300,
                       stop_lying_iter=100, mom_switch_iter=100, learning_rate=200.0, nthreads=2)
    assert np.abs(Y - golden["e2e_Y"]).max() <= 1e-9
    idx = [49, 99, 149, 199, 249, 299]
    assert np.allclose(costs[idx], golden["e2e_costs"][idx], rtol=1e-9)


def test_restated_loop_on_a_given_P_matches_reference_fixture(orc, golden):
    """The loop alone (TSNE::run with load_affinities = 1) on the P the reference builds
    (X centred and scaled by its largest magnitude, VP-tree kNN, calibration,
    symmetrisation, normalisation) reproduces the reference's run."""
    X = golden["e2e_X"]
    X = X - np.cumsum(X, axis=0)[-1] / len(X)  # zeroMean's sequential column sums
    X = X / np.abs(X).max()
    r, c, v = orc.gaussian_perplexity(X, 15.0, 45, nthreads=2)
    r, c, v = orc.symmetrize(r, c, v, len(X))
    v = v / np.cumsum(v)[-1]  # the reference's sequential sum of P
    Y, costs = orc.run_from_P(r, c, v, golden["e2e_Y0"], max_iter=300, stop_lying_iter=100, mom_switch_iter=100,
                              learning_rate=200.0, nthreads=2)
    assert np.abs(Y - golden["e2e_Y"]).max() <= 1e-9
    idx = [49, 99, 149, 199, 249, 299]
    assert np.allclose(costs[idx], golden["e2e_costs"][idx], rtol=1e-9)


def test_restated_knn_is_exact(orc, golden):
    X = golden["sim_X"][:600]
    idx, dist = orc.knn(X, 11, 2)
    full = np.sqrt(((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
    ref = np.sort(full, axis=1)[:, :11]
    assert np.allclose(dist, ref, rtol=0, atol=1e-12)


def test_parity_check_catches_a_planted_error(orc, golden):
    """A perturbation of the size the GPU tolerance allows must not go unnoticed."""
    val = golden["sym_val"] / golden["sym_val"].sum()
    dC, _ = orc.fft_gradient(golden["sym_row"], golden["sym_col"], val, golden["Y2"], 3, 1.0, 50, 1, 1.0)
    bad = dC.copy()
    bad[::7] *= 1.01
    assert rel_l2(bad, golden["g2_df1_dC"]) > 1e-4
    # a different interpolation grid changes the result well above the tolerance
    dC2, _ = orc.fft_gradient(golden["sym_row"], golden["sym_col"], val, golden["Y2"], 3, 1.0, 80, 1, 1.0)
    assert rel_l2(dC2, golden["g2_df1_dC"]) > 1e-4


needs_ref = pytest.mark.skipif(not oracle.reference_available(), reason="reference checker not built here")


@needs_ref
@pytest.mark.parametrize("D,df", [(2, 1.0), (2, 0.7), (1, 1.0), (1, 2.0)])
def test_restated_equals_compiled_reference_on_fresh_inputs(orc, D, df):
    ref = oracle.Reference()
    rng = np.random.default_rng(7 + D)
    N = 1500
    Y = rng.standard_normal((N, D)) * 8
    K = 12
    cols = rng.integers(0, N, (N, K)).astype(np.uint32).ravel()
    row = (np.arange(N + 1) * K).astype(np.uint32)
    val = rng.random(N * K)
    val /= val.sum()
    a, za = ref.fft_gradient(row, cols, val, Y, 3, 1.0, 50, 1, df)
    b, zb = orc.fft_gradient(row, cols, val, Y, 3, 1.0, 50, 3, df)
    assert rel_l2(b, a) < 1e-12 and abs(za - zb) <= 1e-12 * abs(za)


@needs_ref
def test_reference_fft_gradient_close_to_exact_gradient():
    """The interpolation gradient of the compiled reference (with the project FFT) against
    the reference's own O(N^2) exact gradient: validates the FFT shim in place."""
    ref = oracle.Reference()
    rng = np.random.default_rng(3)
    N = 800
    Y = rng.standard_normal((N, 2)) * 6
    P = np.zeros((N, N))
    r = np.repeat(np.arange(N), 8)
    c = rng.integers(0, N, N * 8)
    np.add.at(P, (r, c), rng.random(N * 8))
    P = P + P.T
    np.fill_diagonal(P, 0)
    P /= P.sum()
    nz = [np.nonzero(P[i])[0] for i in range(N)]
    row = np.concatenate([[0], np.cumsum([len(z) for z in nz])]).astype(np.uint32)
    col = np.concatenate(nz).astype(np.uint32)
    val = np.concatenate([P[i, nz[i]] for i in range(N)])
    dC, _ = ref.fft_gradient(row, col, val, Y, 3, 1.0, 50, 1, 1.0)
    ex = ref.exact_gradient(P, Y, 1.0)
    assert rel_l2(dC, ex) < 2e-2
