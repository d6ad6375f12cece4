"""Learned warm start of the perplexity calibration on the GPU, checked against the CPU
checker (oracle/mlp.py) and against the plain bisection it seeds."""
import json

import numpy as np
import pytest

import mlp

pytestmark = pytest.mark.gpu


def _mixture(N, D, seed):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((12, D)) * 4.0
    X = c[rng.integers(0, 12, N)] + rng.standard_normal((N, D)) * rng.uniform(0.5, 2.0, (N, 1))
    X -= X.mean(0)
    return X / np.abs(X).max()


@pytest.mark.parametrize("K,n,seed", [(90, 700, 0), (30, 257, 1), (151, 64, 2)])
def test_training_gradient_matches_cpu_checker(gpu_lib, K, n, seed):
    rng = np.random.default_rng(seed)
    d = np.sort(rng.gamma(3.0, 1.0, (n, K)) * rng.uniform(0.2, 5.0, (n, 1)), axis=1)
    beta = np.array([mlp.bisection_beta(r, 30.0) for r in d])
    p = (rng.standard_normal(mlp.param_count(K)) * 0.15).astype(np.float32)
    assert gpu_lib.mlp_param_count(K) == mlp.param_count(K)
    mu, sd = 0.3, 1.7
    loss, g = gpu_lib.mlp_loss_grad(p, d, beta, mu, sd)
    loss_ref, g_ref = mlp.loss_grad(p.astype(np.float64), d, beta, mu, sd)
    # FP32 kernels (features, activations, atomically summed gradients) vs FP64
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)


def test_learned_calibration_matches_bisection_and_saves_evaluations(gpu_lib):
    N, perp, K = 60000, 30.0, 90
    X = _mixture(N, 20, 3)
    gpu_lib.set_calibration("bisection")
    r0, c0, v0 = gpu_lib.gaussian_perplexity(X, perp, K)
    plain = gpu_lib.calibration_stats()
    gpu_lib.set_calibration("learned")
    try:
        r1, c1, v1 = gpu_lib.gaussian_perplexity(X, perp, K)
        st = gpu_lib.calibration_stats()
    finally:
        gpu_lib.set_calibration("bisection")
    assert np.array_equal(r0, r1) and np.array_equal(c0, c1)
    nh = int(st["rows_harvest"])
    assert nh == 10000 and st["rows"] == N
    P0 = v0.reshape(N, K)
    P1 = v1.reshape(N, K)
    # harvested rows: the plain bisection itself
    assert np.array_equal(P0[:nh], P1[:nh])
    # predicted rows: |H - log perplexity| < 1e-6 (the plain rule stops at 1e-5)
    H1 = -(P1[nh:] * np.log(P1[nh:])).sum(1)
    assert np.abs(H1 - np.log(perp)).max() < 1e-6 + 1e-12
    H0 = -(P0 * np.log(P0)).sum(1)
    assert np.abs(H0 - np.log(perp)).max() < 1e-5 + 1e-12
    # the two P agree to what the plain bisection's tolerance leaves open
    assert np.abs(P1 - P0).max() <= 2e-3 * P0.max()
    # what the network gains: entropy evaluations per row
    assert plain["evals_plain"] > 10
    msg = json.dumps(st)
    assert st["evals_warm"] < st["evals_plain"] / 3.0, msg
    assert st["loss_last"] < 0.2 * st["loss_first"], msg


def test_learned_calibration_run_final_kl_within_one_percent(gpu_lib):
    N = 30000
    X = _mixture(N, 30, 4)
    Y0 = np.random.default_rng(5).standard_normal((N, 2)) * 1e-4
    kw = dict(Y0=Y0, perplexity=30.0, learning_rate=N / 12.0, max_iter=500, knn_algo=2)
    _, c_plain = gpu_lib.run(X, **kw)
    gpu_lib.set_calibration("learned")
    try:
        _, c_learned = gpu_lib.run(X, **kw)
        st = gpu_lib.calibration_stats()
    finally:
        gpu_lib.set_calibration("bisection")
    assert st["rows_harvest"] == 10000 and st["evals_warm"] < st["evals_plain"]
    assert abs(c_learned[-1] - c_plain[-1]) <= 0.01 * abs(c_plain[-1])
