"""The learned-calibration network's CPU checker against finite differences (no GPU)."""
import numpy as np

import mlp


def _pairs(n=64, K=30, seed=0):
    rng = np.random.default_rng(seed)
    d = np.sort(rng.gamma(3.0, 1.0, (n, K)) * rng.uniform(0.2, 5.0, (n, 1)), axis=1)
    beta = np.array([mlp.bisection_beta(r, 10.0) for r in d])
    return d, beta


def test_param_layout_roundtrip():
    K = 30
    p = np.arange(mlp.param_count(K), dtype=np.float64)
    assert np.array_equal(mlp.pack(*mlp.unpack(p, K)), p)
    assert mlp.param_count(90) == 64 * 90 + 64 + 64 * 64 + 64 + 64 + 1


def test_backprop_matches_central_differences():
    d, beta = _pairs()
    K = d.shape[1]
    rng = np.random.default_rng(1)
    p = rng.standard_normal(mlp.param_count(K)) * 0.2
    mu, sd = 0.5, 1.3
    _, g = mlp.loss_grad(p, d, beta, mu, sd)
    idx = rng.choice(len(p), 60, replace=False)
    for i in idx:
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (mlp.loss_grad(p + e, d, beta, mu, sd)[0] - mlp.loss_grad(p - e, d, beta, mu, sd)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_target_is_scale_free():
    """beta * mean(d) does not change when all distances scale (the network's premise)."""
    d, beta = _pairs(8)
    s = d.mean(1)
    b2 = np.array([mlp.bisection_beta(r * 7.0, 10.0) for r in d])
    assert np.allclose(beta * s, b2 * s * 7.0, rtol=1e-4)
