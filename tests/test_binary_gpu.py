"""The drop-in fast_tsne binary and Python wrapper on the GPU."""
import os
import subprocess

import numpy as np
import pytest

import fast_tsne as ft
import oracle

pytestmark = pytest.mark.gpu


def test_binary_rejects_wrong_version():
    r = subprocess.run([ft.BINARY, "0.0.0"], capture_output=True, text=True)
    assert r.returncode != 0 and "wrong version" in r.stdout


def test_wrapper_end_to_end_matches_reference_kl(golden, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    Y, loss = ft.fast_tsne(golden["e2e_X"], perplexity=15, max_iter=300, stop_early_exag_iter=100,
                           mom_switch_iter=100, learning_rate=200, initialization=golden["e2e_Y0"],
                           knn_algo="vp-tree", return_loss=True)
    ref = golden["e2e_costs"]
    # 1,000 points, FP32 form: the optimiser's chaos spreads the KL of repeated runs by up to
    # 1.4e-2 after the exaggeration (see test_run_gpu.py); 1% is tested at 5,000 points there
    for i in (99, 199, 299):
        assert abs(loss[i] - ref[i]) <= 3e-2 * ref[i]
    assert np.isnan(loss[0]) and Y.shape == (len(golden["e2e_X"]), 2)
    assert not [f for f in os.listdir(tmp_path) if f.endswith(".dat")]


def test_wrapper_1d_with_annoy_request(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    rng = np.random.default_rng(5)
    X = np.concatenate([rng.standard_normal((150, 6)) + c for c in (0, 5, 10)])
    Y = ft.fast_tsne(X, map_dims=1, perplexity=10, max_iter=200, df=0.5, initialization="random", seed=3)
    assert Y.shape == (450, 1) and np.isfinite(Y).all()
