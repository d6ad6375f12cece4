"""PCA initialisation on the GPU (fast_tsne.py:186-197 of the reference uses scikit-learn's
PCA; scikit-learn is not on every machine, so the check is an FP64 SVD with its sign rule).
The Gram matrix and the projection are the library's own kernels; 2500 x 200 with 120
components takes the projection in slices of the components."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _svd_pca(X, k):
    Xc = X - X.mean(0)
    U, S, Vt = np.linalg.svd(Xc, full_matrices=False)
    Vt = Vt[:k]
    # scikit-learn's svd_flip(u_based_decision=False): largest |entry| of each component positive
    s = np.sign(Vt[np.arange(k), np.argmax(np.abs(Vt), axis=1)])
    return Xc @ (Vt * s[:, None]).T


@pytest.mark.parametrize("N,D,k", [(5000, 50, 2), (1200, 7, 1), (3000, 120, 2), (20, 3, 3), (2500, 200, 120)])
def test_pca_matches_fp64_svd(gpu_lib, N, D, k):
    rng = np.random.default_rng(N + D)
    X = rng.standard_normal((N, D)) * np.linspace(5.0, 0.5, D) + rng.standard_normal(D) * 3
    Y = gpu_lib.pca(X, k)
    ref = _svd_pca(X, k)
    assert np.abs(Y - ref).max() <= 1e-8 * np.abs(ref).max()


def test_wrapper_uses_gpu_pca(gpu_lib, monkeypatch):
    import fast_tsne as ft
    rng = np.random.default_rng(1)
    X = rng.standard_normal((800, 10)) * np.linspace(3.0, 1.0, 10)
    init = ft._pca_init(X, 2, -1)
    ref = _svd_pca(X, 2)
    ref = ref / np.std(ref[:, 0]) * 1e-4
    assert np.abs(init - ref).max() <= 1e-10
