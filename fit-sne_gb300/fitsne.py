"""Python binding of the GB300 FIt-SNE library (ctypes over ``include/fitsne_gb300.h``).

Every function here calls the in-tree ``libfitsne_gb300.so``; there is no CPU fallback:
if the library is missing or no GPU is present the call raises :class:`FitsneError`.
Names and argument meanings follow the reference's C++ interface (``TSNE::run``,
``computeFftGradient`` ...); see the C header for the citation of each entry point.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfitsne_gb300.so")
BIN_PATH = os.path.join(HERE, "bin", "fast_tsne")

_u32p = ctypes.POINTER(ctypes.c_uint)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int)
_lib = None

# exported symbols and their signatures (restype, argtypes)
_SIGS = {
    "fitsne_run": (ctypes.c_int, [_f64p, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, _f64p,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_uint, ctypes.c_int,
                                  ctypes.c_int, _f64p, ctypes.c_double, ctypes.c_double]),
    "fitsne_fft_gradient": (ctypes.c_int, [_u32p, _u32p, _f64p, _f64p, ctypes.c_int, ctypes.c_int, _f64p,
                                           ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, _f64p]),
    "fitsne_evaluate_error_fft": (ctypes.c_int, [_u32p, _u32p, _f64p, _f64p, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_double, ctypes.c_double, _f64p]),
    "fitsne_knn": (ctypes.c_int, [_f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u32p, _f64p]),
    "fitsne_distances2similarities": (ctypes.c_int, [_f64p, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                     ctypes.c_double, ctypes.c_int, _f64p, _f64p]),
    "fitsne_gaussian_perplexity": (ctypes.c_int, [_f64p, ctypes.c_int, ctypes.c_int,
                                                  ctypes.POINTER(_u32p), ctypes.POINTER(_u32p),
                                                  ctypes.POINTER(_f64p), ctypes.c_double, ctypes.c_int,
                                                  ctypes.c_double, ctypes.c_uint, ctypes.c_int, _f64p]),
    "fitsne_symmetrize": (ctypes.c_int, [ctypes.POINTER(_u32p), ctypes.POINTER(_u32p), ctypes.POINTER(_f64p),
                                         ctypes.c_int]),
    "fitsne_load_data": (ctypes.c_int, [ctypes.c_char_p] + [ctypes.c_void_p] * 32),
    "fitsne_save_data": (ctypes.c_int, [ctypes.c_char_p, _f64p, _f64p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int]),
    "fitsne_session_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int, _u32p,
                                             _u32p, _f64p, _f64p, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_int]),
    "fitsne_session_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, _f64p]),
    "fitsne_session_create_from_data": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), _f64p, ctypes.c_int,
                                                       ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                       ctypes.c_double, ctypes.c_int, _f64p, _f64p, ctypes.c_int,
                                                       ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                       ctypes.POINTER(ctypes.c_ulonglong)]),
    "fitsne_session_gradient": (ctypes.c_int, [ctypes.c_void_p, _f64p, _f64p]),
    "fitsne_session_get_y": (ctypes.c_int, [ctypes.c_void_p, _f64p]),
    "fitsne_session_set_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fitsne_session_set_graphs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fitsne_session_stage_times": (ctypes.c_int, [ctypes.c_void_p, _f64p]),
    "fitsne_session_launch_shapes": (ctypes.c_int, [ctypes.c_void_p, _i32p]),
    "fitsne_session_destroy": (None, [ctypes.c_void_p]),
    "fitsne_fft_gradient_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                   ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                                   _f64p, ctypes.c_void_p]),
    "fitsne_batch_run": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_f64p), _i32p, _i32p, ctypes.POINTER(_f64p),
                                        ctypes.c_int, _f64p, _f64p, _i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_f64p), _f64p]),
    "fitsne_pca": (ctypes.c_int, [_f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p]),
    "fitsne_set_calibration": (None, [ctypes.c_int]),
    "fitsne_get_calibration": (ctypes.c_int, []),
    "fitsne_calibration_stats": (ctypes.c_int, [_f64p]),
    "fitsne_mlp_param_count": (ctypes.c_int, [ctypes.c_int]),
    "fitsne_mlp_loss_grad": (ctypes.c_int, [_f32p, ctypes.c_int, _f64p, _f64p, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_double, _f32p, _f64p]),
    "fitsne_set_precision": (None, [ctypes.c_int]),
    "fitsne_get_precision": (ctypes.c_int, []),
    "fitsne_last_error": (ctypes.c_char_p, []),
    "fitsne_version": (ctypes.c_char_p, []),
    "fitsne_free": (None, [ctypes.c_void_p]),
}


class FitsneError(RuntimeError):
    """Raised when the native library is missing or a call fails."""


def lib() -> ctypes.CDLL:
    """Loads the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FitsneError("libfitsne_gb300.so not built: run fit-sne_gb300/build.py")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def exported_symbols() -> list[str]:
    """Names declared by the C header (those this binding knows)."""
    return list(_SIGS)


def _check(rc: int) -> None:
    if rc != 0:
        msg = lib().fitsne_last_error()
        raise FitsneError("fitsne error %d: %s" % (rc, msg.decode() if msg else ""))


def _p(a, t):
    return a.ctypes.data_as(t)


def _csr(row_P, col_P, val_P):
    row = np.ascontiguousarray(row_P, dtype=np.uint32)
    col = np.ascontiguousarray(col_P, dtype=np.uint32)
    val = np.ascontiguousarray(val_P, dtype=np.float64)
    if len(col) == 0:
        col = np.zeros(1, np.uint32)
        val = np.zeros(1, np.float64)
    return row, col, val


def set_precision(bits: int) -> None:
    """32 (default FP32 form) or 64 (plain FP64 form) for the one-shot entry points."""
    lib().fitsne_set_precision(int(bits))


def get_precision() -> int:
    return int(lib().fitsne_get_precision())


def batch_run(Xs, perplexities, learning_rates=None, Y0s=None, seeds=None, no_dims=2, max_iter=1000,
              stop_lying_iter=250, mom_switch_iter=250, momentum=0.5, final_momentum=0.8, early_exag_coeff=12.0,
              nterms=3, intervals_per_integer=1.0, min_num_intervals=50, max_step_norm=5.0):
    """Batched form: independent embeddings advanced together (fitsne_batch_run).
    Returns (list of Y, list of costs, stats dict)."""
    nj = len(Xs)
    Xs = [np.ascontiguousarray(X, dtype=np.float64) for X in Xs]
    N = np.array([X.shape[0] for X in Xs], dtype=np.int32)
    D = np.array([X.shape[1] for X in Xs], dtype=np.int32)
    perp = np.ascontiguousarray(perplexities, dtype=np.float64)
    lr = np.ascontiguousarray(learning_rates if learning_rates is not None else [max(200.0, n / 12.0) for n in N],
                              dtype=np.float64)
    skip = Y0s is not None
    Ys = [np.ascontiguousarray(Y0s[j], dtype=np.float64).reshape(N[j], no_dims).copy() if skip
          else np.zeros((N[j], no_dims)) for j in range(nj)]
    sd = np.ascontiguousarray(seeds if seeds is not None else np.arange(nj), dtype=np.int32)
    costs = [np.zeros(max(1, max_iter)) for _ in range(nj)]
    xp = (_f64p * nj)(*[_p(X, _f64p) for X in Xs])
    yp = (_f64p * nj)(*[_p(Y, _f64p) for Y in Ys])
    cp = (_f64p * nj)(*[_p(c, _f64p) for c in costs])
    stats = np.zeros(5)
    _check(lib().fitsne_batch_run(nj, xp, _p(N, _i32p), _p(D, _i32p), yp, no_dims, _p(perp, _f64p), _p(lr, _f64p),
                                  _p(sd, _i32p), int(skip), max_iter, stop_lying_iter, mom_switch_iter, momentum,
                                  final_momentum, early_exag_coeff, nterms, intervals_per_integer, min_num_intervals,
                                  max_step_norm, cp, _p(stats, _f64p)))
    keys = ["similarity_s", "iterate_s", "graph_launches", "graph_instantiations", "chunks_redone"]
    return Ys, costs, dict(zip(keys, stats.tolist()))


def pca(X, n_components=2):
    """First principal components of X on the GPU (fitsne_pca)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    Y = np.zeros((N, n_components))
    _check(lib().fitsne_pca(_p(X, _f64p), N, D, int(n_components), _p(Y, _f64p)))
    return Y


def set_calibration(mode) -> None:
    """"bisection" (0, the reference's; default) or "learned" (1, MLP warm start) for the
    similarity stage's perplexity calibration."""
    m = {"bisection": 0, "learned": 1}.get(mode, mode)
    lib().fitsne_set_calibration(int(m))


def get_calibration() -> str:
    return "learned" if lib().fitsne_get_calibration() == 1 else "bisection"


def calibration_stats() -> dict:
    """Statistics of the last calibration (see fitsne_calibration_stats in the header)."""
    out = np.zeros(12)
    _check(lib().fitsne_calibration_stats(out.ctypes.data_as(_f64p)))
    keys = ["rows", "rows_harvest", "rows_fallback", "train_steps", "evals_plain", "evals_warm", "loss_first",
            "loss_last", "ms_harvest", "ms_train", "ms_infer", "ms_warm"]
    return dict(zip(keys, out.tolist()))


def mlp_param_count(K: int) -> int:
    return int(lib().fitsne_mlp_param_count(int(K)))


def mlp_loss_grad(params, dist, beta, mu=0.0, sd=1.0):
    """(loss, grad) of the calibration network on the GPU for the rows of dist (nrows x K)."""
    dist = np.ascontiguousarray(dist, dtype=np.float64)
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    params = np.ascontiguousarray(params, dtype=np.float32)
    nrows, K = dist.shape
    grad = np.zeros_like(params)
    loss = np.zeros(1)
    _check(lib().fitsne_mlp_loss_grad(params.ctypes.data_as(_f32p), K, dist.ctypes.data_as(_f64p),
                                      beta.ctypes.data_as(_f64p), nrows, float(mu), float(sd),
                                      grad.ctypes.data_as(_f32p), loss.ctypes.data_as(_f64p)))
    return float(loss[0]), grad


def fft_gradient(row_P, col_P, val_P, Y, nterms=3, intervals_per_integer=1.0, min_num_intervals=50, df=1.0):
    """One FFT-interpolation gradient (computeFftGradient* of the reference).

    Returns ``(dC, sum_Q)`` with dC of Y's shape (N x no_dims)."""
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    if Y.ndim == 1:
        Y = Y[:, None]
    N, d = Y.shape
    row, col, val = _csr(row_P, col_P, val_P)
    dC = np.zeros((N, d))
    z = ctypes.c_double(0.0)
    _check(lib().fitsne_fft_gradient(_p(row, _u32p), _p(col, _u32p), _p(val, _f64p), _p(Y, _f64p), N, d,
                                     _p(dC, _f64p), int(nterms), float(intervals_per_integer),
                                     int(min_num_intervals), float(df), ctypes.byref(z)))
    return dC, z.value


def evaluate_error_fft(row_P, col_P, val_P, Y, df, sum_Q) -> float:
    """KL over the edges with a given Z (evaluateErrorFft of the reference)."""
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    if Y.ndim == 1:
        Y = Y[:, None]
    N, d = Y.shape
    row, col, val = _csr(row_P, col_P, val_P)
    c = ctypes.c_double(0.0)
    _check(lib().fitsne_evaluate_error_fft(_p(row, _u32p), _p(col, _u32p), _p(val, _f64p), _p(Y, _f64p), N, d,
                                           float(df), float(sum_Q), ctypes.byref(c)))
    return c.value


def knn(X, K):
    """Exact K nearest neighbours, self included: ``(indices[N,K] u32, distances[N,K])``."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    idx = np.zeros((N, K), np.uint32)
    dist = np.zeros((N, K))
    _check(lib().fitsne_knn(_p(X, _f64p), N, D, int(K), _p(idx, _u32p), _p(dist, _f64p)))
    return idx, dist


def distances2similarities(Dist, perplexity, sigma=-1.0, perplexity_list=None):
    """Row-wise calibration of K neighbour distances: ``(P[nrows,K], betas[nrows])``."""
    Dist = np.ascontiguousarray(Dist, dtype=np.float64)
    nrows, K = Dist.shape
    P = np.zeros_like(Dist)
    betas = np.zeros(nrows)
    pl = np.ascontiguousarray(perplexity_list if perplexity_list is not None else [0.0], dtype=np.float64)
    npl = 0 if perplexity_list is None else len(perplexity_list)
    _check(lib().fitsne_distances2similarities(_p(Dist, _f64p), _p(P, _f64p), nrows, K, float(perplexity),
                                               float(sigma), npl, _p(pl, _f64p), _p(betas, _f64p)))
    return P, betas


def _take_malloced(ptr, n, ctype, dtype):
    arr = np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True) if n else np.zeros(0, dtype)
    lib().fitsne_free(ctypes.cast(ptr, ctypes.c_void_p))
    return arr


def gaussian_perplexity(X, perplexity, K, sigma=-1.0, perplexity_list=None):
    """kNN + calibration (computeGaussianPerplexity, VP-tree overload): CSR (row, col, val)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    r, c, v = _u32p(), _u32p(), _f64p()
    pl = np.ascontiguousarray(perplexity_list if perplexity_list is not None else [0.0], dtype=np.float64)
    npl = 0 if perplexity_list is None else len(perplexity_list)
    _check(lib().fitsne_gaussian_perplexity(_p(X, _f64p), N, D, ctypes.byref(r), ctypes.byref(c),
                                            ctypes.byref(v), float(perplexity), int(K), float(sigma), 0, npl,
                                            _p(pl, _f64p)))
    row = _take_malloced(r, N + 1, ctypes.c_uint, np.uint32)
    nnz = int(row[-1])
    return row, _take_malloced(c, nnz, ctypes.c_uint, np.uint32), _take_malloced(v, nnz, ctypes.c_double,
                                                                                   np.float64)


def _malloc_copy(a, ctype):
    libc = ctypes.CDLL(None)
    libc.malloc.restype = ctypes.c_void_p
    libc.malloc.argtypes = [ctypes.c_size_t]
    n = max(1, a.nbytes)
    p = libc.malloc(n)
    if not p:
        raise MemoryError
    ctypes.memmove(p, a.ctypes.data, a.nbytes)
    return ctypes.cast(p, ctypes.POINTER(ctype))


def symmetrize(row_P, col_P, val_P, N):
    """(P + P^T)/2 on the union pattern (symmetrizeMatrix): returns the new CSR."""
    row, col, val = _csr(row_P, col_P, val_P)
    r = _malloc_copy(row, ctypes.c_uint)
    c = _malloc_copy(col, ctypes.c_uint)
    v = _malloc_copy(val, ctypes.c_double)
    rc = lib().fitsne_symmetrize(ctypes.byref(r), ctypes.byref(c), ctypes.byref(v), int(N))
    _check(rc)
    row2 = _take_malloced(r, N + 1, ctypes.c_uint, np.uint32)
    nnz = int(row2[-1])
    return row2, _take_malloced(c, nnz, ctypes.c_uint, np.uint32), _take_malloced(v, nnz, ctypes.c_double,
                                                                                   np.float64)


def run(X, no_dims=2, perplexity=30.0, theta=0.5, rand_seed=-1, Y0=None, max_iter=1000, stop_lying_iter=250,
        mom_switch_iter=250, momentum=0.5, final_momentum=0.8, learning_rate=200.0, K=-1, sigma=-1.0,
        nbody_algorithm=2, knn_algo=2, early_exag_coeff=12.0, no_momentum_during_exag=False,
        start_late_exag_iter=-1, late_exag_coeff=-1.0, n_trees=50, search_k=-1, nterms=3,
        intervals_per_integer=1.0, min_num_intervals=50, nthreads=0, load_affinities=0, perplexity_list=None,
        df=1.0, max_step_norm=5.0):
    """TSNE::run with the reference's argument meaning; returns ``(Y, costs)``."""
    # fitsne_run only reads X, but uploading from a fresh copy measured faster on the GB300
    # hosts: at N = 1M x 50 the similarity stage took 0.24 s after the copy (~0.04 s) against
    # 0.33 - 0.37 s straight from the caller's array
    X = np.ascontiguousarray(X, dtype=np.float64).copy()
    N, D = X.shape
    Y = np.zeros((N, no_dims)) if Y0 is None else np.ascontiguousarray(Y0, dtype=np.float64).reshape(N, no_dims).copy()
    costs = np.zeros(max_iter)
    pl = np.ascontiguousarray(perplexity_list if perplexity_list is not None else [0.0], dtype=np.float64)
    npl = 0 if perplexity_list is None else len(perplexity_list)
    _check(lib().fitsne_run(_p(X, _f64p), N, D, _p(Y, _f64p), int(no_dims), float(perplexity), float(theta),
                            int(rand_seed), 0 if Y0 is None else 1, int(max_iter), int(stop_lying_iter),
                            int(mom_switch_iter), float(momentum), float(final_momentum), float(learning_rate),
                            int(K), float(sigma), int(nbody_algorithm), int(knn_algo), float(early_exag_coeff),
                            _p(costs, _f64p), int(bool(no_momentum_during_exag)), int(start_late_exag_iter),
                            float(late_exag_coeff), int(n_trees), int(search_k), int(nterms),
                            float(intervals_per_integer), int(min_num_intervals), int(nthreads),
                            int(load_affinities), npl, _p(pl, _f64p), float(df), float(max_step_norm)))
    return Y, costs


class Session:
    """Device-resident optimisation of one embedding (P and Y stay on the GPU)."""

    def __init__(self, row_P, col_P, val_P, Y0, nterms=3, intervals_per_integer=1.0, min_num_intervals=50,
                 df=1.0, precision=32):
        Y0 = np.ascontiguousarray(Y0, dtype=np.float64)
        if Y0.ndim == 1:
            Y0 = Y0[:, None]
        self.N, self.no_dims = Y0.shape
        self._row, self._col, self._val = _csr(row_P, col_P, val_P)
        h = ctypes.c_void_p()
        _check(lib().fitsne_session_create(ctypes.byref(h), self.N, self.no_dims, _p(self._row, _u32p),
                                           _p(self._col, _u32p), _p(self._val, _f64p), _p(Y0, _f64p), int(nterms),
                                           float(intervals_per_integer), int(min_num_intervals), float(df),
                                           int(precision)))
        self._h = h

    @classmethod
    def from_data(cls, X, Y0, perplexity=30.0, K=-1, sigma=-1.0, perplexity_list=None, nterms=3,
                  intervals_per_integer=1.0, min_num_intervals=50, df=1.0, precision=32):
        """Builds P on the GPU from the data (as TSNE::run does) and keeps it there."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        Y0 = np.ascontiguousarray(Y0, dtype=np.float64)
        if Y0.ndim == 1:
            Y0 = Y0[:, None]
        N, D = X.shape
        pl = np.ascontiguousarray(perplexity_list if perplexity_list is not None else [0.0], dtype=np.float64)
        npl = 0 if perplexity_list is None else len(perplexity_list)
        if perplexity_list is not None:
            perplexity = 0.0
        self = cls.__new__(cls)
        self.N, self.no_dims = Y0.shape
        h = ctypes.c_void_p()
        nnz = ctypes.c_ulonglong(0)
        _check(lib().fitsne_session_create_from_data(ctypes.byref(h), _p(X, _f64p), N, D, self.no_dims,
                                                     float(perplexity), int(K), float(sigma), npl, _p(pl, _f64p),
                                                     _p(Y0, _f64p), int(nterms), float(intervals_per_integer),
                                                     int(min_num_intervals), float(df), int(precision),
                                                     ctypes.byref(nnz)))
        self._h = h
        self.nnz = int(nnz.value)
        return self

    def gradient(self):
        """Gradient at the current Y without an update: ``(dC, sum_Q)``."""
        dC = np.zeros((self.N, self.no_dims))
        z = ctypes.c_double(0.0)
        _check(lib().fitsne_session_gradient(self._h, _p(dC, _f64p), ctypes.byref(z)))
        return dC, z.value

    def run(self, it0, it1, max_iter=1000, stop_lying_iter=250, mom_switch_iter=250, momentum=0.5,
            final_momentum=0.8, learning_rate=200.0, early_exag_coeff=12.0, no_momentum_during_exag=False,
            start_late_exag_iter=-1, late_exag_coeff=-1.0, max_step_norm=5.0, costs=None):
        cp = _p(costs, _f64p) if costs is not None else None
        _check(lib().fitsne_session_run(self._h, int(it0), int(it1), int(max_iter), int(stop_lying_iter),
                                        int(mom_switch_iter), float(momentum), float(final_momentum),
                                        float(learning_rate), float(early_exag_coeff),
                                        int(bool(no_momentum_during_exag)), int(start_late_exag_iter),
                                        float(late_exag_coeff), float(max_step_norm), cp))

    def get_y(self):
        Y = np.zeros((self.N, self.no_dims))
        _check(lib().fitsne_session_get_y(self._h, _p(Y, _f64p)))
        return Y

    def set_timing(self, on=True):
        _check(lib().fitsne_session_set_timing(self._h, int(bool(on))))

    def set_graphs(self, on=True):
        _check(lib().fitsne_session_set_graphs(self._h, int(bool(on))))

    def stage_times(self):
        out = np.zeros(10)
        _check(lib().fitsne_session_stage_times(self._h, _p(out, _f64p)))
        return out

    def launch_shapes(self):
        """The autotuner's choices: attraction shape index, rows per work item, edges per lane,
        attraction form (0 full CSR, 2 tiled), FFT threads per block."""
        out = np.zeros(5, np.int32)
        _check(lib().fitsne_session_launch_shapes(self._h, _p(out, _i32p)))
        keys = ["attr_shape", "attr_rows_per_item", "attr_edges_per_lane", "attr_form", "fft_threads"]
        return dict(zip(keys, [int(v) for v in out]))

    def close(self):
        if getattr(self, "_h", None):
            lib().fitsne_session_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
