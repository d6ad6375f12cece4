"""CPU oracle access (TEST INFRASTRUCTURE ONLY).

Two checkers live under oracle/:
  * ``Restated``  -- oracle/_build/libfitsne_oracle.so, the C restatement of the reference
    algorithm (fitsne_oracle.c); builds anywhere with gcc and is the CPU baseline;
  * ``Reference`` -- oracle/_ref/libfitsne_ref.so, the UNMODIFIED reference sources compiled
    against the project FFT shim; only buildable where the reference tree is present.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESTATED_LIB = os.path.join(HERE, "_build", "libfitsne_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfitsne_ref.so")
REF_BIN = os.path.join(HERE, "_ref", "fast_tsne_ref")

_u32p = ctypes.POINTER(ctypes.c_uint)
_f64p = ctypes.POINTER(ctypes.c_double)


def _p(a, t):
    return a.ctypes.data_as(t)


def build_restated(force: bool = False) -> str:
    """Compiles the C restatement (gcc, OpenMP) into oracle/_build/."""
    if force or not os.path.exists(RESTATED_LIB) or \
            os.path.getmtime(RESTATED_LIB) < max(os.path.getmtime(os.path.join(HERE, f))
                                                 for f in ("fitsne_oracle.c", "fft64.c", "fft64.h")):
        subprocess.run(["make", "-C", HERE, "restate"], check=True, capture_output=True)
    return RESTATED_LIB


def reference_dir() -> str:
    """The FIt-SNE checkout: $FITSNE_REFERENCE_DIR when set, else a directory named
    ``reference`` beside this repository."""
    env = os.environ.get("FITSNE_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build_reference(ref_root: str | None = None) -> str | None:
    """Compiles the reference checker when the reference tree exists; else None."""
    ref_root = ref_root or reference_dir()
    if not os.path.isdir(os.path.join(ref_root, "src")):
        return REF_LIB if os.path.exists(REF_LIB) else None
    subprocess.run(["make", "-C", HERE, "ref", "REF=" + ref_root], check=True, capture_output=True)
    return REF_LIB


def _csr(row, col, val):
    return (np.ascontiguousarray(row, np.uint32), np.ascontiguousarray(col, np.uint32),
            np.ascontiguousarray(val, np.float64))


class _Common:
    prefix = ""

    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        L, pf = self.lib, self.prefix
        f = getattr(L, pf + "fft_gradient")
        f.restype = ctypes.c_double
        f.argtypes = [_u32p, _u32p, _f64p, _f64p, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int,
                      ctypes.c_double, ctypes.c_int, ctypes.c_uint, ctypes.c_double]
        f = getattr(L, pf + "evaluate_error_fft")
        f.restype = ctypes.c_double
        f.argtypes = [_u32p, _u32p, _f64p, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        f = getattr(L, pf + "distances2similarities")
        f.restype = ctypes.c_double
        f.argtypes = [_f64p, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                      ctypes.c_int, _f64p]
        f = getattr(L, pf + "gaussian_perplexity_vptree")
        f.restype = None
        f.argtypes = [_f64p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_u32p), ctypes.POINTER(_u32p),
                      ctypes.POINTER(_f64p), ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_uint,
                      ctypes.c_int, _f64p]
        f = getattr(L, pf + "symmetrize")
        f.restype = None
        f.argtypes = [ctypes.POINTER(_u32p), ctypes.POINTER(_u32p), ctypes.POINTER(_f64p), ctypes.c_int]
        f = getattr(L, pf + "run")
        f.restype = ctypes.c_int
        f.argtypes = [_f64p, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                      ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                      ctypes.c_double, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                      ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_uint, ctypes.c_int,
                      ctypes.c_int, _f64p, ctypes.c_double, ctypes.c_double]
        f = getattr(L, pf + "free")
        f.restype = None
        f.argtypes = [ctypes.c_void_p]

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def fft_gradient(self, row, col, val, Y, nterms=3, ipi=1.0, min_num_intervals=50, nthreads=1, df=1.0):
        row, col, val = _csr(row, col, val)
        Y = np.ascontiguousarray(Y, np.float64)
        if Y.ndim == 1:
            Y = Y[:, None]
        N, d = Y.shape
        dC = np.zeros((N, d))
        z = self._fn("fft_gradient")(_p(row, _u32p), _p(col, _u32p), _p(val, _f64p), _p(Y, _f64p), N, d,
                                     _p(dC, _f64p), nterms, ipi, min_num_intervals, nthreads, df)
        return dC, z

    def evaluate_error_fft(self, row, col, val, Y, df, sum_Q):
        row, col, val = _csr(row, col, val)
        Y = np.ascontiguousarray(Y, np.float64)
        if Y.ndim == 1:
            Y = Y[:, None]
        N, d = Y.shape
        return self._fn("evaluate_error_fft")(_p(row, _u32p), _p(col, _u32p), _p(val, _f64p), _p(Y, _f64p), N, d,
                                              df, sum_Q)

    def distances2similarities(self, Drow, perplexity, sigma=-1.0, perplexity_list=None):
        """One row of K non-squared distances (self removed), as the kNN paths call it."""
        Drow = np.ascontiguousarray(Drow, np.float64)
        P = np.zeros_like(Drow)
        pl = np.ascontiguousarray(perplexity_list if perplexity_list is not None else [0.0], np.float64)
        npl = 0 if perplexity_list is None else len(perplexity_list)
        beta = self._fn("distances2similarities")(_p(Drow, _f64p), _p(P, _f64p), len(Drow), -1, perplexity,
                                                  sigma, 0, npl, _p(pl, _f64p))
        return P, beta

    def _take(self, ptr, n, dtype):
        arr = np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True) if n else np.zeros(0, dtype)
        self._fn("free")(ctypes.cast(ptr, ctypes.c_void_p))
        return arr

    def gaussian_perplexity(self, X, perplexity, K, sigma=-1.0, nthreads=1, perplexity_list=None):
        X = np.ascontiguousarray(X, np.float64)
        N, D = X.shape
        r, c, v = _u32p(), _u32p(), _f64p()
        pl = np.ascontiguousarray(perplexity_list if perplexity_list is not None else [0.0], np.float64)
        npl = 0 if perplexity_list is None else len(perplexity_list)
        self._fn("gaussian_perplexity_vptree")(_p(X, _f64p), N, D, ctypes.byref(r), ctypes.byref(c),
                                               ctypes.byref(v), perplexity, K, sigma, nthreads, npl, _p(pl, _f64p))
        row = self._take(r, N + 1, np.uint32)
        nnz = int(row[-1])
        return row, self._take(c, nnz, np.uint32), self._take(v, nnz, np.float64)

    def symmetrize(self, row, col, val, N):
        libc = ctypes.CDLL(None)
        libc.malloc.restype = ctypes.c_void_p
        libc.malloc.argtypes = [ctypes.c_size_t]

        def mc(a, t):
            p = libc.malloc(max(1, a.nbytes))
            ctypes.memmove(p, a.ctypes.data, a.nbytes)
            return ctypes.cast(p, ctypes.POINTER(t))
        row, col, val = _csr(row, col, val)
        r, c, v = mc(row, ctypes.c_uint), mc(col, ctypes.c_uint), mc(val, ctypes.c_double)
        self._fn("symmetrize")(ctypes.byref(r), ctypes.byref(c), ctypes.byref(v), N)
        row2 = self._take(r, N + 1, np.uint32)
        nnz = int(row2[-1])
        return row2, self._take(c, nnz, np.uint32), self._take(v, nnz, np.float64)

    def run(self, X, Y0, no_dims=2, perplexity=30.0, max_iter=1000, stop_lying_iter=250, mom_switch_iter=250,
            momentum=0.5, final_momentum=0.8, learning_rate=200.0, K=-1, sigma=-1.0, early_exag_coeff=12.0,
            no_momentum_during_exag=0, start_late_exag_iter=-1, late_exag_coeff=-1.0, nterms=3, ipi=1.0,
            min_num_intervals=50, nthreads=1, perplexity_list=None, df=1.0, max_step_norm=5.0, knn_algo=2,
            rand_seed=-1, load_affinities=0):
        X = np.ascontiguousarray(X, np.float64).copy()
        N, D = X.shape
        skip = Y0 is not None
        Y = np.zeros((N, no_dims)) if Y0 is None else np.ascontiguousarray(Y0, np.float64).reshape(N, no_dims).copy()
        costs = np.zeros(max_iter)
        pl = np.ascontiguousarray(perplexity_list if perplexity_list is not None else [0.0], np.float64)
        npl = 0 if perplexity_list is None else len(perplexity_list)
        if perplexity_list is not None:
            perplexity = 0.0
        rc = self._fn("run")(_p(X, _f64p), N, D, _p(Y, _f64p), no_dims, perplexity, 0.5, rand_seed, int(skip),
                             max_iter, stop_lying_iter, mom_switch_iter, momentum, final_momentum, learning_rate, K,
                             sigma, 2, knn_algo, early_exag_coeff, _p(costs, _f64p), int(no_momentum_during_exag),
                             start_late_exag_iter, late_exag_coeff, 50, -1, nterms, ipi, min_num_intervals,
                             nthreads, int(load_affinities), npl, _p(pl, _f64p), df, max_step_norm)
        if rc != 0:
            raise RuntimeError("run returned %d" % rc)
        return Y, costs


class Reference(_Common):
    """The unmodified reference compiled against the FFT shim."""
    prefix = "ref_"

    def __init__(self, path: str = REF_LIB):
        super().__init__(path)
        self.lib.ref_exact_gradient.restype = None
        self.lib.ref_exact_gradient.argtypes = [_f64p, _f64p, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_double]

    def exact_gradient(self, P, Y, df=1.0):
        P = np.ascontiguousarray(P, np.float64)
        Y = np.ascontiguousarray(Y, np.float64)
        if Y.ndim == 1:
            Y = Y[:, None]
        N, d = Y.shape
        dC = np.zeros((N, d))
        self.lib.ref_exact_gradient(_p(P, _f64p), _p(Y, _f64p), N, d, _p(dC, _f64p), df)
        return dC


class Restated(_Common):
    """The C restatement (fitsne_oracle.c)."""
    prefix = "orc_"

    def __init__(self, path: str = RESTATED_LIB):
        super().__init__(path)
        L = self.lib
        L.orc_knn.restype = None
        L.orc_knn.argtypes = [_f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u32p, _f64p, ctypes.c_int]
        L.orc_run_from_P.restype = ctypes.c_int
        L.orc_run_from_P.argtypes = [_u32p, _u32p, _f64p, ctypes.c_int, _f64p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_uint, ctypes.c_double,
                                     ctypes.c_double]
        L.orc_gradient_step.restype = ctypes.c_int
        L.orc_gradient_step.argtypes = [_u32p, _u32p, _f64p, _f64p, _f64p, _f64p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_uint,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_double]

    def knn(self, X, K, nthreads=1):
        """Exact brute-force kNN in FP64 (self included): indices, non-squared distances."""
        X = np.ascontiguousarray(X, np.float64)
        N, D = X.shape
        idx = np.zeros((N, K), np.uint32)
        dist = np.zeros((N, K))
        self.lib.orc_knn(_p(X, _f64p), N, D, K, _p(idx, _u32p), _p(dist, _f64p), nthreads)
        return idx, dist

    def run_from_P(self, row, col, val, Y0, max_iter=1000, stop_lying_iter=250, mom_switch_iter=250, momentum=0.5,
                   final_momentum=0.8, learning_rate=200.0, early_exag_coeff=12.0, no_momentum_during_exag=0,
                   start_late_exag_iter=-1, late_exag_coeff=-1.0, nterms=3, ipi=1.0, min_num_intervals=50,
                   nthreads=1, df=1.0, max_step_norm=5.0):
        """TSNE::run's loop on a given (symmetrised, normalised) P from Y0, as with
        load_affinities = 1: returns (Y, costs)."""
        row, col, val = _csr(row, col, val)
        Y = np.ascontiguousarray(Y0, np.float64).copy()
        if Y.ndim == 1:
            Y = Y[:, None]
        N, d = Y.shape
        costs = np.zeros(max(1, max_iter))
        self.lib.orc_run_from_P(_p(row, _u32p), _p(col, _u32p), _p(val, _f64p), N, _p(Y, _f64p), d, max_iter,
                                stop_lying_iter, mom_switch_iter, momentum, final_momentum, learning_rate,
                                early_exag_coeff, _p(costs, _f64p), int(no_momentum_during_exag),
                                start_late_exag_iter, late_exag_coeff, nterms, ipi, min_num_intervals, nthreads, df,
                                max_step_norm)
        return Y, costs

    def gradient_step(self, row, col, val, Y, uY, gains, nterms=3, ipi=1.0, min_num_intervals=50, nthreads=1,
                      df=1.0, exag=1.0, momentum=0.5, learning_rate=200.0, use_gains=1, max_step_norm=5.0):
        """One iteration of the reference loop (gradient + update + zero-mean) in place."""
        row, col, val = _csr(row, col, val)
        N, d = Y.shape
        return self.lib.orc_gradient_step(_p(row, _u32p), _p(col, _u32p), _p(val, _f64p), _p(Y, _f64p),
                                          _p(uY, _f64p), _p(gains, _f64p), N, d, nterms, min_num_intervals, ipi,
                                          nthreads, 0, df, exag, momentum, learning_rate, use_gains, max_step_norm)


def reference_available() -> bool:
    return os.path.exists(REF_LIB)
