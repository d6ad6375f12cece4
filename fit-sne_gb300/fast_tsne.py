"""Drop-in replacement of the reference's Python wrapper (fast_tsne.py of FIt-SNE v1.2.1).

Same function, same arguments and defaults, same data.dat / result.dat protocol and the same
``bin/fast_tsne <version> <infile> <outfile> <nthreads>`` call; the binary it runs is this
package's GPU build.  Usage is unchanged::

    import sys; sys.path.append('path/to/fit-sne_gb300')
    from fast_tsne import fast_tsne
    Z = fast_tsne(X)

Differences: knn_algo='annoy' (the reference default) is served by the exact GPU kNN;
nbody_algo='Barnes-Hut' and theta=0 (exact t-SNE) are outside this build and make the
binary exit with an error.  PCA initialisation runs on the GPU (``fitsne.pca``: the
covariance's leading eigenvectors with scikit-learn's sign rule); ``FITSNE_PCA=sklearn``
uses scikit-learn's PCA instead, as the reference does.
"""
from __future__ import annotations

import os
import sys
import struct
import subprocess
from datetime import datetime

import numpy as np

VERSION = "1.2.1"
BINARY = os.path.join(os.path.dirname(os.path.realpath(__file__)), "bin", "fast_tsne")


def _pca_init(X, map_dims, seed):
    """First map_dims principal components, scaled to std 1e-4 on the first axis
    (fast_tsne.py:186-197 of the reference).  Computed on the GPU (fitsne_pca: the
    covariance's leading eigenvectors, each component's largest-magnitude entry positive,
    as scikit-learn's PCA does); FITSNE_PCA=sklearn uses scikit-learn instead."""
    if os.environ.get("FITSNE_PCA") == "sklearn":
        from sklearn.decomposition import PCA
        solver = "arpack" if X.shape[1] > map_dims else "auto"
        pca = PCA(n_components=map_dims, svd_solver=solver, random_state=seed if seed != -1 else None)
        init = pca.fit_transform(X)
    else:
        sys.path.insert(0, os.path.dirname(os.path.realpath(__file__)))
        import fitsne
        init = fitsne.pca(X, map_dims)
    init = init / np.std(init[:, 0])
    return init * 0.0001


def write_data_file(path, X, theta, perplexity, perplexity_list, map_dims, max_iter, stop_early_exag_iter,
                    mom_switch_iter, momentum, final_momentum, learning_rate, max_step_norm, K, sigma, nbody_algo,
                    knn_algo, early_exag_coeff, no_momentum_during_exag, n_trees, search_k, start_late_exag_iter,
                    late_exag_coeff, nterms, intervals_per_integer, min_num_intervals, seed, df, load_affinities,
                    initialization):
    """Writes the binary parameter file in the field order the binary reads."""
    n, d = X.shape
    with open(path, "wb") as f:
        f.write(struct.pack("=i", n))
        f.write(struct.pack("=i", d))
        f.write(struct.pack("=d", theta))
        f.write(struct.pack("=d", perplexity))
        if perplexity == 0:
            f.write(struct.pack("=i", len(perplexity_list)))
            for p in perplexity_list:
                f.write(struct.pack("=d", p))
        for fmt, v in (("=i", map_dims), ("=i", max_iter), ("=i", stop_early_exag_iter), ("=i", mom_switch_iter),
                       ("=d", momentum), ("=d", final_momentum), ("=d", learning_rate), ("=d", max_step_norm),
                       ("=i", K), ("=d", sigma), ("=i", nbody_algo), ("=i", knn_algo), ("=d", early_exag_coeff),
                       ("=i", no_momentum_during_exag), ("=i", n_trees), ("=i", search_k),
                       ("=i", start_late_exag_iter), ("=d", late_exag_coeff), ("=i", nterms),
                       ("=d", intervals_per_integer), ("=i", min_num_intervals)):
            f.write(struct.pack(fmt, v))
        f.write(np.ascontiguousarray(X, dtype=np.float64).tobytes())
        f.write(struct.pack("=i", seed))
        f.write(struct.pack("=d", df))
        f.write(struct.pack("=i", load_affinities))
        if initialization is not None:
            f.write(np.ascontiguousarray(initialization, dtype=np.float64).tobytes())


def read_result_file(path, max_iter):
    """Reads result.dat: the embedding and the loss (NaN where it was not evaluated)."""
    with open(path, "rb") as f:
        (n,) = struct.unpack("=i", f.read(4))
        (md,) = struct.unpack("=i", f.read(4))
        Y = np.frombuffer(f.read(8 * n * md), dtype=np.float64).reshape(n, md).copy()
        (_,) = struct.unpack("=i", f.read(4))
        loss = np.frombuffer(f.read(8 * max_iter), dtype=np.float64).copy()
    loss[np.arange(1, max_iter + 1) % 50 > 0] = np.nan
    return Y, loss


def fast_tsne(X, theta=0.5, perplexity=30, map_dims=2, max_iter=750, stop_early_exag_iter=250, K=-1, sigma=-1,
              nbody_algo="FFT", knn_algo="annoy", mom_switch_iter=250, momentum=0.5, final_momentum=0.8,
              learning_rate="auto", early_exag_coeff=12, no_momentum_during_exag=False, n_trees=50, search_k=None,
              start_late_exag_iter="auto", late_exag_coeff=-1, nterms=3, intervals_per_integer=1,
              min_num_intervals=50, seed=-1, initialization="pca", load_affinities=None, perplexity_list=None, df=1,
              return_loss=False, nthreads=-1, max_step_norm=5):
    """Run t-SNE on the GPU; arguments as in the reference wrapper (see its docstring).

    Returns the N x map_dims embedding, and the loss array when return_loss is True."""
    X = np.array(X).astype(float)
    if learning_rate == "auto":
        learning_rate = np.max((200, X.shape[0] / early_exag_coeff))
    if start_late_exag_iter == "auto":
        start_late_exag_iter = stop_early_exag_iter if late_exag_coeff > 0 else -1
    if isinstance(initialization, str) and initialization == "pca":
        initialization = _pca_init(X, map_dims, seed)
    if perplexity_list is not None:
        perplexity = 0  # the binary reads a perplexity list when perplexity == 0
    if sigma > 0 and K > 0:
        perplexity = -1  # fixed bandwidth when perplexity == -1
    if search_k is None:
        if perplexity > 0:
            search_k = 3 * perplexity * n_trees
        elif perplexity == 0:
            search_k = 3 * np.max(perplexity_list) * n_trees
        else:
            search_k = K * n_trees
    codes_nbody = {"Barnes-Hut": 1, "FFT": 2}
    if nbody_algo not in codes_nbody:
        raise ValueError("nbody_algo should be 'Barnes-Hut' or 'FFT'")
    codes_knn = {"vp-tree": 2, "annoy": 1}
    if knn_algo not in codes_knn:
        raise ValueError("knn_algo should be 'vp-tree' or 'annoy'")
    load_code = {"load": 1, "save": 2}.get(load_affinities, 0)
    if nthreads == -1:
        nthreads = 0
    if max_step_norm == "none":
        max_step_norm = -1
    init = None
    if not isinstance(initialization, str) or initialization != "random":
        init = np.array(initialization).astype(float)

    stamp = str(datetime.now()) + "-" + str(np.random.randint(0, 1000000000))
    infile = os.path.join(os.getcwd(), "data_%s.dat" % stamp)
    outfile = os.path.join(os.getcwd(), "result_%s.dat" % stamp)
    write_data_file(infile, X, theta, perplexity, perplexity_list, map_dims, max_iter, stop_early_exag_iter,
                    mom_switch_iter, momentum, final_momentum, learning_rate, max_step_norm, K, sigma,
                    codes_nbody[nbody_algo], codes_knn[knn_algo], early_exag_coeff, int(bool(no_momentum_during_exag)),
                    n_trees, int(search_k), start_late_exag_iter, late_exag_coeff, nterms, intervals_per_integer,
                    min_num_intervals, seed, df, load_code, init)
    try:
        subprocess.call([BINARY, VERSION, os.path.basename(infile), os.path.basename(outfile), "{}".format(nthreads)],
                        cwd=os.getcwd())
        Y, loss = read_result_file(outfile, max_iter)
    finally:
        for p in (infile, outfile):
            if os.path.exists(p):
                os.remove(p)
    if loss.size == 1:
        loss = loss[np.newaxis]
    return (Y, loss) if return_loss else Y
