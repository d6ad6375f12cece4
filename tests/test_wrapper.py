"""The drop-in Python wrapper: option mapping and the data.dat it writes, checked against
the reference wrapper's documented layout with a stub in place of the binary."""
import os
import stat
import struct
import sys

import numpy as np
import pytest

import fast_tsne as ft


@pytest.fixture
def stub_binary(tmp_path, monkeypatch):
    """A stand-in binary that copies the data file and writes a valid result file."""
    script = tmp_path / "fast_tsne_stub.py"
    script.write_text(
        "import sys, struct, shutil\n"
        "ver, inf, outf = sys.argv[1:4]\n"
        "shutil.copy(inf, 'captured.dat')\n"
        "raw = open(inf,'rb').read()\n"
        "n, d = struct.unpack('=ii', raw[:8])\n"
        "open(outf,'wb').write(struct.pack('=ii', n, 2) + b'\\x00'*(16*n) + struct.pack('=i', 100) + b'\\x00'*800)\n")
    exe = tmp_path / "stub.sh"
    exe.write_text("#!/bin/sh\nexec %s %s \"$@\"\n" % (sys.executable, script))
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setattr(ft, "BINARY", str(exe))
    monkeypatch.chdir(tmp_path)
    return tmp_path


def parse(raw):
    o = {}
    off = 0

    def take(fmt):
        nonlocal off
        v = struct.unpack_from(fmt, raw, off)
        off += struct.calcsize(fmt)
        return v[0] if len(v) == 1 else v
    o["n"], o["d"] = take("=ii")
    o["theta"], o["perplexity"] = take("=dd")
    if o["perplexity"] == 0:
        k = take("=i")
        o["plist"] = list(struct.unpack_from("=%dd" % k, raw, off))
        off += 8 * k
    names = [("no_dims", "i"), ("max_iter", "i"), ("stop", "i"), ("mom_switch", "i"), ("mom", "d"), ("fmom", "d"),
             ("lr", "d"), ("msn", "d"), ("K", "i"), ("sigma", "d"), ("nbody", "i"), ("knn", "i"), ("exag", "d"),
             ("nomom", "i"), ("n_trees", "i"), ("search_k", "i"), ("start_late", "i"), ("late", "d"), ("nterms", "i"),
             ("ipi", "d"), ("min_int", "i")]
    for nm, f in names:
        o[nm] = take("=" + f)
    o["X"] = np.frombuffer(raw, np.float64, o["n"] * o["d"], off)
    off += 8 * o["n"] * o["d"]
    o["seed"], = struct.unpack_from("=i", raw, off)
    o["df"], = struct.unpack_from("=d", raw, off + 4)
    o["load"], = struct.unpack_from("=i", raw, off + 12)
    rest = raw[off + 16:]
    o["init"] = np.frombuffer(rest, np.float64) if rest else None
    return o


def test_defaults_and_auto_options(stub_binary):
    X = np.random.default_rng(0).standard_normal((50, 4))
    Y, loss = ft.fast_tsne(X, initialization="random", max_iter=100, return_loss=True)
    o = parse(open(stub_binary / "captured.dat", "rb").read())
    assert (o["n"], o["d"], o["no_dims"], o["max_iter"], o["stop"]) == (50, 4, 2, 100, 250)
    assert o["lr"] == 200.0 and o["start_late"] == -1 and o["knn"] == 1 and o["nbody"] == 2
    assert o["search_k"] == 3 * 30 * 50 and o["init"] is None and o["load"] == 0
    assert np.array_equal(o["X"], X.ravel())
    assert Y.shape == (50, 2) and np.isnan(loss[0]) and not np.isnan(loss[49])


def test_perplexity_list_sigma_and_late_exaggeration(stub_binary):
    X = np.random.default_rng(1).standard_normal((30, 3))
    ft.fast_tsne(X, perplexity_list=[3, 10], late_exag_coeff=4, initialization="random", max_iter=100,
                 knn_algo="vp-tree", load_affinities="save", max_step_norm="none")
    o = parse(open(stub_binary / "captured.dat", "rb").read())
    assert o["perplexity"] == 0 and o["plist"] == [3.0, 10.0]
    assert o["start_late"] == 250 and o["late"] == 4.0 and o["knn"] == 2 and o["load"] == 2 and o["msn"] == -1
    ft.fast_tsne(X, sigma=2.0, K=10, initialization="random", max_iter=100)
    o = parse(open(stub_binary / "captured.dat", "rb").read())
    assert o["perplexity"] == -1 and o["K"] == 10 and o["sigma"] == 2.0 and o["search_k"] == 500


def test_pca_initialisation_scale(stub_binary, monkeypatch):
    pytest.importorskip("sklearn")
    monkeypatch.setenv("FITSNE_PCA", "sklearn")  # the GPU PCA is tested in test_pca_gpu.py
    X = np.random.default_rng(2).standard_normal((60, 5)) * [5, 3, 1, 1, 1]
    ft.fast_tsne(X, max_iter=100)
    o = parse(open(stub_binary / "captured.dat", "rb").read())
    init = o["init"].reshape(60, 2)
    assert abs(np.std(init[:, 0]) - 1e-4) < 1e-10


def test_bad_option_strings_raise(monkeypatch):
    pytest.importorskip("sklearn")
    monkeypatch.setenv("FITSNE_PCA", "sklearn")
    X = np.zeros((10, 2))
    with pytest.raises(ValueError):
        ft.fast_tsne(X, nbody_algo="exact")
    with pytest.raises(ValueError):
        ft.fast_tsne(X, knn_algo="hnsw", initialization="random")
