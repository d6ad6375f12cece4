"""The C ABI: the library builds, loads and exports every symbol the header declares;
host-only entry points (file formats, settings, errors) work without a GPU."""
import ctypes
import os
import re
import struct

import numpy as np
import pytest

import fitsne
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fitsne_gb300.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fitsne_[a-z0-9_]+)\s*\(", txt)))


def test_library_exists_and_loads():
    assert os.path.exists(fitsne.LIB_PATH)
    fitsne.lib()


def test_every_header_symbol_is_exported():
    names = header_functions()
    assert len(names) >= 20
    lib = fitsne.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(names) == sorted(fitsne.exported_symbols())


def test_version_and_precision_switch():
    assert fitsne.lib().fitsne_version() == b"1.2.1"
    fitsne.set_precision(64)
    assert fitsne.get_precision() == 64
    fitsne.set_precision(32)
    assert fitsne.get_precision() == 32


def _write_data(path, n=5, d=3, perplexity=2.0, plist=None, with_init=True, trailer=True):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((n, d))
    Y0 = rng.standard_normal((n, 2))
    with open(path, "wb") as f:
        f.write(struct.pack("=iidd", n, d, 0.5, perplexity))
        if perplexity == 0:
            f.write(struct.pack("=i", len(plist)))
            f.write(np.array(plist, float).tobytes())
        f.write(struct.pack("=iiii", 2, 100, 25, 25))
        f.write(struct.pack("=dddd", 0.5, 0.8, 200.0, 5.0))
        f.write(struct.pack("=idii", -1, -1.0, 2, 2))
        f.write(struct.pack("=diiii", 12.0, 0, 50, 150, -1))
        f.write(struct.pack("=did", -1.0, 3, 1.0))
        f.write(struct.pack("=i", 50))
        f.write(X.tobytes())
        if trailer:
            f.write(struct.pack("=idi", 42, 0.5, 2))
            if with_init:
                f.write(Y0.tobytes())
    return X, Y0


def _load(path):
    lib = fitsne.lib()
    out = {k: ctypes.c_int() for k in ("n", "d", "no_dims", "rand_seed", "max_iter", "stop", "mom_switch", "K",
                                       "nbody", "knn", "nomom", "n_trees", "search_k", "start_late", "nterms",
                                       "min_int", "skip", "load_aff", "plen")}
    dbl = {k: ctypes.c_double() for k in ("theta", "perp", "mom", "fmom", "lr", "sigma", "exag", "late", "ipi", "df",
                                          "msn")}
    data = ctypes.POINTER(ctypes.c_double)()
    Y = ctypes.POINTER(ctypes.c_double)()
    plist = ctypes.POINTER(ctypes.c_double)()
    b = ctypes.byref
    rc = lib.fitsne_load_data(path.encode(), b(data), b(Y), b(out["n"]), b(out["d"]), b(out["no_dims"]),
                              b(dbl["theta"]), b(dbl["perp"]), b(out["rand_seed"]), b(out["max_iter"]), b(out["stop"]),
                              b(out["mom_switch"]), b(dbl["mom"]), b(dbl["fmom"]), b(dbl["lr"]), b(out["K"]),
                              b(dbl["sigma"]), b(out["nbody"]), b(out["knn"]), b(dbl["exag"]), b(out["nomom"]),
                              b(out["n_trees"]), b(out["search_k"]), b(out["start_late"]), b(dbl["late"]),
                              b(out["nterms"]), b(dbl["ipi"]), b(out["min_int"]), b(out["skip"]), b(out["load_aff"]),
                              b(out["plen"]), b(plist), b(dbl["df"]), b(dbl["msn"]))
    return rc, out, dbl, data, Y, plist


def test_load_data_reads_every_field(tmp_path):
    p = str(tmp_path / "data.dat")
    X, Y0 = _write_data(p)
    rc, o, d, data, Y, _ = _load(p)
    assert rc == 0
    assert (o["n"].value, o["d"].value, o["no_dims"].value, o["max_iter"].value) == (5, 3, 2, 100)
    assert (o["rand_seed"].value, o["load_aff"].value, o["skip"].value, o["plen"].value) == (42, 2, 1, 0)
    assert (d["df"].value, d["lr"].value, d["msn"].value, o["n_trees"].value, o["search_k"].value) == (0.5, 200.0, 5.0,
                                                                                                          50, 150)
    assert np.array_equal(np.ctypeslib.as_array(data, (5 * 3,)).reshape(5, 3), X)
    assert np.array_equal(np.ctypeslib.as_array(Y, (10,)).reshape(5, 2), Y0)


def test_load_data_perplexity_list_and_missing_trailer(tmp_path):
    p = str(tmp_path / "d.dat")
    _write_data(p, perplexity=0.0, plist=[3.0, 30.0], trailer=False)
    rc, o, d, _, _, plist = _load(p)
    assert rc == 0 and o["plen"].value == 2
    assert list(np.ctypeslib.as_array(plist, (2,))) == [3.0, 30.0]
    assert o["skip"].value == 0 and o["rand_seed"].value == 0 and d["df"].value == 1.0


def test_load_data_missing_file_is_an_io_error(tmp_path):
    rc = _load(str(tmp_path / "nope.dat"))[0]
    assert rc == -2


def test_save_data_layout(tmp_path):
    p = str(tmp_path / "r.dat")
    Y = np.arange(8, dtype=float).reshape(4, 2)
    costs = np.arange(3, dtype=float)
    dp = ctypes.POINTER(ctypes.c_double)
    assert fitsne.lib().fitsne_save_data(p.encode(), Y.ctypes.data_as(dp), costs.ctypes.data_as(dp), 4, 2, 3) == 0
    raw = open(p, "rb").read()
    assert struct.unpack("=ii", raw[:8]) == (4, 2)
    assert np.array_equal(np.frombuffer(raw[8:72]), Y.ravel())
    assert struct.unpack("=i", raw[72:76]) == (3,) and np.array_equal(np.frombuffer(raw[76:]), costs)


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_compute_without_gpu_fails_loudly():
    with pytest.raises(fitsne.FitsneError):
        fitsne.fft_gradient(np.array([0, 1, 2], np.uint32), np.array([1, 0], np.uint32), np.array([.5, .5]),
                            np.zeros((2, 2)))


def test_argument_errors_are_reported_before_any_device_work():
    lib = fitsne.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    X = np.zeros((4, 2))
    Y = np.zeros((4, 2))
    c = np.zeros(10)
    # perplexity too large for N (the reference exits with status 1 here)
    rc = lib.fitsne_run(X.ctypes.data_as(dp), 4, 2, Y.ctypes.data_as(dp), 2, 30.0, 0.5, 1, 1, 10, 2, 2, .5, .8, 200.0,
                        -1, -1.0, 2, 2, 12.0, c.ctypes.data_as(dp), 0, -1, -1.0, 50, -1, 3, 1.0, 50, 0, 0, 0, None, 1.0,
                        5.0)
    assert rc == -3 and b"Perplexity" in lib.fitsne_last_error()
    # Barnes-Hut is outside this build
    rc = lib.fitsne_run(X.ctypes.data_as(dp), 4, 2, Y.ctypes.data_as(dp), 2, 1.0, 0.5, 1, 1, 10, 2, 2, .5, .8, 200.0,
                        -1, -1.0, 1, 2, 12.0, c.ctypes.data_as(dp), 0, -1, -1.0, 50, -1, 3, 1.0, 50, 0, 0, 0, None, 1.0,
                        5.0)
    assert rc == -4
