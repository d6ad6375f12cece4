"""Build recipe of the GB300 library and the drop-in ``fast_tsne`` binary.

Compiles every ``csrc/*.cu`` for sm_103a with nvcc (in parallel, one translation unit per
process), links ``libfitsne_gb300.so`` (CUDA runtime linked statically) next to this file
and the ``bin/fast_tsne`` executable against it.  Objects go to ``_build/``.  A unit is
rebuilt when it, or any header under ``csrc/`` or ``include/``, is newer than its object.

Usage: ``python fit-sne_gb300/build.py [--force]``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfitsne_gb300.so")
BIN_DIR = os.path.join(HERE, "bin")
BIN = os.path.join(BIN_DIR, "fast_tsne")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                  "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if force or _stale(obj, [src] + _headers()):
        cmd = [_nvcc()] + NVFLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stdout + r.stderr))
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the library and the binary; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN_DIR, exist_ok=True)
    lib_srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    lib_srcs = [s for s in lib_srcs if os.path.basename(s) != "main.cpp"]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(lib_srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), lib_srcs))
    if force or _stale(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stdout + r.stderr))
        if verbose:
            print("linked", LIB)
    main_src = os.path.join(CSRC, "main.cpp")
    if os.path.exists(main_src) and (force or _stale(BIN, [main_src, LIB])):
        cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), main_src, "-o", BIN,
               "-L" + HERE, "-lfitsne_gb300", "-Wl,-rpath,$ORIGIN/..", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("binary link failed:\n%s\n%s" % (" ".join(cmd), r.stdout + r.stderr))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
