"""The tensor-core kNN's per-query candidate heap (knn_heap.cuh), compiled for the host."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_candidate_heap_keeps_the_c_smallest(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "knn_heap_check"
    subprocess.run([cxx, "-O2", "-std=c++17", os.path.join(HERE, "knn_heap_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
