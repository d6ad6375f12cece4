"""fitsne_fft_gradient_noalloc: the gradient entry point for callers that cannot allocate
device memory (a framework that owns the device memory through its own pool, or a loop
where an allocation is not allowed).  The caller passes device buffers; the library takes
its temporaries from one fixed device array.  Its result must match the allocating entry
point, fitsne_fft_gradient, within the tolerance of the gradient tests (relative L2 1e-4,
Z 1e-5), on two calls in a row (the array keeps the previous call's contents).

This file is collected last on purpose (test_zz_*): if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dtype=dtype, device="cuda")


def _noalloc(lib, row, col, val, Y, df, nterms=3, ipi=1.0, min_int=50):
    N, D = Y.shape
    d_row = _dev(row.astype(np.int32), torch.int32)
    d_col = _dev(col.astype(np.int32), torch.int32)
    d_val = _dev(val.astype(np.float32), torch.float32)
    d_Y = _dev(Y, torch.float64)
    d_dC = torch.zeros((N, D), dtype=torch.float64, device="cuda")
    z = ctypes.c_double(0.0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.fitsne_fft_gradient_noalloc(d_row.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), d_Y.data_ptr(), N, D,
                                         d_dC.data_ptr(), nterms, ipi, min_int, df, ctypes.byref(z), stream)
    torch.cuda.synchronize()
    return rc, d_dC.cpu().numpy(), z.value


@pytest.mark.parametrize("yk,df", [("Y2", 1.0), ("Y2", 0.5), ("Y1", 1.0), ("Y1", 0.5)])
def test_noalloc_gradient_matches_allocating_entry_point(gpu_lib, golden, yk, df):
    lib = gpu_lib.lib()
    row, col = golden["sym_row"], golden["sym_col"]
    val = golden["sym_val"] / golden["sym_val"].sum()
    Y = golden[yk]
    gpu_lib.set_precision(32)
    ref, zref = gpu_lib.fft_gradient(row, col, val, Y, 3, 1.0, 50, df)
    for _ in range(2):  # two calls in a row on the shared array
        rc, dC, z = _noalloc(lib, row, col, val, Y, df)
        assert rc == 0, lib.fitsne_last_error()
        assert rel_l2(dC, ref) < 1e-4
        assert abs(z - zref) <= 1e-5 * abs(zref)


@pytest.mark.parametrize("nterms", [5, 8])
def test_noalloc_gradient_at_more_interpolation_points(gpu_lib, golden, nterms):
    """The grid buffers are carved from the actual grid, so a small embedding works at any
    n_interpolation_points; nterms = 5 is also checked against the reference's gradient."""
    lib = gpu_lib.lib()
    row, col = golden["sym_row"], golden["sym_col"]
    val = golden["sym_val"] / golden["sym_val"].sum()
    Y = golden["Y2"]
    # nterms = 5 on the reference fixture's grid parameters (intervals_per_integer 2,
    # min_num_intervals 30); nterms = 8 on the defaults
    ipi, min_int = (2.0, 30) if nterms == 5 else (1.0, 50)
    gpu_lib.set_precision(32)
    ref, zref = gpu_lib.fft_gradient(row, col, val, Y, nterms, ipi, min_int, 1.0)
    for _ in range(2):
        rc, dC, z = _noalloc(lib, row, col, val, Y, 1.0, nterms=nterms, ipi=ipi, min_int=min_int)
        assert rc == 0, lib.fitsne_last_error()
        assert rel_l2(dC, ref) < 1e-4
        assert abs(z - zref) <= 1e-5 * abs(zref)
        if nterms == 5:
            assert rel_l2(dC, golden["g2_nt5_dC"]) < 1e-4
            assert abs(z - float(golden["g2_nt5_Z"])) <= 1e-5 * float(golden["g2_nt5_Z"])


def test_noalloc_rejects_inputs_beyond_its_limits(gpu_lib, golden):
    lib = gpu_lib.lib()
    row, col = golden["sym_row"], golden["sym_col"]
    val = golden["sym_val"] / golden["sym_val"].sum()
    # a grid too large for the fixed array: 160 boxes per dimension x 8 nodes
    rc, _, _ = _noalloc(lib, row, col, val, golden["Y2"], 1.0, nterms=8, min_int=160)
    assert rc == -13 and b"scratch" in lib.fitsne_last_error()
    # too many points: real (small) device buffers, so that no check order can hand a
    # kernel an invalid address; the N check rejects the call before any device work
    d_row = torch.zeros(16, dtype=torch.int32, device="cuda")
    d_col = torch.zeros(16, dtype=torch.int32, device="cuda")
    d_val = torch.zeros(16, dtype=torch.float32, device="cuda")
    d_Y = torch.zeros(16, dtype=torch.float64, device="cuda")
    d_dC = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = lib.fitsne_fft_gradient_noalloc(d_row.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), d_Y.data_ptr(),
                                         300000, 2, d_dC.data_ptr(), 3, 1.0, 50, 1.0, None, None)
    assert rc == -3 and b"exceeds" in lib.fitsne_last_error()
    # null buffers are rejected as argument errors
    rc = lib.fitsne_fft_gradient_noalloc(None, None, None, None, 100, 2, None, 3, 1.0, 50, 1.0, None, None)
    assert rc == -3
