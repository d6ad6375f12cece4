"""GPU gradient parity against the reference (golden fixtures made by the reference).

Tolerances: the FP32 form must stay within relative L2 1e-4 of the reference's FP64
gradient on identical Y and P (the stated target) and Z within 1e-5; the FP64 form must
agree to rounding (1e-9)."""
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

CASES = [("g2_df1", "Y2", 1.0), ("g2_df05", "Y2", 0.5), ("g2_df3", "Y2", 3.0), ("g1_df1", "Y1", 1.0),
         ("g1_df05", "Y1", 0.5), ("g0_df1", "Y0", 1.0)]
TOL = {32: (1e-4, 1e-5), 64: (1e-9, 1e-10)}


def _P(golden):
    val = golden["sym_val"]
    return golden["sym_row"], golden["sym_col"], val / val.sum()


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("name,yk,df", CASES)
def test_fft_gradient_matches_reference(gpu_lib, golden, bits, name, yk, df):
    row, col, val = _P(golden)
    gpu_lib.set_precision(bits)
    try:
        dC, z = gpu_lib.fft_gradient(row, col, val, golden[yk], 3, 1.0, 50, df)
    finally:
        gpu_lib.set_precision(32)
    gtol, ztol = TOL[bits]
    assert abs(z - float(golden[name + "_Z"])) / abs(float(golden[name + "_Z"])) < ztol
    assert rel_l2(dC, golden[name + "_dC"]) < gtol


@pytest.mark.parametrize("bits", [32, 64])
def test_fft_gradient_nterms5(gpu_lib, golden, bits):
    row, col, val = _P(golden)
    gpu_lib.set_precision(bits)
    try:
        dC, z = gpu_lib.fft_gradient(row, col, val, golden["Y2"], 5, 2.0, 30, 1.0)
    finally:
        gpu_lib.set_precision(32)
    gtol, ztol = TOL[bits]
    assert abs(z - float(golden["g2_nt5_Z"])) / float(golden["g2_nt5_Z"]) < ztol
    assert rel_l2(dC, golden["g2_nt5_dC"]) < gtol


@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("name,yk,df", CASES)
def test_kl_matches_reference(gpu_lib, golden, bits, name, yk, df):
    row, col, val = _P(golden)
    gpu_lib.set_precision(bits)
    try:
        c = gpu_lib.evaluate_error_fft(row, col, val, golden[yk], df, float(golden[name + "_Z"]))
    finally:
        gpu_lib.set_precision(32)
    ref = float(golden[name + "_KL"])
    assert abs(c - ref) / abs(ref) < (1e-5 if bits == 32 else 1e-10)


def _box_geometry(Y, min_int=50, ipi=1.0):
    """Box count and width of the 2-D grid (the reference's rule, nbodyfft.cpp / tsne.cpp:1039-1060)."""
    allowed = [25, 36, 50, 55, 60, 65, 70, 75, 80, 85, 90, 96, 100, 110, 120, 130, 140, 150, 175, 200]
    v = Y.ravel()
    mx, mn = v.max(), v[1:].min()
    nb = int(max(min_int, (mx - mn) / ipi))
    if nb < 200:
        nb = next(a for a in allowed if a >= nb)
    return mn, (mx - mn) / nb


def test_fp32_box_index_agrees_with_fp64_on_a_box_edge(gpu_lib, golden):
    """A point whose float box quotient rounds across an edge must still be interpolated
    from the box the FP64 form (and the reference) picks: from the other box its
    repulsion differs by the interpolation error, far above FP32 rounding."""
    row, col, val = _P(golden)
    Y = golden["Y2"].copy()
    mn, bw = _box_geometry(Y)
    i = int(np.argsort(np.abs(Y[:, 0] - np.median(Y[:, 0])))[0])  # an interior point
    k = int((Y[i, 0] - mn) / bw)
    found = False
    for rel in np.geomspace(1e-9, 1e-6, 400):
        x = mn + bw * (k + 1) * (1.0 - rel)
        hi = np.float32(x)
        x = float(hi) + float(np.float32(x - float(hi)))  # representable as a float pair
        q32 = np.float32(np.float32(x - mn) * np.float32(1.0 / bw))
        if int((x - mn) / bw) == k and int(q32) == k + 1:
            found = True
            break
    assert found
    Y[i, 0] = x
    assert _box_geometry(Y) == (mn, bw)
    out = {}
    for bits in (32, 64):
        gpu_lib.set_precision(bits)
        try:
            out[bits] = gpu_lib.fft_gradient(row, col, val, Y, 3, 1.0, 50, 1.0)
        finally:
            gpu_lib.set_precision(32)
    g32, g64 = out[32][0], out[64][0]
    assert np.linalg.norm(g32[i] - g64[i]) / np.linalg.norm(g64[i]) < 1e-4
    assert rel_l2(g32, g64) < 1e-5


# attraction launch shapes: 11 over the full CSR (kNumAttrShapes), then the tiled form over the
# half-stored symmetric P (kAttrTilesShape = 11; FP32 form, the FP64 form takes shape 10 for it)
N_SHAPES = 12


@pytest.mark.parametrize("shape", range(N_SHAPES))
@pytest.mark.parametrize("bits", [32, 64])
@pytest.mark.parametrize("name,yk", [("g2_df1", "Y2"), ("g1_df1", "Y1")])
def test_every_attraction_shape_gives_the_reference_gradient(gpu_lib, golden, monkeypatch, bits, shape, name, yk):
    """Each launch shape of the attraction pass (the autotuner's candidates, fixed through
    FITSNE_ATTR_SHAPE) computes the reference's gradient within the FP32 / FP64 tolerances."""
    monkeypatch.setenv("FITSNE_ATTR_SHAPE", str(shape))
    row, col, val = _P(golden)
    gpu_lib.set_precision(bits)
    try:
        dC, z = gpu_lib.fft_gradient(row, col, val, golden[yk], 3, 1.0, 50, 1.0)
    finally:
        gpu_lib.set_precision(32)
    assert rel_l2(dC, golden[name + "_dC"]) < TOL[bits][0]


@pytest.mark.parametrize("bits", [32, 64])
def test_every_attraction_shape_takes_the_same_steps(gpu_lib, monkeypatch, bits):
    """The fused update (gains, momentum, clipping, double-float Y) is the same code in every
    shape: 3 iterations from the same start agree with shape 0's up to the summation order of
    the attraction (FP32 1e-4, FP64 1e-9 relative).  Longer runs drift apart in FP32: the
    gains rule jumps (+0.2 or x0.8) on the sign of a gradient component, and a component near
    zero flips with the last bits of the sum (20 iterations: 6e-4 between shapes 0 and 1)."""
    rng = np.random.default_rng(4)
    c = rng.standard_normal((6, 10)) * 4.0
    X = c[rng.integers(0, 6, 3000)] + rng.standard_normal((3000, 10))
    Y0 = rng.standard_normal((3000, 2)) * 1e-4
    gpu_lib.set_precision(bits)
    try:
        out = []
        for shape in range(N_SHAPES):
            monkeypatch.setenv("FITSNE_ATTR_SHAPE", str(shape))
            Y, _ = gpu_lib.run(X, Y0=Y0, perplexity=30.0, max_iter=3, learning_rate=250.0)
            out.append(Y)
    finally:
        gpu_lib.set_precision(32)
    for shape in range(1, N_SHAPES):
        assert rel_l2(out[shape], out[0]) < (1e-4 if bits == 32 else 1e-9), shape


@pytest.mark.parametrize("threads", [64, 128, 512])
@pytest.mark.parametrize("bits", [32, 64])
def test_every_fft_block_size_gives_the_reference_gradient(gpu_lib, golden, monkeypatch, bits, threads):
    """The 2-D FFT passes accept any block size the autotuner may pick (FITSNE_FFT_THREADS
    fixes it): the same gradient within the FP32 / FP64 tolerances, on the default grid and on
    the finer nterms = 5 fixture."""
    monkeypatch.setenv("FITSNE_FFT_THREADS", str(threads))
    row, col, val = _P(golden)
    gpu_lib.set_precision(bits)
    try:
        dC, z = gpu_lib.fft_gradient(row, col, val, golden["Y2"], 3, 1.0, 50, 1.0)
        dC5, z5 = gpu_lib.fft_gradient(row, col, val, golden["Y2"], 5, 2.0, 30, 1.0)
    finally:
        gpu_lib.set_precision(32)
    assert rel_l2(dC, golden["g2_df1_dC"]) < TOL[bits][0]
    assert abs(z - float(golden["g2_df1_Z"])) < TOL[bits][1] * float(golden["g2_df1_Z"])
    assert rel_l2(dC5, golden["g2_nt5_dC"]) < TOL[bits][0]


def test_tiled_attraction_runs_for_a_symmetric_P(gpu_lib, golden, monkeypatch):
    """With a symmetric P the FP32 form's tiled shape runs two kernels (attraction into the
    accumulator, then the update): one launch per iteration more than the full-CSR shapes,
    and the same steps within the FP32 tolerance."""
    row, col, val = _P(golden)
    launches, ys = {}, {}
    for shape in (10, 11):
        monkeypatch.setenv("FITSNE_ATTR_SHAPE", str(shape))
        s = gpu_lib.Session(row, col, val, golden["Y2"], precision=32)
        try:
            s.set_graphs(False)
            s.run(300, 310, learning_rate=200.0)
            launches[shape] = s.stage_times()[9]
            ys[shape] = s.get_y()
            assert s.launch_shapes()["attr_form"] == (2 if shape == 11 else 0)
        finally:
            s.close()
    assert launches[11] == launches[10] + 10, launches
    assert rel_l2(ys[11], ys[10]) < 1e-4


def test_tiled_attraction_falls_back_on_an_asymmetric_P(gpu_lib, golden, monkeypatch):
    """The calibrated kNN matrix before symmetrisation is not symmetric: the tiled shape must
    detect it and take the full CSR (the reference's attraction works for any P)."""
    monkeypatch.setenv("FITSNE_ATTR_SHAPE", "11")
    row, col, val = golden["knn_row"], golden["knn_col"], golden["knn_val"] / golden["knn_val"].sum()
    d32, _ = gpu_lib.fft_gradient(row, col, val, golden["Y2"], 3, 1.0, 50, 1.0)
    gpu_lib.set_precision(64)
    try:
        d64, _ = gpu_lib.fft_gradient(row, col, val, golden["Y2"], 3, 1.0, 50, 1.0)
    finally:
        gpu_lib.set_precision(32)
    assert rel_l2(d32, d64) < 1e-4


def test_tiled_attraction_across_many_tiles_and_renumberings(gpu_lib, monkeypatch):
    """The tiled attraction on 30,000 points: 8 blocks of 4,096, so up to 36 tiles, and a last
    block of 1,328 points.  A session runs 310 iterations with it, through the locality
    renumberings at 50, 150 and 300 (the tiles are rebuilt after each); its gradient at the end
    matches the restated reference gradient (FP64) on the same Y and P, and the full-CSR
    shape's."""
    import oracle
    oracle.build_restated()
    orc = oracle.Restated()
    rng = np.random.default_rng(30)
    c = rng.standard_normal((12, 20)) * 4.0
    X = c[rng.integers(0, 12, 30000)] + rng.standard_normal((30000, 20))
    X = X - np.cumsum(X, axis=0)[-1] / len(X)
    X /= np.abs(X).max()
    row, col, val = gpu_lib.gaussian_perplexity(X, 30.0, 90)
    row, col, val = gpu_lib.symmetrize(row, col, val, len(X))
    val = val / np.cumsum(val)[-1]
    Y0 = rng.standard_normal((len(X), 2)) * 1e-4
    monkeypatch.setenv("FITSNE_ATTR_SHAPE", "11")
    s = gpu_lib.Session(row, col, val, Y0, precision=32)
    try:
        s.run(0, 310, learning_rate=len(X) / 12.0)
        assert s.launch_shapes()["attr_form"] == 2
        Y = s.get_y()
        d11, z11 = s.gradient()
    finally:
        s.close()
    dref, zref = orc.fft_gradient(row, col, val, Y, 3, 1.0, 50, os.cpu_count() or 4, 1.0)
    assert rel_l2(d11, dref) < 1e-4
    assert abs(z11 - zref) < 1e-5 * zref
    monkeypatch.setenv("FITSNE_ATTR_SHAPE", "10")
    d10, _ = gpu_lib.fft_gradient(row, col, val, Y, 3, 1.0, 50, 1.0)
    assert rel_l2(d11, d10) < 1e-4
