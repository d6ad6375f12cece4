"""Device-resident iterations (fitsne_session_*) against the restated update loop."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nd,df", [(2, 1.0), (1, 0.5)])
def test_session_iterations_match_restated_loop(gpu_lib, golden, nd, df):
    orc = oracle.Restated(oracle.build_restated())
    row, col = golden["sym_row"], golden["sym_col"]
    val = golden["sym_val"] / golden["sym_val"].sum()
    Y0 = golden["Y2"][:, :nd] * 0.05
    s = gpu_lib.Session(row, col, val, Y0, df=df, precision=64)
    s.run(0, 30, max_iter=30, stop_lying_iter=10, mom_switch_iter=10, learning_rate=200.0, early_exag_coeff=12.0)
    Yg = s.get_y()
    s.close()
    Y = Y0.copy()
    uY = np.zeros_like(Y)
    gains = np.ones_like(Y)
    exag, mom = 12.0, 0.5
    for it in range(30):
        orc.gradient_step(row, col, val, Y, uY, gains, df=df, exag=exag, momentum=mom, learning_rate=200.0)
        if it == 10:
            exag, mom = 1.0, 0.8
    assert rel_l2(Yg, Y) < 1e-9


def test_session_fp32_tracks_fp64(gpu_lib, golden):
    row, col = golden["sym_row"], golden["sym_col"]
    val = golden["sym_val"] / golden["sym_val"].sum()
    out = []
    for bits in (32, 64):
        s = gpu_lib.Session(row, col, val, golden["Y0"], precision=bits)
        s.run(0, 5, max_iter=60, stop_lying_iter=30, mom_switch_iter=30, learning_rate=200.0, early_exag_coeff=12.0)
        out.append(s.get_y())
        s.close()
    # a few steps only: the optimiser amplifies rounding differences chaotically
    assert rel_l2(out[0], out[1]) < 1e-4


def test_session_stage_timing(gpu_lib, golden):
    val = golden["sym_val"] / golden["sym_val"].sum()
    s = gpu_lib.Session(golden["sym_row"], golden["sym_col"], val, golden["Y2"])
    s.set_timing(True)
    s.run(300, 301)
    t = s.stage_times()
    s.close()
    assert t[5] > 0 and t[6] >= 25 and t[7] >= 2 * 3 * t[6]
