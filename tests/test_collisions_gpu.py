"""Inner-boundary lists that name a cell twice (collisions) or nothing
(empty), against the oracle, bitwise.  The reference applies its lists in turn (srf, mid,
zero), each entry in order, so a cell named twice ends with its last
entry's values and BandE's resistive term adds once per entry.  The
lists its own set-up builds never collide; these are the lists a caller
may pass: a repeat inside each list and a cell in two lists."""
import numpy as np
import pytest

import test_routines_gpu as R
from _support import Inputs, assert_same, run_both

pytestmark = pytest.mark.gpu


def colliding(lists):
    L = {k: v.copy() for k, v in lists.items()}
    L["ijsrf"][5] = L["ijsrf"][4]     # srf: the second entry reads the first's result (max with rho)
    L["ijmid"][1] = L["ijmid"][0]     # mid: repeated, other parameters
    L["ijzero"][0] = L["ijsrf"][3]    # a srf cell in the zero list too
    L["ijzero"][2] = L["ijzero"][1]
    return L


def test_bndry_inner_colliding_lists():
    I = Inputs("tiny2")
    p = I.p
    L = colliding(I.lists)
    args = [list(I.wrk), L["parm_srf"], L["parm_mid"], L["parm_zero"], L["ijsrf"], L["numsrf"], L["ijmid"],
            L["nummid"], L["ijzero"], L["numzero"], L["ijsrf"].shape[0], L["ijmid"].shape[0], L["ijzero"].shape[0],
            p]
    oa, ga = run_both("bndry_inner", args)
    for q in range(34):
        assert_same(ga[0][q], oa[0][q], f"bndry_inner field {q}")


def test_bande_colliding_lists():
    I = Inputs("tiny2")
    p = I.p
    L = colliding(I.lists)
    box = 1
    ef = I.scratch(1.0, 3)
    bs = [(I.b0[q, box - 1] + I.cur[31 + q, box - 1]).astype(np.float32) for q in range(3)]
    cur = I.scratch(0.1, 3)
    ev = I.scratch(0.1, 3)
    btot = I.scratch(1.0)[0]
    args = (ef + bs + cur + ev + [btot, I.cur[30], I.cur[0], I.cur[10], I.cur[20], I.resistive, p.resist, p.reynolds]
            + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, L["ijmid"], L["nummid"], L["ijzero"], p.mbndry,
                             L["numzero"], L["ijmid"].shape[0], L["ijzero"].shape[0]]
            + [float(p.xspac[box - 1])] * 3)
    oa, ga = run_both("bande", args)
    for k in range(3):
        assert_same(ga[k], oa[k], f"BandE efld{k}")


@pytest.mark.parametrize("graph", [False, True])
def test_engine_steps_with_colliding_lists(graph):
    """Three nested boxes, two main steps, the engine against the oracle's
    main loop with the colliding lists."""
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    st = make_config("tiny3")
    st.lists = colliding(st.lists)
    om = OracleModel(st, omp=True)
    om.init_steps()
    for _ in range(2):
        assert om.main_step() == 0
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        m.run(2, graph=graph)
        g = m.state()
        m.close()
    for q in range(34):
        assert_same(g[q], om.cur[q], f"field {q}")


@pytest.mark.parametrize("empty", ["srf", "mid", "zero", "all"])
def test_bndry_inner_and_bande_empty_lists(empty):
    """Lists with no entries (count 0) leave the fields to the other lists."""
    I = Inputs("tiny2")
    p = I.p
    L = {k: v.copy() for k, v in I.lists.items()}
    for name in (("srf", "mid", "zero") if empty == "all" else (empty,)):
        L["num" + name][:] = 0
    args = [list(I.wrk), L["parm_srf"], L["parm_mid"], L["parm_zero"], L["ijsrf"], L["numsrf"], L["ijmid"],
            L["nummid"], L["ijzero"], L["numzero"], L["ijsrf"].shape[0], L["ijmid"].shape[0], L["ijzero"].shape[0],
            p]
    oa, ga = run_both("bndry_inner", args)
    for q in range(34):
        assert_same(ga[0][q], oa[0][q], f"bndry_inner field {q}")
    box = 1
    ef = I.scratch(1.0, 3)
    bs = [(I.b0[q, box - 1] + I.cur[31 + q, box - 1]).astype(np.float32) for q in range(3)]
    cur = I.scratch(0.1, 3)
    ev = I.scratch(0.1, 3)
    args = (ef + bs + cur + ev + [I.scratch(1.0)[0], I.cur[30], I.cur[0], I.cur[10], I.cur[20], I.resistive,
                                  p.resist, p.reynolds]
            + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, L["ijmid"], L["nummid"], L["ijzero"], p.mbndry,
                             L["numzero"], L["ijmid"].shape[0], L["ijzero"].shape[0]]
            + [float(p.xspac[box - 1])] * 3)
    oa, ga = run_both("bande", args)
    for k in range(3):
        assert_same(ga[k], oa[k], f"BandE efld{k}")
