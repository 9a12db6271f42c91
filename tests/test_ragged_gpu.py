"""Drop-in routines on anisotropic boxes whose sizes leave ragged tiles in
every direction (nx, ny, nz all different; remainders 13, 5 and 1 against
the 32-wide tile rows, 5 and 9 against 8- and 16-row tiles, 17 and 5
interior planes), against the oracle, bitwise (div B: against the FP64
build, as its drop-in test states).  The boxes are the first
cells of each box of the three-box 49x49x25 grid (Inputs.crop); the first
and the last box of the array are used, so the per-box offsets are
exercised too."""
import ctypes

import numpy as np
import pytest

import test_routines_gpu as R
from _support import Inputs, assert_same, copy_args, run_both

pytestmark = pytest.mark.gpu

SHAPES = [(45, 29, 19), (33, 41, 7)]
CASES = [(s, box) for s in SHAPES for box in (1, 3)]


def ragged(shape, seed=7):
    return Inputs("mid3", seed=seed).crop(*shape)


@pytest.mark.parametrize("shape,box", CASES)
def test_push_ion_ragged(shape, box):
    I = ragged(shape)
    for s in ("q", "o"):
        args = R.push_ion_args(I, s, box)
        oa, ga = run_both("push_ion", args)
        for k in list(range(7)) + [21, 22, 23, 38, 39, 40]:
            assert_same(ga[k], oa[k], f"push_ion {s} arg {k}")


@pytest.mark.parametrize("shape,box", CASES)
def test_push_fields_and_currents_ragged(shape, box):
    I = ragged(shape)
    p = I.p
    ev, ef = I.scratch(0.1, 3), I.scratch(0.01, 3)
    rx = float(p.xspac[box - 1])
    args = [I.wrk[30], I.old[30], I.cur[30]] + ev + [p.gamma, p.gamma1] + I.dims(box) + [0.02, rx, rx, rx]
    oa, ga = run_both("push_elec", args)
    assert_same(ga[2], oa[2], "push_elec epres")
    args = [I.cur[31], I.cur[32], I.cur[33], I.old[31], I.old[32], I.old[33]] + ef + I.dims(box) + [0.02, rx, rx, rx]
    oa, ga = run_both("push_bfld", args)
    for k in range(3):
        assert_same(ga[k], oa[k], f"push_bfld b{k}")
    cur = I.scratch(1.0, 3)
    args = [I.cur[31], I.cur[32], I.cur[33]] + I.dims(box) + cur + [rx, rx, rx]
    oa, ga = run_both("calcur", args)
    for k in (8, 9, 10):
        assert_same(ga[k], oa[k], f"calcur {k}")
    out = I.scratch(1.0, 4)
    args = [I.cur[31], I.cur[32], I.cur[33], I.b0[0], I.b0[1], I.b0[2]] + I.dims(box) + [1e-5] + out
    oa, ga = run_both("total_b", args)
    for k in range(12, 16):
        assert_same(ga[k], oa[k], f"total_b {k}")


@pytest.mark.parametrize("shape,box", CASES)
def test_lapidus_ragged(shape, box):
    I = ragged(shape)
    v = I.scratch(0.2, 3)
    args = R.species(I.cur, "h") + R.species(I.wrk, "h") + v + I.dims(box) + [0.1, 0.1, 0.1, 0.03, 0]
    oa, ga = run_both("lap_plasma", args)
    for k in range(10, 20):
        assert_same(ga[k], oa[k], f"lap_plasma {k}")
    args = [I.cur[31], I.cur[32], I.cur[33], I.wrk[31], I.wrk[32], I.wrk[33]] + v + I.dims(box) + [0.1, 0.1, 0.1, 0.03]
    oa, ga = run_both("lap_bfld", args)
    for k in (3, 4, 5):
        assert_same(ga[k], oa[k], f"lap_bfld {k}")


@pytest.mark.parametrize("shape,box", CASES)
def test_flux_correction_ragged(shape, box):
    I = ragged(shape)
    p = I.p
    tmp = I.scratch(1.0, 3)
    for q in (0, 31):
        args = [I.cur[q], I.old[q], I.wrk[q]] + I.dims(box) + [0.05] + tmp
        oa, ga = run_both("fcsmooth", args)
        assert_same(ga[0], oa[0], f"fcsmooth field {q}")
    args = [list(I.cur), list(I.wrk), list(I.old)] + tmp + I.dims(box) + [p.difrho, p.diferg]
    oa, ga = run_both("flux_correct", args, oracle_drop=(3, 4, 5))
    for q in range(34):
        assert_same(ga[0][q], oa[0][q], f"flux_correct field {q}")


@pytest.mark.parametrize("shape,box", CASES)
def test_guards_ragged(shape, box):
    I = ragged(shape)
    R.guard_inputs(I, box)
    p = I.p
    f = I.cur
    args = ([f[0], f[4], f[5], f[6], f[7], f[8], f[9], p.rmassq, f[10], f[14], f[15], f[16], f[17], f[18], f[19],
             p.rmassh, f[20], f[24], f[25], f[26], f[27], f[28], f[29], p.rmasso, f[30]] + I.dims(box) + [p.o_conc])
    oa, ga = run_both("set_rho", args)
    for k in [0, 1, 2, 3, 4, 5, 6, 8, 9, 10, 11, 12, 13, 14, 16, 17, 18, 19, 20, 21, 22, 24]:
        assert_same(ga[k], oa[k], f"set_rho arg {k}")
    btot = np.zeros(I.box3, np.float32)
    vlim = p.vlim_factor * box
    args = (I.dims(box)[:4] + [box, p.rmassq, p.rmassh, p.rmasso, 0, p.smallbit, p.aniso_limit, vlim, p.qvlim,
                               p.hvlim, p.ovlim, p.qclim, p.hclim, p.oclim, p.cslim,
                               f[31], f[32], f[33], I.b0[0], I.b0[1], I.b0[2]]
            + [f[q] for q in range(30)] + [f[30], btot])
    from oracle import oracle
    from g3m3_gb300.api import Context
    oa = copy_args(args)
    oo = [ctypes.c_float() for _ in range(6)]
    oracle.call("set_speed_agrd", *oa, *[ctypes.addressof(x) for x in oo])
    ga = copy_args(args)
    go = [ctypes.c_float() for _ in range(6)]
    with Context() as ctx:
        ctx.call("set_speed_agrd", *ga, *[ctypes.addressof(x) for x in go])
        for a in ga:
            if isinstance(a, np.ndarray):
                ctx.sync_to_host(a)
    for k in range(25, 57):
        assert_same(ga[k], oa[k], f"set_speed_agrd arg {k}")
    for x, y, n in zip(go, oo, ("pxmax", "pymax", "pzmax", "csmax", "alfmax", "fastest")):
        assert x.value == y.value, (n, x.value, y.value)


@pytest.mark.parametrize("shape,box", CASES)
def test_divb_correct_ragged(shape, box):
    """The div B projection on the anisotropic boxes: the bar of
    test_routines_gpu.py::test_divb_correct (B at least as close to the
    FP64 solve as the reference's FP32 solve, residual, iteration count)."""
    R.check_divb(ragged(shape), box, 1e-4)


def _inside_coarser(I, box):
    """The box's cells interpolate from cells of box+1 that exist."""
    p = I.p
    for ax, n in (("x", p.nx), ("y", p.ny), ("z", p.nz)):
        lo_f, hi_f = getattr(p, f"grd_{ax}min")[box - 1], getattr(p, f"grd_{ax}max")[box - 1]
        lo_c, hi_c = getattr(p, f"grd_{ax}min")[box], getattr(p, f"grd_{ax}max")[box]
        dc = (hi_c - lo_c) / (n - 1)
        if not (lo_f >= lo_c and (hi_f - lo_c) / dc + 2 <= n):
            return False
    return True


@pytest.mark.parametrize("box", [1, 2])
def test_flanks_and_corer_ragged(box):
    """flanks, corer and flanks_synced between a 45x29x19 box and its
    coarser neighbour (cut from the same grid, so the finer box still lies
    inside the coarser one)."""
    I = ragged((45, 29, 19))
    assert _inside_coarser(I, box)
    p = I.p
    g = I.grid()
    t_old = (ctypes.c_double * p.n_grids)(*([0.0] * p.n_grids))
    t_new = (ctypes.c_double * p.n_grids)(*([0.2] * p.n_grids))
    work = np.zeros(I.box3, np.float32)
    for q in (0, 7, 33):
        args = [I.wrk[q], I.cur[q], I.old[q]] + I.dims(box) + [t_new, t_old, 0.07, work] + g
        oa, ga = run_both("flanks", args)
        assert_same(ga[0], oa[0], f"flanks box {box} field {q}")
        oa, ga = run_both("corer", [I.cur[q]] + I.dims(box) + g)
        assert_same(ga[0], oa[0], f"corer box {box} field {q}")
        oa, ga = run_both("flanks_synced", [I.cur[q]] + I.dims(box) + g)
        assert_same(ga[0], oa[0], f"flanks_synced box {box} field {q}")
