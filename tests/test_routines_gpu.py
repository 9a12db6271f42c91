"""Per-routine parity: every drop-in entry point of libg3m3_gpu.so against
the oracle's restatement of the same reference routine, on seeded inputs,
called with the reference's argument lists.  Bitwise unless noted."""
import ctypes

import numpy as np
import pytest

from _support import Inputs, assert_same, rel_l2, run_both

pytestmark = pytest.mark.gpu

SP = {"q": 0, "h": 10, "o": 20}


def species(arr, s):
    b = SP[s]
    return [arr[b + i] for i in range(10)]


def push_ion_args(I, s, box, delt=0.01):
    p = I.p
    b0 = I.b0[:, box - 1]
    bs = [(b0[q] + I.cur[31 + q, box - 1]).astype(np.float32) for q in range(3)]
    btot = np.maximum(np.sqrt(bs[0] ** 2 + bs[1] ** 2 + bs[2] ** 2), 1e-5).astype(np.float32)
    efld = I.scratch(0.01, 3)
    tv = I.scratch(0.1, 3)
    qv = I.scratch(1.0, 3)
    out, old, src = species(I.cur, s), species(I.old, s), species(I.wrk, s)
    mass = {"q": p.rmassq, "h": p.rmassh, "o": p.rmasso}[s]
    g = I.grid()
    o7 = [out[0], out[4], out[5], out[6], out[1], out[2], out[3]]
    d7 = [old[0], old[4], old[5], old[6], old[1], old[2], old[3]]
    s7 = [src[0], src[4], src[5], src[6], src[1], src[2], src[3]]
    return (o7 + d7 + s7 + out[7:10] + old[7:10] + src[7:10] + bs + [btot] + efld + [mass] + qv + tv
            + [p.gamma, p.gamma1] + I.dims(box) + [delt, p.grav, p.re_equiv, p.reynolds] + g + [0])


@pytest.mark.parametrize("cfg,box,s", [("tiny2", 1, "q"), ("tiny2", 2, "o"), ("small", 1, "h")])
def test_push_ion(cfg, box, s):
    I = Inputs(cfg)
    args = push_ion_args(I, s, box)
    oa, ga = run_both("push_ion", args)
    for k in list(range(7)) + [21, 22, 23, 38, 39, 40]:   # the 10 outputs and qv
        assert_same(ga[k], oa[k], f"push_ion arg {k}")


@pytest.mark.parametrize("box,rx", [(1, 1.0), (2, 2.0), (1, 0.7)])
def test_push_elec_bfld(box, rx):
    I = Inputs("tiny2")
    p = I.p
    ev = I.scratch(0.1, 3)
    ef = I.scratch(0.01, 3)
    args = [I.wrk[30], I.old[30], I.cur[30]] + ev + [p.gamma, p.gamma1] + I.dims(box) + [0.02, rx, rx, rx]
    oa, ga = run_both("push_elec", args)
    assert_same(ga[2], oa[2], "push_elec epres")
    args = [I.cur[31], I.cur[32], I.cur[33], I.old[31], I.old[32], I.old[33]] + ef + I.dims(box) + [0.02, rx, rx, rx]
    oa, ga = run_both("push_bfld", args)
    for k in range(3):
        assert_same(ga[k], oa[k], f"push_bfld b{k}")


@pytest.mark.parametrize("cfg,box", [("tiny2", 1), ("tiny2", 2), ("small", 1)])
def test_calcur_total_b(cfg, box):
    I = Inputs(cfg)
    rx = float(I.p.xspac[box - 1])
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


def test_fnd_evel_vtot():
    I = Inputs("tiny2")
    p = I.p
    box = 1
    sp = []
    for s in ("q", "h", "o"):
        f = species(I.cur, s)
        sp += [f[1], f[2], f[3], f[0]]
    cur = I.scratch(0.1, 3)
    out = I.scratch(1.0, 6)
    args = sp + cur + out + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, p.reynolds]
    oa, ga = run_both("fnd_evel", args)
    for k in range(15, 21):
        assert_same(ga[k], oa[k], f"fnd_evel {k}")
    out = I.scratch(1.0, 3)
    args = sp + out + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso]
    oa, ga = run_both("fnd_vtot", args)
    for k in range(12, 15):
        assert_same(ga[k], oa[k], f"fnd_vtot {k}")


@pytest.mark.parametrize("box", [1, 2])
def test_bande(box):
    I = Inputs("tiny2")
    p = I.p
    L = I.lists
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


def test_fnd_pres():
    I = Inputs("tiny2")
    f = species(I.cur, "h")
    out = [np.zeros_like(I.cur[0]) for _ in range(3)]
    v = I.scratch(0.1, 3)
    b = I.scratch(0.1, 3)
    args = [f[4], f[5], f[6], f[7], f[8], f[9]] + out + v + b + I.dims(2)
    oa, ga = run_both("fnd_pres", args)
    for k in (6, 7, 8):
        assert_same(ga[k][1], oa[k][1], f"fnd_pres {k}")


@pytest.mark.parametrize("box", [1, 2])
def test_lapidus(box):
    I = Inputs("tiny2")
    p = I.p
    v = I.scratch(0.2, 3)
    args = species(I.cur, "o") + species(I.wrk, "o") + v + I.dims(box) + [0.1, 0.1, 0.1, 0.03, 0]
    oa, ga = run_both("lap_plasma", args)
    for k in range(10, 20):
        assert_same(ga[k], oa[k], f"lap_plasma {k}")
    args = [I.cur[30], I.wrk[30]] + v + I.dims(box) + [0.1, 0.1, 0.1, 0.03]
    oa, ga = run_both("lap_elec", args)
    assert_same(ga[1], oa[1], "lap_elec")
    args = [I.cur[31], I.cur[32], I.cur[33], I.wrk[31], I.wrk[32], I.wrk[33]] + v + I.dims(box) + [0.1, 0.1, 0.1, 0.03]
    oa, ga = run_both("lap_bfld", args)
    for k in (3, 4, 5):
        assert_same(ga[k], oa[k], f"lap_bfld {k}")


@pytest.mark.parametrize("cfg,box,chi", [("tiny2", 1, 0.008), ("tiny2", 2, 0.3), ("small", 1, 0.004)])
def test_fcsmooth(cfg, box, chi):
    I = Inputs(cfg)
    tmp = I.scratch(1.0, 3)
    for q in (0, 5, 31):
        args = [I.cur[q], I.old[q], I.wrk[q]] + I.dims(box) + [chi] + tmp
        oa, ga = run_both("fcsmooth", args)
        assert_same(ga[0], oa[0], f"fcsmooth field {q}")


def test_flux_correct():
    I = Inputs("tiny2")
    p = I.p
    box = 2
    vv = I.scratch(1.0, 3)
    args = [list(I.cur), list(I.wrk), list(I.old)] + vv + I.dims(box) + [p.difrho, p.diferg]
    oa, ga = run_both("flux_correct", args, oracle_drop=(3, 4, 5))
    for q in range(34):
        assert_same(ga[0][q], oa[0][q], f"flux_correct field {q}")


def guard_inputs(I, box):
    """Plant cells that trip set_rho and the speed limiter."""
    rng = np.random.default_rng(11)
    p = I.p
    c = I.cur
    nz, ny, nx = p.nz, p.ny, p.nx
    for _ in range(12):
        k, j, i = rng.integers(1, nz - 1), rng.integers(1, ny - 1), rng.integers(1, nx - 1)
        s = 10 * int(rng.integers(0, 3))
        kind = int(rng.integers(0, 4))
        if kind == 0:
            c[s + 0, box - 1, k, j, i] = -1e-5           # density below the floor
        elif kind == 1:
            c[s + 5, box - 1, k, j, i] = -abs(c[s + 5, box - 1, k, j, i])   # negative pressure
        elif kind == 2:
            c[s + 1, box - 1, k, j, i] = 50.0 * c[s + 0, box - 1, k, j, i]  # fast
        else:
            c[s + 4, box - 1, k, j, i] = 400.0 * c[s + 0, box - 1, k, j, i]  # hot
        c[30, box - 1, k, j, i] = -abs(c[30, box - 1, k, j, i]) * 1e3       # negative, hot electrons


@pytest.mark.parametrize("box", [1, 2])
def test_set_rho(box):
    I = Inputs("tiny2")
    guard_inputs(I, box)
    p = I.p
    f = I.cur
    args = ([f[0], f[4], f[5], f[6], f[7], f[8], f[9], p.rmassq, f[10], f[14], f[15], f[16], f[17], f[18], f[19],
             p.rmassh, f[20], f[24], f[25], f[26], f[27], f[28], f[29], p.rmasso, f[30]] + I.dims(box) + [p.o_conc])
    oa, ga = run_both("set_rho", args)
    for k in [0, 1, 2, 3, 4, 5, 6, 8, 9, 10, 11, 12, 13, 14, 16, 17, 18, 19, 20, 21, 22, 24]:
        assert_same(ga[k], oa[k], f"set_rho arg {k}")


@pytest.mark.parametrize("box", [1, 2])
def test_set_speed_agrd(box):
    I = Inputs("tiny2")
    guard_inputs(I, box)
    p = I.p
    f = I.cur
    btot = np.zeros(I.box3, np.float32)
    outs = [ctypes.c_float() for _ in range(6)]
    vlim = p.vlim_factor * box
    args = (I.dims(box)[:4] + [box, p.rmassq, p.rmassh, p.rmasso, 0, p.smallbit, p.aniso_limit, vlim, p.qvlim,
                               p.hvlim, p.ovlim, p.qclim, p.hclim, p.oclim, p.cslim,
                               f[31], f[32], f[33], I.b0[0], I.b0[1], I.b0[2]]
            + [f[q] for q in range(30)] + [f[30], btot])
    from oracle import oracle
    from g3m3_gb300.api import Context
    from _support import copy_args
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
    del outs
    for k in range(25, 57):
        assert_same(ga[k], oa[k], f"set_speed_agrd arg {k}")
    for x, y, n in zip(go, oo, ("pxmax", "pymax", "pzmax", "csmax", "alfmax", "fastest")):
        assert x.value == y.value, (n, x.value, y.value)


def test_store_array():
    I = Inputs("tiny2")
    args = [I.old[0], I.cur[0]] + I.dims(2)
    oa, ga = run_both("store_array", args)
    assert_same(ga[0], oa[0], "store_array")


def test_bndry_outer():
    I = Inputs("tiny2")
    p = I.p
    args = [list(I.wrk), I.b0[0], I.b0[1], I.b0[2], p]
    oa, ga = run_both("bndry_outer", args)
    for q in range(34):
        assert_same(ga[0][q], oa[0][q], f"bndry_outer field {q}")


def test_bndry_inner():
    I = Inputs("tiny2")
    p = I.p
    L = I.lists
    args = [list(I.wrk), L["parm_srf"], L["parm_mid"], L["parm_zero"], L["ijsrf"], L["numsrf"], L["ijmid"],
            L["nummid"], L["ijzero"], L["numzero"], L["ijsrf"].shape[0], L["ijmid"].shape[0], L["ijzero"].shape[0],
            p]
    oa, ga = run_both("bndry_inner", args)
    for q in range(34):
        assert_same(ga[0][q], oa[0][q], f"bndry_inner field {q}")


@pytest.mark.parametrize("tt", [0.0, 0.37, 1.0])
def test_flanks(tt):
    I = Inputs("tiny3")
    p = I.p
    g = I.grid()
    for box in (1, 2):
        t_old = (ctypes.c_double * p.n_grids)(*([0.0] * p.n_grids))
        t_new = (ctypes.c_double * p.n_grids)(*([0.2] * p.n_grids))
        work = np.zeros(I.box3, np.float32)
        for q in (0, 7, 30, 33):
            args = [I.wrk[q], I.cur[q], I.old[q]] + I.dims(box) + [t_new, t_old, 0.2 * tt, work] + g
            oa, ga = run_both("flanks", args)
            assert_same(ga[0], oa[0], f"flanks box {box} field {q}")


def test_corer_and_synced():
    I = Inputs("tiny3")
    g = I.grid()
    for box in (1, 2):
        for q in (0, 9, 32):
            oa, ga = run_both("corer", [I.cur[q]] + I.dims(box) + g)
            assert_same(ga[0], oa[0], f"corer box {box} field {q}")
            oa, ga = run_both("flanks_synced", [I.cur[q]] + I.dims(box) + g)
            assert_same(ga[0], oa[0], f"flanks_synced box {box} field {q}")


def divergence(bx, by, bz, rx):
    d = np.zeros_like(bx, dtype=np.float64)
    d[1:-1, 1:-1, 1:-1] = ((bx[1:-1, 1:-1, 2:] - bx[1:-1, 1:-1, :-2]) + (by[1:-1, 2:, 1:-1] - by[1:-1, :-2, 1:-1])
                           + (bz[2:, 1:-1, 1:-1] - bz[:-2, 1:-1, 1:-1])) / (2.0 * rx)
    return d


@pytest.mark.parametrize("cfg,errlim", [("tiny2", 1e-4), ("tiny2", 1e-6), ("small", 1e-4)])
def test_divb_correct(cfg, errlim):
    """Compared with the FP64 build: the oracle sums dot products serially
    in FP32 as the reference does, the library in FP64; the library's B must
    be as close to the FP64 solve as the reference's (tests/_divb_parity.py)."""
    check_divb(Inputs(cfg), 1, errlim)


def check_divb(I, box, errlim):
    p = I.p
    pos = (ctypes.c_int * 7)(p.nx * p.ny, p.nx, 1, 0, -1, -p.nx, -p.nx * p.ny)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    b = [I.cur[31].copy(), I.cur[32].copy(), I.cur[33].copy()]
    from oracle import oracle
    from g3m3_gb300.api import Context
    ob = [x.copy() for x in b]
    it_o = oracle.call("divb_correct", *I.dims(box), 7, pos, xs, errlim, *ob)
    gb = [x.copy() for x in b]
    it_g = ctypes.c_int()
    with Context() as ctx:
        ctx.call("divb_correct", *I.dims(box), 7, pos, xs, errlim, *gb, ctypes.addressof(it_g))
        ctx.sync_to_host(*gb)
    rx = float(xs[box - 1])
    d0 = divergence(*(x[box - 1] for x in b), rx)
    dg = divergence(*(x[box - 1] for x in gb), rx)
    do = divergence(*(x[box - 1] for x in ob), rx)
    # both reduce the divergence; the GPU residual meets the reference criterion
    assert np.linalg.norm(dg) < np.linalg.norm(d0)
    assert np.linalg.norm(dg) <= 1.5 * np.linalg.norm(do) + 1e-6 * np.linalg.norm(d0)
    # per component, the GPU's B is at least as close to the FP64 build's
    # (within the stated slack) as the reference's FP32 solve is
    import _divb_parity as D
    b8, _ = D.divb_correct_r8(*I.dims(box), pos, xs, errlim, *b)
    for q in range(3):
        eg, er = D.rel(gb[q][box - 1], b8[q][box - 1]), D.rel(ob[q][box - 1], b8[q][box - 1])
        assert eg <= D.SLACK * er + D.FLOOR, (q, eg, er, it_o, it_g.value)
    assert abs(it_g.value - it_o) <= max(3, 0.25 * it_o), (it_g.value, it_o)


def test_sample_points():
    I = Inputs("tiny3")
    p = I.p
    rng = np.random.default_rng(3)
    n = 64
    gmin = np.array([[p.grd_xmin[b], p.grd_ymin[b], p.grd_zmin[b]] for b in range(p.n_grids)], np.float32)
    gmax = np.array([[p.grd_xmax[b], p.grd_ymax[b], p.grd_zmax[b]] for b in range(p.n_grids)], np.float32)
    xyz = (rng.uniform(-1, 1, (n, 3)) * np.array([20.0, 20.0, 8.0]) * p.re_equiv).astype(np.float32)
    # points outside every box: findgrid clamps them into the outermost box
    # (cft_findgrid.f90:49-54) and trilin_interp extrapolates from there
    xyz[-6:] = (np.array([[500.0, 0, 0], [-500.0, 3, 1], [0, 400.0, 0], [2, -400.0, 1], [0, 1, 300.0],
                          [-1, 0, -300.0]]) * p.re_equiv).astype(np.float32)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    field = I.cur[32]
    out = np.zeros(n, np.float32)
    from oracle import oracle
    from g3m3_gb300.api import Context
    with Context() as ctx:
        ctx.call("sample_points", field, p.nx, p.ny, p.nz, p.n_grids, gmin, gmax, xs, p.re_equiv, xyz, n, out)
        ctx.sync_to_host(out)
    for t in range(n):
        gp = (ctypes.c_int * 4)()
        oracle.call("findgrid", np.ascontiguousarray(xyz[t]), p.n_grids, gmin, gmax, xs, gp, p.re_equiv)
        i, j, k, b = gp[0], gp[1], gp[2], gp[3]
        cube = np.zeros((2, 3), np.float32)
        for a in range(3):
            cube[0, a] = (gmin[b - 1, a] + (gp[a] - 1.0) * xs[b - 1]) * p.re_equiv
            cube[1, a] = cube[0, a] + xs[b - 1] * p.re_equiv
        q = np.ascontiguousarray(field[b - 1, k - 1:k + 1, j - 1:j + 1, i - 1:i + 1])  # (z,y,x) = Fortran (2,2,2)
        v = ctypes.c_float()
        oracle.call("trilin_interp", np.ascontiguousarray(xyz[t]), cube, q, ctypes.addressof(v))
        assert out[t] == v.value, (t, out[t], v.value)


@pytest.mark.parametrize("recurse,redo_lim,x0", [(0, 0, 0.0), (1, 2, 0.3)])
def test_sparse_solver(recurse, redo_lim, x0):
    """Banded CGNR on a symmetric, diagonally dominant 7-band system, from a
    zero or a random start; compared at the solver's tolerance (FP64 dot
    products here, FP32 in the oracle)."""
    from oracle import oracle
    from g3m3_gb300.api import Context
    nx = ny = nz = 11
    n = nx * ny * nz
    pos = np.array([nx * ny, nx, 1, 0, -1, -nx, -nx * ny], np.int32)
    coef = np.array([1, 1, 1, -6.5, 1, 1, 1], np.float32)
    bm = np.ascontiguousarray(np.repeat(coef[None, :], n, axis=0))   # banded_matrix(7, n), column-major
    rng = np.random.default_rng(17)
    b = rng.standard_normal(n).astype(np.float32)
    start = (x0 * rng.standard_normal(n)).astype(np.float32)
    errlim = 1e-6
    xo = start.copy()
    r2o = ctypes.c_float()
    it_o = oracle.call("sparse_solver", 7, n, pos, errlim, recurse, redo_lim, b, xo, ctypes.addressof(r2o), bm)
    xg = start.copy()
    r2g = ctypes.c_float()
    with Context() as ctx:
        ctx.call("sparse_solver", 7, n, pos, errlim, recurse, redo_lim, b, xg, ctypes.addressof(r2g), bm)
        ctx.sync_to_host(xg)
    # the residual the library reports is the residual of its solution
    def op(x):
        out = np.zeros(n, np.float64)
        for c, p in zip(coef, pos):
            idx = np.arange(n) + p
            ok = (idx >= 0) & (idx < n)
            out[ok] += float(c) * x[idx[ok]]
        return out
    r2_true = float(np.sum((op(xg.astype(np.float64)) - b) ** 2))
    assert r2_true <= 1.01 * float(np.sum(b.astype(np.float64) ** 2)) * n * errlim ** 2 * 1.5 + 1e-12
    assert abs(r2g.value - r2_true) <= 0.05 * r2_true + 1e-10
    assert rel_l2(xg, xo) < 1e-2, (rel_l2(xg, xo), it_o)


@pytest.mark.parametrize("cfg,box", [("tiny2", 1), ("tiny2", 2), ("small", 1)])
def test_flux_counter(cfg, box):
    """Wall sums in the reference's serial order: the six fluxes are the
    oracle's bits, for inflow and outflow walls alike."""
    I = Inputs(cfg)
    p = I.p
    f = I.cur
    rng = np.random.default_rng(23)
    moms = []
    for s in range(3):
        for q in range(3):
            a = f[10 * s + 1 + q].copy()
            a += (0.3 * rng.standard_normal(a.shape)).astype(np.float32)   # both signs on every wall
            moms.append(a)
    args = moms + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, 1.7e3]
    from oracle import oracle
    from g3m3_gb300.api import Context
    oo = [ctypes.c_float() for _ in range(6)]
    oracle.call("flux_counter", *args, *[ctypes.addressof(x) for x in oo])
    go = [ctypes.c_float() for _ in range(6)]
    with Context() as ctx:
        ctx.call("flux_counter", *args, *[ctypes.addressof(x) for x in go])
    for x, y, n in zip(go, oo, ("q in", "q out", "h in", "h out", "o in", "o out")):
        assert x.value == y.value, (n, x.value, y.value)
    assert any(x.value != 0.0 for x in go)
