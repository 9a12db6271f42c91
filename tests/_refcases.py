"""Per-routine cases shared by the reference pin, the reference-made golden
digests and their GPU check.

Each case builds its seeded inputs and runs one routine on one side:
``"ref"`` (the reference's own Fortran, compiled through
oracle/fortran_to_c.py), ``"oracle"`` (the CPU restatement) or ``"gpu"``
(the library's drop-in entry of the same name), and returns the routine's
results by name -- every array argument after the call, inputs included, and
the scalars it returns.  The argument lists are the reference's dummy lists
(sub_*.f90 headers); the oracle and the library take the same lists, with
34-field tables where the reference passes the 34 arrays one by one
(flux_correct, bndry_outer, bndry_inner, bndry_flanks, bndry_corer).
"""
from __future__ import annotations

import ctypes

import numpy as np

from _support import Inputs, copy_args, tables

SP = {"q": 0, "h": 10, "o": 20}
# a species' ten fields in the reference's usual dummy order
# rho, presx, presy, presz, presxy, presxz, presyz, px, py, pz
FC_ORDER = [0, 4, 5, 6, 7, 8, 9, 1, 2, 3]
FIELD_OF = {"rho": 0, "px": 1, "py": 2, "pz": 3, "presx": 4, "presy": 5, "presz": 6, "presxy": 7,
            "presxz": 8, "presyz": 9}


def species(arr, s):
    b = SP[s]
    return [arr[b + i] for i in range(10)]


def field_index(name):
    """34-table index of a reference dummy such as wrkhpresxy, oldbz, epres;
    returns (prefix, index) with prefix '', 'wrk' or 'old'."""
    for pre in ("wrk", "old", ""):
        if not name.startswith(pre):
            continue
        rest = name[len(pre):]
        if rest == "epres":
            return pre, 30
        if rest in ("bx", "by", "bz"):
            return pre, 31 + "xyz".index(rest[1])
        if rest[:1] in SP and rest[1:] in FIELD_OF:
            return pre, SP[rest[0]] + FIELD_OF[rest[1:]]
    raise KeyError(name)


# ---------------------------------------------------------------- running

def _gpu(name, a, extra=()):
    from g3m3_gb300.api import Context
    targs, keep = tables(a)
    with Context() as ctx:
        ctx.call(name, *targs, *extra)
        for x in a:
            if isinstance(x, np.ndarray):
                ctx.sync_to_host(x)
            elif isinstance(x, list):
                for y in x:
                    if isinstance(y, np.ndarray):
                        ctx.sync_to_host(y)
        ctx.synchronize()
    del keep


def _oracle(name, a, extra=()):
    from oracle import oracle
    targs, keep = tables(a)
    r = oracle.call(name, *targs, *extra)
    del keep
    return r


def uniform(side, name, args, ignore=(), scalars=0):
    """Routines whose oracle, library and reference argument lists are the
    same; the last `scalars` arguments are scalar results (REAL, by
    reference)."""
    a = copy_args(args)
    outs = [ctypes.c_float() for _ in range(scalars)]
    if side == "ref":
        import _refpin
        _refpin.call(name, *a, *outs)
    elif side == "oracle":
        _oracle(name, a, [ctypes.addressof(x) for x in outs])
    else:
        _gpu(name, a, [ctypes.addressof(x) for x in outs])
    res = {f"arg{i}": x for i, x in enumerate(a) if isinstance(x, np.ndarray) and i not in ignore}
    for i, x in enumerate(outs):
        res[f"out{i}"] = np.float32(x.value)
    return res


def table_results(f):
    return {f"field{q}": f[q] for q in range(34)}


# ---------------------------------------------------------------- cases

def push_ion_args(I, s, box, delt):
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


def c_push_ion(side, cfg, box, s, delt):
    I = Inputs(cfg)
    return uniform(side, "push_ion", push_ion_args(I, s, box, delt))


def c_push_elec(side, box, rx):
    I = Inputs("tiny2")
    p = I.p
    ev = I.scratch(0.1, 3)
    return uniform(side, "push_elec", [I.wrk[30], I.old[30], I.cur[30]] + ev + [p.gamma, p.gamma1]
                   + I.dims(box) + [0.02, rx, rx, rx])


def c_push_bfld(side, box, rx):
    I = Inputs("tiny2")
    ef = I.scratch(0.01, 3)
    return uniform(side, "push_bfld", [I.cur[31], I.cur[32], I.cur[33], I.old[31], I.old[32], I.old[33]] + ef
                   + I.dims(box) + [0.02, rx, rx, rx])


def c_calcur(side, cfg, box):
    I = Inputs(cfg)
    rx = float(I.p.xspac[box - 1])
    return uniform(side, "calcur", [I.cur[31], I.cur[32], I.cur[33]] + I.dims(box) + I.scratch(1.0, 3)
                   + [rx, rx, rx])


def _sp(I):
    sp = []
    for s in ("q", "h", "o"):
        f = species(I.cur, s)
        sp += [f[1], f[2], f[3], f[0]]
    return sp


def c_fnd_evel(side, box):
    I = Inputs("tiny2")
    p = I.p
    return uniform(side, "fnd_evel", _sp(I) + I.scratch(0.1, 3) + I.scratch(1.0, 6) + I.dims(box)
                   + [p.rmassq, p.rmassh, p.rmasso, p.reynolds])


def c_fnd_vtot(side, box):
    I = Inputs("tiny2")
    p = I.p
    return uniform(side, "fnd_vtot", _sp(I) + I.scratch(1.0, 3) + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso])


def c_fnd_pres(side, box):
    I = Inputs("tiny2")
    f = species(I.cur, "h")
    out = [np.zeros_like(I.cur[0]) for _ in range(3)]
    return uniform(side, "fnd_pres", [f[4], f[5], f[6], f[7], f[8], f[9]] + out + I.scratch(0.1, 3)
                   + I.scratch(0.1, 3) + I.dims(box))


def c_bande(side, box):
    I = Inputs("tiny2")
    p = I.p
    L = I.lists
    bs = [(I.b0[q, box - 1] + I.cur[31 + q, box - 1]).astype(np.float32) for q in range(3)]
    args = (I.scratch(1.0, 3) + bs + I.scratch(0.1, 3) + I.scratch(0.1, 3)
            + [I.scratch(1.0)[0], I.cur[30], I.cur[0], I.cur[10], I.cur[20], I.resistive, p.resist, p.reynolds]
            + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, L["ijmid"], L["nummid"], L["ijzero"], p.mbndry,
                             L["numzero"], L["ijmid"].shape[0], L["ijzero"].shape[0]]
            + [float(p.xspac[box - 1])] * 3)
    return uniform(side, "bande", args)


def c_lap_plasma(side, box, iso):
    I = Inputs("tiny2")
    v = I.scratch(0.2, 3)
    return uniform(side, "lap_plasma", species(I.cur, "o") + species(I.wrk, "o") + v + I.dims(box)
                   + [0.1, 0.07, 0.1, 0.03, iso])


def c_lap_elec(side, box):
    I = Inputs("tiny2")
    v = I.scratch(0.2, 3)
    return uniform(side, "lap_elec", [I.cur[30], I.wrk[30]] + v + I.dims(box) + [0.1, 0.1, 0.1, 0.03])


def c_lap_bfld(side, box):
    I = Inputs("tiny2")
    v = I.scratch(0.2, 3)
    return uniform(side, "lap_bfld", [I.cur[31], I.cur[32], I.cur[33], I.wrk[31], I.wrk[32], I.wrk[33]] + v
                   + I.dims(box) + [0.1, 0.1, 0.09, 0.03])


def c_fcsmooth(side, cfg, box, chi, q):
    I = Inputs(cfg)
    tmp = I.scratch(1.0, 3)
    # the three work arrays are the reference's scratch, not results
    return uniform(side, "fcsmooth", [I.cur[q], I.old[q], I.wrk[q]] + I.dims(box) + [chi] + tmp,
                   ignore=(9, 10, 11))


def c_flux_correct(side, box):
    I = Inputs("tiny2")
    p = I.p
    vv = I.scratch(1.0, 3)
    cur, wrk, old = (np.array(x) for x in (I.cur, I.wrk, I.old))
    if side == "ref":
        import _refpin
        ref = []
        for s in ("q", "h", "o"):
            b = SP[s]
            ref += [cur[b + k] for k in FC_ORDER] + [wrk[b + k] for k in FC_ORDER] + [old[b + k] for k in FC_ORDER]
        ref += ([cur[30], wrk[30], old[30], cur[31], cur[32], cur[33], wrk[31], wrk[32], wrk[33],
                 old[31], old[32], old[33]] + vv + I.dims(box)
                + [p.difrho, p.diferg, np.array(p.xspac[: p.n_grids], np.float32), 0])
        _refpin.call("flux_correct", *ref)
        return table_results(cur)
    tc, tw, to = list(cur), list(wrk), list(old)
    if side == "oracle":
        _oracle("flux_correct", [tc, tw, to] + vv + I.dims(box) + [p.difrho, p.diferg])
    else:
        _gpu("flux_correct", [tc, tw, to] + I.dims(box) + [p.difrho, p.diferg])
    return table_results(cur)


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
            c[s + 0, box - 1, k, j, i] = -1e-5            # density below the floor
        elif kind == 1:
            c[s + 5, box - 1, k, j, i] = -abs(c[s + 5, box - 1, k, j, i])    # negative pressure
        elif kind == 2:
            c[s + 1, box - 1, k, j, i] = 50.0 * c[s + 0, box - 1, k, j, i]   # fast
        else:
            c[s + 4, box - 1, k, j, i] = 400.0 * c[s + 0, box - 1, k, j, i]  # hot
        c[30, box - 1, k, j, i] = -abs(c[30, box - 1, k, j, i]) * 1e3        # negative, hot electrons


def c_set_rho(side, box):
    I = Inputs("tiny2")
    guard_inputs(I, box)
    p = I.p
    f = I.cur
    return uniform(side, "set_rho", [f[0], f[4], f[5], f[6], f[7], f[8], f[9], p.rmassq, f[10], f[14], f[15],
                                     f[16], f[17], f[18], f[19], p.rmassh, f[20], f[24], f[25], f[26], f[27],
                                     f[28], f[29], p.rmasso, f[30]] + I.dims(box) + [p.o_conc])


def c_set_speed_agrd(side, box):
    """Anisotropic limiter path (isotropic = .false.); the six maxima too."""
    I = Inputs("tiny2")
    guard_inputs(I, box)
    p = I.p
    f = I.cur
    vlim = p.vlim_factor * box
    args = (I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, 0, p.smallbit, p.aniso_limit, vlim, p.qvlim,
                           p.hvlim, p.ovlim, p.qclim, p.hclim, p.oclim, p.cslim,
                           f[31], f[32], f[33], I.b0[0], I.b0[1], I.b0[2]]
            + [f[q] for q in range(30)] + [f[30], np.zeros(I.box3, np.float32)])
    return uniform(side, "set_speed_agrd", args, scalars=6)


def nan_speed_inputs(I, box, plant):
    """Cells whose limiter speeds are NaN or infinite: density -smallbit
    (rho + smallbit = 0) with zero momenta and pressures gives NaN, with a
    momentum gives inf; three negative densities give a NaN Alfven speed.
    The reference folds its maxima in loop order with amax1, so a NaN resets
    the running value: 'last' puts the NaN on the last element of the
    species loops, 'mid' an inf and then a NaN in the first species and
    the Alfven NaN halfway through."""
    p = I.p
    c = I.cur
    b = box - 1
    sb = np.float32(-np.float32(p.smallbit))

    def nan_cell(s, k, j, i, px=0.0):
        c[s + 0, b, k, j, i] = sb
        c[s + 1, b, k, j, i] = px
        c[s + 2, b, k, j, i] = 0.0
        c[s + 3, b, k, j, i] = 0.0
        for q in (4, 5, 6):
            c[s + q, b, k, j, i] = 0.0

    nz, ny, nx = p.nz, p.ny, p.nx
    if plant == "last":
        nan_cell(20, nz - 2, ny - 2, nx - 2)
    else:
        nan_cell(0, 2, 3, 4, px=5.0)          # inf, then
        nan_cell(0, nz // 2, ny // 2, 5)      # NaN in the first species loop
        for s in (0, 10, 20):                 # the Alfven speed's NaN
            c[s, b, nz // 2, ny // 2 + 1, 3] = -1.0


def c_set_speed_agrd_nan(side, box, plant):
    """The maxima where speeds are NaN or infinite (nan_speed_inputs)."""
    I = Inputs("tiny2")
    nan_speed_inputs(I, box, plant)
    p = I.p
    f = I.cur
    vlim = p.vlim_factor * box
    args = (I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, 0, p.smallbit, p.aniso_limit, vlim, p.qvlim,
                           p.hvlim, p.ovlim, p.qclim, p.hclim, p.oclim, p.cslim,
                           f[31], f[32], f[33], I.b0[0], I.b0[1], I.b0[2]]
            + [f[q] for q in range(30)] + [f[30], np.zeros(I.box3, np.float32)])
    return uniform(side, "set_speed_agrd", args, scalars=6)


def c_store_array(side):
    I = Inputs("tiny2")
    return uniform(side, "store_array", [I.old[0], I.cur[0]] + I.dims(2))


def c_bndry_outer(side, cfg):
    I = Inputs(cfg)
    p = I.p
    f = np.array(I.wrk)
    if side == "ref":
        import _refpin
        sp, offd = [], []
        for s in ("q", "h", "o"):
            b = SP[s]
            sp += [f[b], f[b + 4], f[b + 5], f[b + 6], f[b + 1], f[b + 2], f[b + 3]]
            offd += [f[b + 7], f[b + 8], f[b + 9]]
        _refpin.call("bndry_outer", *(sp + [f[30]] + offd + [
            p.rmassq, p.rmassh, p.rmasso, f[31], f[32], f[33], I.b0[0], I.b0[1], I.b0[2],
            p.nx, p.ny, p.nz, p.n_grids, p.srho, p.rho_frac, p.o_conc, p.spress, p.spx, p.spy, p.spz,
            p.sbx_wind, p.sby_wind, p.sbz_wind, p.ti_te, p.isotropic]))
    else:
        (_oracle if side == "oracle" else _gpu)("bndry_outer", [list(f), I.b0[0], I.b0[1], I.b0[2], p])
    return table_results(f)


def c_bndry_inner(side, cfg):
    I = Inputs(cfg)
    p = I.p
    L = I.lists
    f = np.array(I.wrk)
    if side == "ref":
        import _refpin
        _refpin.set_common("rotation", v_rot=p.v_rot, r_rot=p.r_rot)
        sp, offd = [], []
        for s in ("q", "h", "o"):
            b = SP[s]
            sp += [f[b], f[b + 4], f[b + 5], f[b + 6], f[b + 1], f[b + 2], f[b + 3],
                   {"q": p.rmassq, "h": p.rmassh, "o": p.rmasso}[s]]
            offd += [f[b + 7], f[b + 8], f[b + 9]]
        _refpin.call("bndry_inner", *(
            sp + [f[30], f[31], f[32], f[33]] + offd + [p.nx, p.ny, p.nz, p.n_grids]
            + [L["parm_srf"], L["parm_mid"], L["parm_zero"], L["ijsrf"], L["numsrf"], L["ijmid"], L["nummid"],
               L["ijzero"], L["numzero"], p.mbndry, L["ijsrf"].shape[0], L["ijmid"].shape[0], L["ijzero"].shape[0],
               p.erho, p.epress, p.alpha_e, p.ti_te, p.o_conc, p.re_equiv, p.r_inner, p.sbx_wind, p.spress]
            + I.grid()))
    else:
        (_oracle if side == "oracle" else _gpu)("bndry_inner", [
            list(f), L["parm_srf"], L["parm_mid"], L["parm_zero"], L["ijsrf"], L["numsrf"], L["ijmid"],
            L["nummid"], L["ijzero"], L["numzero"], L["ijsrf"].shape[0], L["ijmid"].shape[0],
            L["ijzero"].shape[0], p])
    return table_results(f)


def _times(p):
    t_old = (ctypes.c_double * p.n_grids)(*([0.0] * p.n_grids))
    t_new = (ctypes.c_double * p.n_grids)(*([0.2] * p.n_grids))
    return t_old, t_new


def c_flanks(side, box, tt, q):
    I = Inputs("tiny3")
    p = I.p
    t_old, t_new = _times(p)
    work = np.zeros(I.box3, np.float32)
    # work is the reference's scratch, not a result
    return uniform(side, "flanks", [I.wrk[q], I.cur[q], I.old[q]] + I.dims(box)
                   + [t_new, t_old, 0.2 * tt, work] + I.grid(), ignore=(11,))


def c_bndry_flanks(side, box):
    """The 34-field wrapper (sub_bndry_flanks.f90:105-209); the oracle side
    calls its per-field flanks in the same order."""
    I = Inputs("tiny3")
    p = I.p
    g = I.grid()
    t_old, t_new = _times(p)
    t = 0.071
    cur, wrk, old = (np.array(x) for x in (I.cur, I.wrk, I.old))
    if side == "ref":
        import _refpin
        arrs = {"wrk": wrk, "old": old, "": cur}
        names = [d["name"] for d in _refpin.dummies("bndry_flanks")]
        ref = []
        for n in names[:102]:
            pre, q = field_index(n)
            ref.append(arrs[pre][q])
        ref += [np.zeros(I.box3, np.float32)] + I.dims(box) + [t_old, t_new, ctypes.c_double(t)] + g
        _refpin.call("bndry_flanks", *ref)
    elif side == "oracle":
        from oracle import oracle
        work = np.zeros(I.box3, np.float32)
        for q in range(34):
            oracle.call("flanks", wrk[q], cur[q], old[q], *I.dims(box), t_new, t_old, t, work, *g)
    else:
        _gpu("bndry_flanks", [list(wrk), list(cur), list(old)] + I.dims(box) + [t_old, t_new, t] + g)
    return table_results(wrk)


def c_bndry_corer(side, box):
    """The 34-field wrapper (sub_bndry_corer.f90:42-111)."""
    I = Inputs("tiny3")
    g = I.grid()
    cur = np.array(I.cur)
    if side == "ref":
        import _refpin
        names = [d["name"] for d in _refpin.dummies("bndry_corer")]
        _refpin.call("bndry_corer", *([cur[field_index(n)[1]] for n in names[:34]] + I.dims(box) + g))
    elif side == "oracle":
        from oracle import oracle
        for q in range(34):
            oracle.call("corer", cur[q], *I.dims(box), *g)
    else:
        _gpu("bndry_corer", [list(cur)] + I.dims(box) + g)
    return table_results(cur)


def c_corer(side, box, q):
    I = Inputs("tiny3")
    return uniform(side, "corer", [I.cur[q]] + I.dims(box) + I.grid())


def c_flanks_synced(side, box, q):
    I = Inputs("tiny3")
    return uniform(side, "flanks_synced", [I.cur[q]] + I.dims(box) + I.grid())


def c_divb_correct(side, cfg, box, errlim):
    """The whole projection with the reference's FP32 dot products, from a
    zero start (bitwise between the reference and the oracle; the library
    sums in FP64 and is checked at the solver's tolerance elsewhere)."""
    I = Inputs(cfg)
    p = I.p
    pos = np.array([p.nx * p.ny, p.nx, 1, 0, -1, -p.nx, -p.nx * p.ny], np.int32)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    args = I.dims(box) + [7, pos, xs, errlim, I.cur[31], I.cur[32], I.cur[33]]
    return uniform(side, "divb_correct", args)


def c_divb_zero(side):
    """An exactly divergence-free B (uniform): the first iteration divides
    0/0, x becomes NaN and the solver returns through its gg = 0 test; the
    interior of B becomes NaN on every side alike."""
    I = Inputs("tiny")
    p = I.p
    pos = np.array([p.nx * p.ny, p.nx, 1, 0, -1, -p.nx, -p.nx * p.ny], np.int32)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    b = [np.full_like(I.cur[31 + q], v) for q, v in enumerate((0.3, -0.1, 0.2))]
    args = I.dims(1) + [7, pos, xs, 1e-4] + b
    if side != "gpu":
        return uniform(side, "divb_correct", args)
    # the library returns an error status unless the solve ends the
    # reference's way (its gg = 0 return), which Context.call would raise
    a = copy_args(args)
    iters = ctypes.c_int()
    _gpu("divb_correct", a, [ctypes.addressof(iters)])
    assert iters.value == 1, iters.value
    return {f"arg{i}": x for i, x in enumerate(a) if isinstance(x, np.ndarray)}


def c_sparse_solver(side, recurse, redo_lim, x0):
    nx = ny = nz = 9
    n = nx * ny * nz
    pos = np.array([nx * ny, nx, 1, 0, -1, -nx, -nx * ny], np.int32)
    coef = np.array([1, 1, 1, -6.5, 1, 1, 1], np.float32)
    bm = np.ascontiguousarray(np.repeat(coef[None, :], n, axis=0))
    rng = np.random.default_rng(17)
    rhs = rng.standard_normal(n).astype(np.float32)
    start = (x0 * rng.standard_normal(n)).astype(np.float32)
    x, b, r2 = start.copy(), bm.copy(), ctypes.c_float()
    if side == "ref":
        import _refpin
        _refpin.call("sparse_solver", 7, n, pos, 1e-6, recurse, redo_lim, rhs, x, r2, b)
    else:
        from oracle import oracle
        oracle.call("sparse_solver", 7, n, pos, 1e-6, recurse, redo_lim, rhs, x, ctypes.addressof(r2), b)
    return {"soln_vec": x, "banded_matrix": b, "residual2": np.float32(r2.value)}


def c_findgrid_trilin(side, seed):
    """findgrid's containing box and corner index, and trilin_interp of a
    seeded cube, for 20 seeded points."""
    I = Inputs("tiny3")
    p = I.p
    rng = np.random.default_rng(seed)
    gmin = np.array([[p.grd_xmin[b], p.grd_ymin[b], p.grd_zmin[b]] for b in range(p.n_grids)], np.float32)
    gmax = np.array([[p.grd_xmax[b], p.grd_ymax[b], p.grd_zmax[b]] for b in range(p.n_grids)], np.float32)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    grid, vals = [], []
    for _ in range(20):
        xyz = (rng.uniform(-1, 1, 3) * np.array([20.0, 20.0, 8.0]) * p.re_equiv).astype(np.float32)
        cube = rng.uniform(-5, 5, (2, 3)).astype(np.float32)
        cube[1] = cube[0] + np.abs(cube[1]) + 0.5
        q = rng.standard_normal((2, 2, 2)).astype(np.float32)
        pt = (cube[0] + rng.uniform(0, 1, 3).astype(np.float32) * (cube[1] - cube[0])).astype(np.float32)
        gp = np.zeros(4, np.int32)
        v = ctypes.c_float()
        if side == "ref":
            import _refpin
            _refpin.call("findgrid", xyz, p.n_grids, gmin, gmax, xs, gp, p.re_equiv, b"craft001")
            _refpin.call("trilin_interp", pt, cube, q, v)
        else:
            from oracle import oracle
            oracle.call("findgrid", xyz, p.n_grids, gmin, gmax, xs, gp, p.re_equiv)
            oracle.call("trilin_interp", pt, cube, q, ctypes.addressof(v))
        grid.append(gp)
        vals.append(v.value)
    return {"gridpt": np.array(grid, np.int32), "scdata": np.array(vals, np.float32)}


def c_flux_counter(side, box):
    I = Inputs("tiny2")
    p = I.p
    f = I.cur
    rng = np.random.default_rng(23)
    moms = []
    for s in range(3):
        for q in range(3):
            a = f[10 * s + 1 + q].copy()
            a += (0.3 * rng.standard_normal(a.shape)).astype(np.float32)   # both signs on every wall
            moms.append(a)
    return uniform(side, "flux_counter", moms + I.dims(box) + [p.rmassq, p.rmassh, p.rmasso, 1.7e3], scalars=6)


# (case id, function, keyword arguments, the library reproduces it bitwise)
CASES = []


def _add(fn, gpu=True, **kw):
    cid = fn.__name__[2:] + "".join(f"-{k}={v}" for k, v in kw.items())
    CASES.append((cid, fn, kw, gpu))


for _cfg, _box, _s, _dt in (("tiny2", 1, "q", 0.01), ("tiny2", 2, "o", 0.005), ("small", 1, "h", 0.01)):
    _add(c_push_ion, cfg=_cfg, box=_box, s=_s, delt=_dt)
for _box, _rx in ((1, 1.0), (2, 2.0), (1, 0.7)):
    _add(c_push_elec, box=_box, rx=_rx)
    _add(c_push_bfld, box=_box, rx=_rx)
for _cfg, _box in (("tiny2", 1), ("tiny2", 2), ("small", 1)):
    _add(c_calcur, cfg=_cfg, box=_box)
for _box in (1, 2):
    _add(c_fnd_evel, box=_box)
    _add(c_fnd_vtot, box=_box)
    _add(c_fnd_pres, box=_box)
    _add(c_bande, box=_box)
    _add(c_lap_elec, box=_box)
    _add(c_lap_bfld, box=_box)
    _add(c_flux_correct, box=_box)
    _add(c_set_rho, box=_box)
    _add(c_set_speed_agrd, box=_box)
    for _plant in ("last", "mid"):
        _add(c_set_speed_agrd_nan, box=_box, plant=_plant)
    _add(c_flux_counter, box=_box)
    _add(c_bndry_flanks, box=_box)
    _add(c_bndry_corer, box=_box)
for _box, _iso in ((1, 0), (2, 0), (1, 1)):
    _add(c_lap_plasma, box=_box, iso=_iso)
for _cfg, _box, _chi in (("tiny2", 1, 0.008), ("tiny2", 2, 0.3), ("small", 1, 0.004)):
    for _q in (0, 5, 31):
        _add(c_fcsmooth, cfg=_cfg, box=_box, chi=_chi, q=_q)
_add(c_store_array)
for _cfg in ("tiny2", "tiny3"):
    _add(c_bndry_outer, cfg=_cfg)
    _add(c_bndry_inner, cfg=_cfg)
for _box in (1, 2):
    for _tt in (0.0, 0.37, 1.0):
        for _q in (0, 7, 30, 33):
            _add(c_flanks, box=_box, tt=_tt, q=_q)
    for _q in (0, 9, 32):
        _add(c_corer, box=_box, q=_q)
        _add(c_flanks_synced, box=_box, q=_q)
for _cfg, _box, _e in (("tiny2", 1, 1e-4), ("tiny2", 2, 1e-6), ("tiny3", 1, 1e-4)):
    _add(c_divb_correct, gpu=False, cfg=_cfg, box=_box, errlim=_e)
_add(c_divb_zero)
for _r, _lim, _x0 in ((0, 0, 0.0), (1, 2, 0.3)):
    _add(c_sparse_solver, gpu=False, recurse=_r, redo_lim=_lim, x0=_x0)
for _seed in (3, 4):
    _add(c_findgrid_trilin, gpu=False, seed=_seed)


def run(cid, side):
    for c, fn, kw, _ in CASES:
        if c == cid:
            return fn(side, **kw)
    raise KeyError(cid)
