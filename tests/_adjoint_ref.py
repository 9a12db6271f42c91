"""FP64 references for the adjoint tests (TEST INFRASTRUCTURE).

The misfit of a virtual-spacecraft run evaluated with the oracle's FP64
build (every REAL in double precision; tests/test_ref_fp64.py pins it to the
reference's own FP64 build) under a given time-step schedule: the same main
steps the library's adjoint differentiates, so that central differences of
it check the library's gradients.  The sampling restates the library's
loss kernel: the smallest box whose open extent holds the point, the cube
at 1 + int((x - min) / spacing), trilinear weights, bx, by, bz and the sum
of the three densities; samples outside every box do not count.
"""
from __future__ import annotations

import numpy as np

WIND = ("srho", "spx", "spy", "spz", "spress", "sbx_wind", "sby_wind", "sbz_wind")


def sample_values(p, cur, xyz):
    """(n, 4) values of bx, by, bz, rho at xyz (n, 3) [planet radii]; NaN
    where no box holds the point.  cur: (34, n_grids, nz, ny, nx)."""
    out = np.full((len(xyz), 4), np.nan)
    for n, X in enumerate(np.asarray(xyz, np.float64)):
        v = X / p.re_equiv
        box = 0
        for b in range(1, p.n_grids + 1):
            mn = np.array([p.grd_xmin[b - 1], p.grd_ymin[b - 1], p.grd_zmin[b - 1]])
            mx = np.array([p.grd_xmax[b - 1], p.grd_ymax[b - 1], p.grd_zmax[b - 1]])
            if (v > mn).all() and (v < mx).all():
                box = b
                break
        if box == 0:
            continue
        mn = np.array([p.grd_xmin[box - 1], p.grd_ymin[box - 1], p.grd_zmin[box - 1]])
        sp = p.xspac[box - 1]
        g = 1 + ((v - mn) / sp).astype(int)
        if (g < 1).any() or g[0] >= p.nx or g[1] >= p.ny or g[2] >= p.nz:
            continue
        c0 = (mn + (g - 1) * sp) * p.re_equiv
        w = (X - c0) / (sp * p.re_equiv)
        i, j, k = g - 1
        val = np.zeros(4)
        for dk in (0, 1):
            for dj in (0, 1):
                for di in (0, 1):
                    wt = (w[0] if di else 1 - w[0]) * (w[1] if dj else 1 - w[1]) * (w[2] if dk else 1 - w[2])
                    c = (box - 1, k + dk, j + dj, i + di)
                    for q in range(3):
                        val[q] += wt * cur[31 + q][c]
                    val[3] += wt * (cur[0][c] + cur[10][c] + cur[20][c])
        out[n] = val
    return out


def oracle_loss(state, wind, schedule, samples, delta=None, real8=True):
    """Misfit of the run: init_steps, the state perturbed by ``delta`` (after
    init_steps, where the library's state gradient is taken), then the main
    steps under ``schedule`` ((N, n_grids) t_stepnew), with wind parameters
    ``wind`` (8)."""
    import ctypes
    from oracle.oracle import OracleModel
    st = state.copy()
    p = type(state.params)()
    ctypes.memmove(ctypes.addressof(p), ctypes.addressof(state.params), ctypes.sizeof(p))
    st.params = p
    for k, v in zip(WIND, wind):
        setattr(p, k, float(np.float32(v)))
    om = OracleModel(st, omp=True, real8=real8)
    om.init_steps()
    if delta is not None:
        om.cur += delta
    xyz, step, target = samples
    loss = 0.0
    for s in range(len(schedule)):
        for b in range(p.n_grids):
            om.s.t_stepnew[b] = float(schedule[s][b])
        assert om.main_step() == 0
        sel = np.nonzero(np.asarray(step) == s + 1)[0]
        if len(sel):
            v = sample_values(p, om.cur, np.asarray(xyz)[sel])
            r = v - np.asarray(target, np.float64)[sel]
            r[np.isnan(r)] = 0.0
            loss += float((r * r).sum())
    return loss


def line_samples(state, nsteps, n=200, seed=20261205, scale=0.1):
    """n samples along a straight line through the outermost box (x from
    near its inflow face to near its back wall, y and z drawn from the seed
    between 15 and 30 % of the box's extent, beside the planet), spread
    evenly over the N main steps; targets are the initial values at the
    points times (1 + scale N(0,1))."""
    p = state.params
    rng = np.random.default_rng(seed)
    ng = p.n_grids
    lo = np.array([p.grd_xmin[ng - 1], p.grd_ymin[ng - 1], p.grd_zmin[ng - 1]]) * p.re_equiv
    hi = np.array([p.grd_xmax[ng - 1], p.grd_ymax[ng - 1], p.grd_zmax[ng - 1]]) * p.re_equiv
    span = hi - lo
    a = lo + span * np.array([0.03, 0.15 + 0.15 * rng.random(), 0.15 + 0.15 * rng.random()])
    b = lo + span * np.array([0.97, 0.15 + 0.15 * rng.random(), 0.15 + 0.15 * rng.random()])
    t = np.linspace(0.0, 1.0, n)
    xyz = (a[None, :] + t[:, None] * (b - a)[None, :]).astype(np.float32)
    step = (1 + (np.arange(n) * nsteps) // n).astype(np.int32)
    v0 = sample_values(p, state.cur.astype(np.float64), xyz)
    v0[np.isnan(v0)] = 0.0
    target = (v0 * (1.0 + scale * rng.standard_normal(v0.shape))).astype(np.float32)
    return xyz, step, target


def wind_of(state):
    return np.array([getattr(state.params, k) for k in WIND], np.float64)
