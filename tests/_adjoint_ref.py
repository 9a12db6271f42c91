"""FP64 references for the adjoint tests (TEST INFRASTRUCTURE).

The misfit of a virtual-spacecraft run evaluated with the oracle's FP64
build (every REAL in double precision; tests/test_ref_fp64.py pins it to the
reference's own FP64 build) under a given time-step schedule: the same main
steps the library's adjoint differentiates, so that central differences of
it check the library's gradients.  The samples are g3m3_gb300.adjoint's
(the same positions, weights and fields as the library's loss kernel).
"""
from __future__ import annotations

import numpy as np

WIND = ("srho", "spx", "spy", "spz", "spress", "sbx_wind", "sby_wind", "sbz_wind")


def sample_values(p, cur, xyz):
    from g3m3_gb300.adjoint import sample_state
    return sample_state(p, cur, xyz)


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


def oracle_jvp(state, wind, schedule, samples, wind_tangent=None, state_tangent=None):
    """The misfit and its exact directional derivative along (wind_tangent,
    state_tangent) from the oracle's FP64 build run in forward-mode dual
    numbers (oracle/dual.h) under ``schedule``: the state tangent is added
    after init_steps, where the library's state gradient is taken.  Returns
    (loss, dloss)."""
    import ctypes
    from oracle.oracle import OracleModel
    st = state.copy()
    p = type(state.params)()
    ctypes.memmove(ctypes.addressof(p), ctypes.addressof(state.params), ctypes.sizeof(p))
    st.params = p
    for k, v in zip(WIND, wind):
        setattr(p, k, float(np.float32(v)))
    om = OracleModel(st, omp=True, dual=True)
    om.set_wind_tangent(np.zeros(8) if wind_tangent is None else wind_tangent)
    om.init_steps()
    if state_tangent is not None:
        om.cur.imag[...] += state_tangent
    xyz, step, target = samples
    loss = dloss = 0.0
    for s in range(len(schedule)):
        for b in range(p.n_grids):
            om.s.t_stepnew[b] = float(schedule[s][b])
        assert om.main_step() == 0
        sel = np.nonzero(np.asarray(step) == s + 1)[0]
        if len(sel):
            x = np.asarray(xyz)[sel]
            v = sample_values(p, om.cur.real, x)
            dv = sample_values(p, om.cur.imag, x)
            r = v - np.asarray(target, np.float64)[sel]
            ok = ~np.isnan(r)
            loss += float((r[ok] ** 2).sum())
            dloss += float((2.0 * r[ok] * dv[ok]).sum())
    return loss, dloss


def line_samples(state, nsteps, n=200, seed=20261205, scale=0.1):
    from g3m3_gb300.adjoint import line_samples as ls
    return ls(state, nsteps, n, seed, scale)


def wind_of(state):
    from g3m3_gb300.adjoint import wind_of as wo
    return wo(state.params)
