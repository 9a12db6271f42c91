"""Per-field distance of three runs of the same main steps with the div B
pass at its configured cadence, against the oracle's FP64 build (every REAL
in double precision; it agrees with the reference's own FP64 build to about
1e-8 relative per field, tests/test_ref_fp64.py):

* ``ref32``: the oracle's FP32 main loop, the reference's FP32 bits
  (FP32 dot products in the CG, as the reference computes them);
* ``gpu``: the library's step engine (FP32 state, FP64 CG dot products).

The engine reproduces ``ref32`` bit for bit until the first div B pass; a
pass changes only B, so right after it the other 31 fields must still be
equal bit for bit.  After it the runs drift apart through B.  The bar
(``check``): for every field, the engine's distance from the FP64 run is at
most SLACK times the reference FP32 build's own distance plus FLOOR -- the
FP64 dot products make the solve at least as good as the reference's, up
to the spread of runs that stop a loosely converged CG at different
iterates.  TEST INFRASTRUCTURE.
"""
from __future__ import annotations

import numpy as np

SLACK = 2.0
FLOOR = 1e-6


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def run(grid, steps, graph=True, omp=True):
    """{n: (gpu, ref32, ref64 states after n main steps)} and the bitwise
    flags of the non-B fields right after the first div B pass."""
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel

    st = make_config(grid)
    every = st.params.divb_every
    assert every > 0
    o32 = OracleModel(st, omp=omp)
    o64 = OracleModel(st, omp=omp, real8=True)
    o32.init_steps()
    o64.init_steps()
    out = {}
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        done = 0
        for n in sorted(set(steps) | {every}):
            while done < n:
                m.run(1, graph=graph)
                assert o32.main_step() == 0
                assert o64.main_step() == 0
                done += 1
            out[n] = (m.state().copy(), o32.cur.copy(), o64.cur.copy())
        m.close()
    return out, every


def table(out):
    """{n: [(field, e_gpu, e_ref32)]} distances from the FP64 run."""
    from g3m3_gb300.params import FIELD_NAMES
    res = {}
    for n, (g, r32, r64) in out.items():
        res[n] = [(FIELD_NAMES[q], rel(g[q], r64[q]), rel(r32[q], r64[q])) for q in range(g.shape[0])]
    return res


def check(res):
    bad = []
    for n, rows in res.items():
        for name, eg, er in rows:
            if not eg <= SLACK * er + FLOOR:
                bad.append((n, name, eg, er))
    return bad


def divb_correct_r8(nx, ny, nz, n_grids, box, pos, xspac, errlim, bx, by, bz):
    """oracle_divb_correct of the FP64 build on float64 copies of bx, by, bz
    (returned, with the iteration count)."""
    import ctypes
    from oracle.oracle import lib
    L = lib(real8=True)
    fn = L.oracle_divb_correct
    fn.restype = ctypes.c_int
    b = [np.ascontiguousarray(x, np.float64).copy() for x in (bx, by, bz)]
    xs = np.ascontiguousarray(xspac, np.float64)
    vp = ctypes.c_void_p
    fn.argtypes = [ctypes.c_int] * 6 + [vp, vp, ctypes.c_double, vp, vp, vp]
    it = fn(nx, ny, nz, n_grids, box, 7, ctypes.addressof(pos), xs.ctypes.data, float(errlim),
            b[0].ctypes.data, b[1].ctypes.data, b[2].ctypes.data)
    return b, it


def divb_all_r8(state):
    """The div B pass of every box (divb_all) in the FP64 build: float64 state."""
    from oracle.oracle import OracleModel
    om = OracleModel(state, real8=True)
    om.divb_all()
    return om.cur
