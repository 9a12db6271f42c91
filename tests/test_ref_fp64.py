"""The FP32 step against the reference's FP64 build (its own main loop with
default REAL in double precision, oracle/fortran_to_c.py).

Stated tolerance: relative L2 error ||f32 - f64|| / ||f64|| of every field
<= 2e-4 after 1 and 20 main steps on three nested 17x17x9 boxes and on the
one-box 61x61x31 grid (measured: at most 7.2e-5 and 1.2e-4 on the nested
boxes, 1.4e-5 and 7.0e-5 on the one box; the production nested grid of five
121x121x61 boxes gives at most 5.9e-5 after one main step, see
oracle/fp64_error.py).  The library equals the reference's FP32 build bit
for bit, so this is also the library's error against FP64.
"""
import pytest

import _refpin
from oracle.fp64_error import errors

pytestmark = pytest.mark.skipif(_refpin.load() is None,
                                reason="reference sources absent: oracle/_ref not built")


@pytest.mark.parametrize("grid", ["tiny3", "small"])
def test_fp32_error_against_fp64_reference(grid):
    for n, e in errors(grid, [1, 20]):
        assert max(e) <= 2e-4, (grid, n, max(e))


@pytest.mark.parametrize("grid,nsteps", [("tiny3", 5), ("small", 3)])
def test_fp64_oracle_against_fp64_reference(grid, nsteps):
    """The oracle's FP64 build (oracle/real8.h), which the div B parity
    tests use as the FP64 run, against the reference's own FP64 build: the
    same main steps to 1e-6 relative L2 per field (measured: median 3e-10,
    largest 6e-8; the FP32 literals of the restatement keep their FP32
    values, which the reference's FP64 build widens)."""
    import numpy as np
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    from oracle.refmain import RefMain
    st = make_config(grid, divb_every=0)
    om = OracleModel(st, real8=True)
    r8 = RefMain(grid, real8=True)
    r8.load_state(om.p, st.cur, np.zeros_like(st.cur), st.cur.copy(), st.b0, st.resistive, om.lists, 0.0,
                  np.zeros(om.p.n_grids))
    om.init_steps()
    r8.init_steps()
    for _ in range(nsteps):
        assert om.main_step() == 0
        r8.steps(1)
    f = r8.fields()
    for q in range(f.shape[0]):
        e = np.linalg.norm(om.cur[q] - f[q]) / np.linalg.norm(f[q])
        assert e < 1e-6, (grid, q, e)
