"""The contracted flavour of the push kernels (g3m3_model_set_contracted:
FMA contraction, reciprocal products for shared denominators) against the
reference's FP32 bits and the FP64 build.

Per main step (from the same state): every field within 1e-5 relative L2
of the reference's FP32 step on the benchmark's nested grid, and on every
grid at most 1.5 times as far from the FP64 build as the reference's FP32
build is (plus 1e-7).  Measured (GB300): 8.3e-6 at most on the nested grid
(median 4.8e-8); the distances to FP64 within 1.43 times the FP32 build's.
"""
import numpy as np
import pytest

from _divb_parity import rel

pytestmark = pytest.mark.gpu


def _compare(grid, steps):
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    st = make_config(grid, divb_every=0)
    o32 = OracleModel(st, omp=True)
    o64 = OracleModel(st, omp=True, real8=True)
    o32.init_steps()
    o64.init_steps()
    out = {}
    with Context() as ctx:
        m = Model(ctx, st)
        ctx.check(m.L.g3m3_model_set_contracted(m.h, 1))
        m.init_steps()
        done = 0
        for n in steps:
            while done < n:
                m.run(1, graph=False)
                assert o32.main_step() == 0
                assert o64.main_step() == 0
                done += 1
            g = m.state()
            out[n] = [(rel(g[q], o32.cur[q]), rel(g[q], o64.cur[q]), rel(o32.cur[q], o64.cur[q])) for q in range(34)]
        m.close()
    return out


@pytest.mark.parametrize("grid,steps,bar", [("nested", [1], 1e-5), ("small", [1, 5], None), ("mid3", [1, 3], None)])
def test_contracted_flavour_accuracy(grid, steps, bar):
    out = _compare(grid, steps)
    for n, rows in out.items():
        e32 = np.array([r[0] for r in rows])
        if bar is not None and n == 1:
            assert e32.max() <= bar, (grid, n, e32.max(), int(np.argmax(e32)))
        for q, (_, e64, r64) in enumerate(rows):
            assert e64 <= 1.5 * r64 + 1e-7, (grid, n, q, e64, r64)
