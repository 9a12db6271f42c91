"""A box larger than any of the benchmark's: one 321x321x161 box (16.6 M
cells, 2.3 GB per state copy), one main step of the step engine against
the oracle's main loop, bitwise (host-launched and graph-replayed).  The
grids of every kernel, the tile counts of the staged kernels and the
index arithmetic all run at 18.6 times the cells of a 121x121x61 box."""
import pytest

from _support import assert_same

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("graph", [False, True])
def test_large_box_one_step(graph):
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    st = make_config("small", limit=160, divb_every=0)
    om = OracleModel(st, omp=True)
    om.init_steps()
    assert om.main_step() == 0
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        m.run(1, graph=graph)
        g = m.state()
        t, tsn, cu = m.times()
        m.close()
    assert cu == om.cell_updates
    for q in range(34):
        assert_same(g[q], om.cur[q], f"field {q}")
