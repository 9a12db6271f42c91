"""Ensembles: members of different box sizes and upstream conditions
advanced together (one CUDA graph per main step, one member at a time from
the host loop, or all members at once on their own streams) give, member by
member, the oracle's bits."""
import numpy as np
import pytest

from _support import assert_same

pytestmark = pytest.mark.gpu

LIMITS = (8, 10, 12)   # boxes of 17x17x9, 21x21x11, 25x25x13


def _members(n=3):
    from g3m3_gb300.state import ensemble_member
    return [ensemble_member(i, n_grids=2, limits=LIMITS) for i in range(n)]


@pytest.mark.parametrize("mode", ["graph", "sequential", "streams"])
def test_ensemble_matches_oracle(mode):
    from g3m3_gb300.api import Context, Ensemble
    from oracle.oracle import OracleModel
    states = _members()
    nsteps = 2
    oms = []
    for st in states:
        om = OracleModel(st, omp=True)
        om.init_steps()
        for _ in range(nsteps):
            assert om.main_step() == 0
        oms.append(om)
    with Context() as ctx:
        ens = Ensemble(ctx, states)
        ens.init_steps()
        graph = mode == "graph"
        ens.run(nsteps, graph=graph, concurrent=mode == "streams")
        k, g, cu = ens.stats()
        outs = [m.state() for m in ens.members]
        times = [m.times() for m in ens.members]
        ens.close()
    assert k > 0
    assert g == (nsteps if graph else 0)
    assert cu == sum(om.cell_updates for om in oms)
    for i, (om, out, (t, tsn, _)) in enumerate(zip(oms, outs, times)):
        for q in range(34):
            assert_same(out[q], om.cur[q], f"member {i} field {q}")
        assert np.array_equal(tsn, om.t_stepnew)
        assert t == om.s.t
