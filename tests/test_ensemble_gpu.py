"""Ensembles: members of different box sizes and upstream conditions
advanced together (one CUDA graph per main step, one member at a time from
the host loop, all members at once on their own streams, or every member's
own step graph at once on its own stream) give, member by member, the
oracle's bits."""
import numpy as np
import pytest

from _support import assert_same

pytestmark = pytest.mark.gpu

LIMITS = (8, 10, 12)   # boxes of 17x17x9, 21x21x11, 25x25x13


def _members(n=3):
    from g3m3_gb300.state import ensemble_member
    return [ensemble_member(i, n_grids=2, limits=LIMITS) for i in range(n)]


@pytest.mark.parametrize("mode", ["graph", "sequential", "streams", "member_graphs"])
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
        ens.run(nsteps, graph=mode in ("graph", "member_graphs"), concurrent=mode in ("streams", "member_graphs"))
        k, g, cu = ens.stats()
        outs = [m.state() for m in ens.members]
        times = [m.times() for m in ens.members]
        ens.close()
    assert k > 0
    assert g == {"graph": nsteps, "member_graphs": nsteps * len(states)}.get(mode, 0)
    assert cu == sum(om.cell_updates for om in oms)
    for i, (om, out, (t, tsn, _)) in enumerate(zip(oms, outs, times)):
        for q in range(34):
            assert_same(out[q], om.cur[q], f"member {i} field {q}")
        assert np.array_equal(tsn, om.t_stepnew)
        assert t == om.s.t


@pytest.mark.parametrize("mode", ["streams", "member_graphs"])
def test_ensemble_divb_inside_steps(mode):
    """Members whose div B pass falls due together run their passes side by
    side (every member's boxes at once): fields div B does not touch are the
    oracle's bits, B is within the CG tolerance of the oracle's cleaning."""
    from g3m3_gb300.api import Context, Ensemble
    from g3m3_gb300.state import ensemble_member
    from oracle.oracle import OracleModel
    from _support import rel_l2
    states = [ensemble_member(i, n_grids=2, limits=LIMITS, divb_every=2, divb_errlim=1e-5) for i in range(3)]
    plain = [ensemble_member(i, n_grids=2, limits=LIMITS, divb_every=0, divb_errlim=1e-5) for i in range(3)]
    nsteps = 2
    oms, befores = [], []
    for st, st0 in zip(states, plain):
        om, o0 = OracleModel(st, omp=True), OracleModel(st0, omp=True)
        om.init_steps()
        o0.init_steps()
        for _ in range(nsteps):
            assert om.main_step() == 0
            assert o0.main_step() == 0
        oms.append(om)
        befores.append(o0.cur)
    with Context() as ctx:
        ens = Ensemble(ctx, states)
        ens.init_steps()
        ens.run(nsteps, graph=mode == "member_graphs", concurrent=True)
        outs = [m.state() for m in ens.members]
        ens.close()
    for i, (om, before, out) in enumerate(zip(oms, befores, outs)):
        for q in range(31):
            assert_same(out[q], om.cur[q], f"member {i} field {q}")
        for q in (31, 32, 33):
            assert rel_l2(out[q] - before[q], om.cur[q] - before[q]) < 0.2


def test_ensemble_autotune_per_box_size():
    """One flux-correction form chosen per distinct box size and shared by
    the members of that size; the members still give the oracle's bits."""
    from g3m3_gb300.api import Context, Ensemble
    from oracle.oracle import OracleModel
    from g3m3_gb300.state import ensemble_member
    states = [ensemble_member(i, n_grids=2, limits=LIMITS) for i in range(4)]   # sizes 17, 21, 25, 17
    with Context() as ctx:
        ens = Ensemble(ctx, states)
        chosen = ens.autotune()
        assert sorted(chosen) == sorted({(s.params.nx, s.params.ny, s.params.nz) for s in states})
        assert all(v in range(8) for v in chosen.values())
        ens.init_steps()
        ens.run(2, graph=True)
        outs = [m.state() for m in ens.members]
    for st, g in zip(states, outs):
        om = OracleModel(st, omp=True)
        om.init_steps()
        for _ in range(2):
            assert om.main_step() == 0
        for q in range(34):
            assert_same(g[q], om.cur[q], f"member field {q}")


def test_ensemble_bench_sizes_one_step():
    """The bench's ensemble shapes: three members of five nested boxes of
    121x121x61, 97x97x49 and 81x81x41 with upstream conditions drawn from
    the seed, the flux-correction forms the autotuner picks for those sizes
    (7, 5, 7), one main step in one CUDA graph: every member's 34 fields are
    the oracle's bits."""
    from g3m3_gb300.api import Context, Ensemble
    from g3m3_gb300.state import ensemble_member
    from oracle.oracle import OracleModel
    states = [ensemble_member(i) for i in range(3)]
    assert [s.params.nx for s in states] == [121, 97, 81]
    with Context() as ctx:
        ens = Ensemble(ctx, states)
        for m, v in zip(ens.members, (7, 5, 7)):
            m.set_variant(1, v)
        ens.init_steps()
        ens.run(1, graph=True)
        outs = [m.state() for m in ens.members]
        ens.close()
    for i, (st, out) in enumerate(zip(states, outs)):
        om = OracleModel(st, omp=True)
        om.init_steps()
        assert om.main_step() == 0
        for q in range(34):
            assert_same(out[q], om.cur[q], f"member {i} field {q}")
