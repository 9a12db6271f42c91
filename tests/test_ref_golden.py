"""The reference's own results, as committed digests
(tests/golden/ref_digests.json, written by tests/golden/make_ref_golden.py
from the reference's Fortran routines compiled through
oracle/fortran_to_c.py): the oracle must reproduce them on the CPU, and the
library's drop-in entries on the GPU, without the reference present."""
import json
import os

import numpy as np
import pytest

import _support  # noqa: F401  (puts the repository root on sys.path)
from _refcases import CASES, run
from golden.make_ref_golden import digests

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "ref_digests.json")))


def _check(cid, results):
    want = GOLDEN["cases"][cid]
    got = digests(results)
    assert sorted(got) == sorted(want), (cid, sorted(got), sorted(want))
    bad = [k for k in want if got[k] != want[k]]
    assert not bad, f"{cid}: {bad} differ from the reference's results"


def test_inputs_match_fixture():
    from g3m3_gb300.state import make_config
    from golden.make_golden import input_digest
    for name, d in GOLDEN["inputs"].items():
        assert input_digest(make_config(name)) == d, f"seeded inputs {name} differ on this machine"


@pytest.mark.parametrize("cid", [c[0] for c in CASES])
def test_oracle_reproduces_reference(cid):
    _check(cid, run(cid, "oracle"))


@pytest.mark.gpu
@pytest.mark.parametrize("cid", [c[0] for c in CASES if c[3]])
def test_library_reproduces_reference(cid):
    _check(cid, run(cid, "gpu"))


def _main_check(name, n, fields, t, t_stepnew, cell_updates):
    want = GOLDEN["main"][name][str(n)]
    got = [digest_of(f) for f in fields]
    bad = [q for q in range(len(want["fields"])) if got[q] != want["fields"][q]]
    assert not bad, f"{name}: fields {bad} after {n} main step(s) differ from the reference's"
    assert float(t) == want["t"]
    assert [float(x) for x in t_stepnew] == want["t_stepnew"]
    assert int(cell_updates) == want["cell_updates"]


def digest_of(a):
    from golden.make_ref_golden import digest
    return digest(a)


@pytest.mark.parametrize("name", sorted(GOLDEN["main"]))
def test_oracle_main_loop_reproduces_reference(name):
    """The reference's main loop on the one-box 61x61x31 grid (20 steps) and
    on the production nested grid (its first main step): the oracle's steps
    give its digests."""
    from golden.make_ref_golden import main_start
    from oracle.oracle import OracleModel
    st, old, wrk = main_start(name)
    om = OracleModel(st, omp=True)
    assert np.array_equal(om.old, old) and np.array_equal(om.wrk, wrk)
    om.init_steps()
    done = 0
    steps = sorted(int(k) for k in GOLDEN["main"][name])
    if name == "nested":
        steps = steps[:1]      # one production main step takes the CPU about 10 s; the GPU test runs all
    for n in steps:
        while done < n:
            assert om.main_step() == 0
            done += 1
        _main_check(name, n, om.cur, om.s.t, om.t_stepnew, om.cell_updates)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GOLDEN["main"]))
@pytest.mark.parametrize("graph", [False, True])
def test_library_main_loop_reproduces_reference(name, graph):
    """The step engine on the same grids, from the same seeded state, gives
    the reference's digests without the oracle running."""
    from g3m3_gb300.api import Context, Model
    from golden.make_ref_golden import main_start
    st, _, _ = main_start(name)
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        done = 0
        for n in sorted(int(k) for k in GOLDEN["main"][name]):
            m.run(n - done, graph=graph)
            done = n
            t, tsn, cu = m.times()
            _main_check(name, n, m.state(), t, np.asarray(tsn), cu)
        m.close()
