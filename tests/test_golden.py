"""Committed golden digests (tests/golden/oracle_digests.json, written by
tests/golden/make_golden.py): the oracle must keep reproducing them (CPU),
and the library must reproduce them on the GPU without the oracle running."""
import json
import os

import numpy as np
import pytest

import _support  # noqa: F401  (puts the repository root on sys.path)

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "oracle_digests.json")))


def _golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _check(name, n, fields, t, tsn, cu):
    rec = GOLDEN["cases"][name]["steps"][str(n)]
    bad = [q for q in range(len(fields)) if fields[q] != rec["fields"][q]]
    assert not bad, f"{name} after {n} step(s): fields {bad} differ from the committed digests"
    assert t == rec["t"]
    assert list(tsn) == rec["t_stepnew"]
    assert cu == rec["cell_updates"]


@pytest.mark.parametrize("name", sorted(GOLDEN["cases"]))
def test_inputs_match_fixture(name):
    from g3m3_gb300.state import make_config
    g = _golden()
    assert g.input_digest(make_config(name)) == GOLDEN["cases"][name]["input"]


@pytest.mark.parametrize("name", sorted(GOLDEN["cases"]))
def test_oracle_reproduces_golden(name):
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    g = _golden()
    om = OracleModel(make_config(name))
    om.init_steps()
    done = 0
    for n in sorted(int(k) for k in GOLDEN["cases"][name]["steps"]):
        while done < n:
            assert om.main_step() == 0
            done += 1
        _check(name, n, g.field_digests(om.cur), float(om.s.t), [float(x) for x in om.t_stepnew],
               int(om.cell_updates))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GOLDEN["cases"]))
@pytest.mark.parametrize("graph", [False, True])
def test_library_reproduces_golden(name, graph):
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    g = _golden()
    st = make_config(name)
    assert g.input_digest(st) == GOLDEN["cases"][name]["input"], "seeded inputs differ on this machine"
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        done = 0
        for n in sorted(int(k) for k in GOLDEN["cases"][name]["steps"]):
            m.run(n - done, graph=graph)
            done = n
            t, tsn, cu = m.times()
            _check(name, n, g.field_digests(m.state()), float(t), [float(x) for x in np.asarray(tsn)],
                   int(cu))
        m.close()
