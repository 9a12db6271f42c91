"""The reference's own results, as committed digests
(tests/golden/ref_digests.json, written by tests/golden/make_ref_golden.py
from the reference's Fortran routines compiled through
oracle/fortran_to_c.py): the oracle must reproduce them on the CPU, and the
library's drop-in entries on the GPU, without the reference present."""
import json
import os

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
