"""The oracle pinned to the reference itself.

Every routine of the oracle's restatement runs beside the reference's own
Fortran routine -- the reference source translated to C by
oracle/fortran_to_c.py and compiled into oracle/_ref/libg3m3_ref.so -- on
the same seeded inputs (tests/_refcases.py), and the two must agree bitwise
(NaN = NaN, +0 = -0) in every array argument afterwards, inputs included,
and in every returned scalar.  Runs on the CPU; skips where the reference's
sources are absent and the library has not been built (the committed
digests of tests/test_ref_golden.py carry the same pin there).
"""
import numpy as np
import pytest

import _refpin
from _refcases import CASES, run
from _support import assert_same

pytestmark = pytest.mark.skipif(_refpin.load() is None,
                                reason="reference sources absent: oracle/_ref not built")


@pytest.mark.parametrize("cid", [c[0] for c in CASES])
def test_oracle_matches_reference(cid):
    ref = run(cid, "ref")
    orc = run(cid, "oracle")
    assert sorted(ref) == sorted(orc)
    for k in ref:
        assert_same(np.asarray(orc[k]), np.asarray(ref[k]), f"{cid} {k}")
