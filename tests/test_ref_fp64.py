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
