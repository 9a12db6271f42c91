"""Writes tests/golden/ref_digests.json: SHA-256 digests of the reference's
own results for every per-routine case of tests/_refcases.py.

The results come from the reference's Fortran routines translated to C and
compiled by oracle/fortran_to_c.py (oracle/_ref/libg3m3_ref.so), so this
needs the reference's sources; the digests it writes let the oracle and the
library be checked against the reference where the sources are absent.

    python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

OUT = os.path.join(HERE, "ref_digests.json")


def digest(a):
    """FP32 bits with +0/-0 and all NaNs folded (the parity bar treats them
    equal); other types as their raw bytes."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = a.copy()
        a[a == 0] = 0.0
        a[np.isnan(a)] = np.float32("nan")
    return hashlib.sha256(a.tobytes()).hexdigest()


def digests(results):
    return {k: digest(np.asarray(v)) for k, v in sorted(results.items())}


def make():
    import _refpin
    from _refcases import CASES, run
    from g3m3_gb300.state import make_config
    from golden.make_golden import input_digest
    if _refpin.load() is None:
        raise SystemExit("the reference's sources are needed (oracle/_ref could not be built)")
    out = {"about": "digests of the reference's own routine results (oracle/fortran_to_c.py); "
                    "cases in tests/_refcases.py",
           "inputs": {n: input_digest(make_config(n)) for n in ("tiny2", "tiny3", "small")},
           "cases": {}}
    for cid, fn, kw, _ in CASES:
        out["cases"][cid] = digests(run(cid, "ref"))
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=0, sort_keys=True)
        fh.write("\n")
    print(f"wrote {len(out['cases'])} cases to {OUT}")


if __name__ == "__main__":
    make()
