"""Writes tests/golden/ref_digests.json: SHA-256 digests of the reference's
own results for every per-routine case of tests/_refcases.py, and of its
main loop on the one-box 61x61x31 grid (20 main steps) and the production
nested grid (5 boxes of 121x121x61, after 1 and 10 main steps).

The results come from the reference's Fortran routines translated to C and
compiled by oracle/fortran_to_c.py (oracle/_ref/libg3m3_ref.so), so this
needs the reference's sources; the digests it writes let the oracle and the
library be checked against the reference where the sources are absent.

    python tests/golden/make_ref_golden.py [--keep-main]
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


# main-loop cases: (name, grid, build with OpenMP, digest after these main
# steps) -- the one-box 61x61x31 grid for 20 steps and the production
# nested grid (5 boxes of 121x121x61) for 10 main steps, no div B pass
MAIN_CASES = [("small", "small", False, [1, 5, 20]), ("nested", "nested", True, [1, 10])]


def main_start(name):
    """The seeded state with the starting copies every side uses: old = 0,
    wrk = cur."""
    from g3m3_gb300.state import make_config
    st = make_config(name, divb_every=0)
    return st, np.zeros_like(st.cur), st.cur.copy()


def main_record(fields, t, t_stepnew, cell_updates):
    return {"fields": [digest(f) for f in fields], "t": float(t),
            "t_stepnew": [float(x) for x in t_stepnew], "cell_updates": int(cell_updates)}


def make_main():
    from oracle.refmain import RefMain
    out = {}
    for name, grid, omp, steps in MAIN_CASES:
        st, old, wrk = main_start(name)
        p = st.params
        rm = RefMain(grid, omp=omp)
        rm.load_state(p, st.cur, old, wrk, st.b0, st.resistive, st.lists, 0.0, np.zeros(p.n_grids))
        rm.init_steps()
        cells = p.nx * p.ny * p.nz
        rec, done, cu = {}, 0, 0
        for n in steps:
            while done < n:
                rm.steps(1)
                cu += sum(rm.box_steps()) * cells
                done += 1
            rec[str(n)] = main_record(rm.fields(), rm.get("t"), rm.array("t_stepnew"), cu)
        out[name] = rec
    return out


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
    if "--keep-main" in sys.argv and os.path.exists(OUT):
        out["main"] = json.load(open(OUT))["main"]   # the main-loop digests take minutes
    else:
        out["main"] = make_main()
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=0, sort_keys=True)
        fh.write("\n")
    print(f"wrote {len(out['cases'])} cases to {OUT}")


if __name__ == "__main__":
    make()
