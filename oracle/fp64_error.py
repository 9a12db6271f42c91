"""Per-field error of the FP32 step against the reference's FP64 build.

TEST INFRASTRUCTURE ONLY.  The reference's own main loop is built with
default REAL in double precision by oracle/fortran_to_c.py (what
``-fdefault-real-8`` gives); the oracle's FP32 main step, which the library
reproduces bit for bit, is run from the same seeded state, and the relative
L2 error ||f32 - f64|| / ||f64|| of every field is printed after the given
numbers of main steps.

    python oracle/fp64_error.py [grid ...]      grids: tiny3 small nested
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

STEPS = {"tiny3": [1, 5, 20], "small": [1, 4, 5, 20], "nested": [1]}


def errors(grid, steps):
    """Yield (main steps, per-field relative L2 errors) for one grid."""
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    from oracle.refmain import RefMain
    st = make_config(grid, divb_every=0)
    om = OracleModel(st, omp=(grid == "nested"))
    r8 = RefMain(grid, omp=(grid == "nested"), real8=True)
    r8.load_state(om.p, om.cur, om.old, om.wrk, om.b0, om.resistive, om.lists, 0.0, np.zeros(om.p.n_grids))
    om.init_steps()
    r8.init_steps()
    done = 0
    for n in steps:
        while done < n:
            assert om.main_step() == 0
            r8.steps(1)
            done += 1
        f64 = r8.fields()
        yield n, [float(np.linalg.norm(om.cur[q].astype(np.float64) - f64[q]) / np.linalg.norm(f64[q]))
                  for q in range(om.cur.shape[0])]


def main(argv):
    from g3m3_gb300.params import FIELD_NAMES
    for grid in argv[1:] or list(STEPS):
        for n, e in errors(grid, STEPS[grid]):
            worst = int(np.argmax(e))
            print(f"{grid} after {n} main step(s): median {np.median(e):.1e}, max {max(e):.1e} ({FIELD_NAMES[worst]})")
            print("   " + " ".join(f"{FIELD_NAMES[q]}:{e[q]:.1e}" for q in range(len(e))))


if __name__ == "__main__":
    main(sys.argv)
