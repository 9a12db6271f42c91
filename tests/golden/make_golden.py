"""Writes tests/golden/oracle_digests.json: SHA-256 digests of the oracle's
state after 1 and 3 main steps of seeded small grids (one box 17x17x9; three
nested boxes 17x17x9), with the time bookkeeping.

The reference ships no golden data; these digests are made by the oracle,
and tests/test_ref_main.py checks that the reference's own set-up and main
loop (translated and compiled by oracle/fortran_to_c.py) give exactly them,
so the library's GPU test against them is a test against the reference.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = [("tiny", [1, 3]), ("tiny3", [1, 3])]
OUT = os.path.join(HERE, "oracle_digests.json")


def canon(a):
    """FP32 bits with +0/-0 and all NaNs folded (the parity bar treats them equal)."""
    a = np.ascontiguousarray(a, np.float32).copy()
    a[a == 0] = 0.0
    a[np.isnan(a)] = np.float32("nan")
    return a


def digest(a):
    return hashlib.sha256(canon(a).tobytes()).hexdigest()


def input_digest(st):
    return digest(np.concatenate([st.cur.ravel(), st.b0.ravel(), st.resistive.ravel()]))


def field_digests(state):
    return [digest(state[q]) for q in range(state.shape[0])]


def make():
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    out = {"format": "sha256 of little-endian float32, +0/-0 and NaNs folded", "cases": {}}
    for name, steps in CASES:
        st = make_config(name)
        om = OracleModel(st)
        om.init_steps()
        rec = {"input": input_digest(st), "shape": list(st.cur.shape), "steps": {}}
        done = 0
        for n in steps:
            while done < n:
                assert om.main_step() == 0
                done += 1
            rec["steps"][str(n)] = {
                "fields": field_digests(om.cur),
                "t": float(om.s.t),
                "t_stepnew": [float(x) for x in om.t_stepnew],
                "cell_updates": int(om.cell_updates),
            }
        out["cases"][name] = rec
    return out


if __name__ == "__main__":
    with open(OUT, "w") as f:
        json.dump(make(), f, indent=1)
    print("wrote", OUT)
