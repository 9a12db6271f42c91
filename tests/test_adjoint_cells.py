"""The generated per-cell reverse sweeps (g3m3_gb300/csrc/adj_cells.cuh).

* The committed header is what g3m3_gb300/adgen.py makes from
  g3m3_gb300/adcells.py today (no hand edits, no stale copy).
* Built for double on the host, every cell's reverse gives the gradient of
  <w, f(x)> that central differences of its forward give, for random
  inputs and weights (tests/adjcheck/check_cells.cpp): both skin-depth
  branches of push_ion, and the flux limiter's branches over 200 draws.
  The bar, 1e-3 relative per input, covers components whose gradient is
  near zero, where FD round-off (about 1e-10 absolute) dominates.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TOL = 1e-3


def test_generated_header_is_current(tmp_path):
    from g3m3_gb300 import adgen
    out = tmp_path / "adj_cells.cuh"
    adgen.generate(str(out))
    committed = open(os.path.join(ROOT, "g3m3_gb300", "csrc", "adj_cells.cuh")).read()
    assert out.read_text() == committed


def test_cell_reverses_match_central_differences(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "check_cells"
    subprocess.run([gxx, "-O1", "-std=c++17", "-o", str(exe), os.path.join(HERE, "adjcheck", "check_cells.cpp")],
                   check=True)
    res = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    rows = [r.split() for r in res if r.strip()]
    names = {r[0] for r in rows}
    assert {"push_ion_cell", "push_ion_cell_strongB", "push_elec_cell", "push_bfld_cell", "curl_cell",
            "total_b_cell", "evel_cell", "vtot_cell", "bande_cell", "lap_speed_cell", "lap_jump_cell",
            "lap_field_cell", "fcs_flux_cell"} <= names
    bad = [(n, float(e)) for n, e in rows if not float(e) <= TOL]
    assert not bad, bad
