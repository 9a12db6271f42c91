"""The oracle's main step pinned to the reference's own main loop.

The reference's time-step set-up and the body of its time loop
(code/3d_main.f90, ``do while(t.lt.tmax)``), translated to C with every
routine they call by oracle/fortran_to_c.py, run from a seeded state; the
oracle's set-up and main step must give the same fields,
time and next time steps bitwise -- on one box and on three nested,
sub-cycled boxes, with and without the div B pass that the reference runs
at a fluid-file time (FP32 dot products on both sides).  Runs on the CPU;
skips where the reference's sources are absent.
"""
import numpy as np
import pytest

import _refpin
from _support import assert_same, same_bits

pytestmark = pytest.mark.skipif(_refpin.load() is None,
                                reason="reference sources absent: oracle/_ref not built")


def _pair(cfg, divb_at):
    """The seeded state in both, after each side's time-step set-up (which
    must agree too)."""
    from oracle.refmain import RefMain
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    om = OracleModel(make_config(cfg))
    rm = RefMain(cfg)
    rm.load_state(om.p, om.cur, om.old, om.wrk, om.b0, om.resistive, om.lists, om.s.t,
                  np.zeros(om.p.n_grids), divb_at=divb_at)
    om.init_steps()
    rm.init_steps()
    _compare(om, rm, f"{cfg} after the time-step set-up")
    return om, rm


def _compare(om, rm, what):
    got = rm.fields()
    for q in range(34):
        assert_same(om.cur[q], got[q], f"{what}: field {q}")
    assert om.s.t == rm.get("t"), what
    assert_same(om.t_stepnew, rm.array("t_stepnew"), f"{what}: t_stepnew")


@pytest.mark.parametrize("cfg,nsteps", [("tiny", 1), ("tiny", 4), ("tiny3", 1), ("tiny3", 3)])
def test_main_steps(cfg, nsteps):
    om, rm = _pair(cfg, None)
    start = om.cur.copy()
    cells = om.p.nx * om.p.ny * om.p.nz
    for _ in range(nsteps):
        cu = om.cell_updates
        assert om.main_step() == 0
        rm.steps(1)
        # the cell-update count the benchmark derives from the reference's schedule
        assert sum(rm.box_steps()) * cells == om.cell_updates - cu
    assert (~same_bits(rm.fields(), start)).sum() > 0.5 * start.size   # the state moved
    _compare(om, rm, f"{cfg} after {nsteps} step(s)")


@pytest.mark.parametrize("cfg,nsteps,divb_step", [("tiny", 1, 1), ("tiny3", 2, 2)])
def test_main_steps_with_divb(cfg, nsteps, divb_step):
    """The div B pass of the main step in which t reaches the fluid-file time."""
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    probe = OracleModel(make_config(cfg))
    probe.init_steps()
    for _ in range(divb_step):
        probe.main_step()
    om, rm = _pair(cfg, divb_at=probe.s.t)
    for n in range(1, nsteps + 1):
        assert om.main_step() == 0
        if n == divb_step:
            om.divb_all()
    rm.steps(nsteps)
    _compare(om, rm, f"{cfg} after {nsteps} step(s), div B in step {divb_step}")


def test_pin_detects_a_change():
    """A one-ulp change in one cell of the reference's input shows up."""
    om, rm = _pair("tiny3", None)
    a = rm.array("hpresx")
    a[1, 4, 6, 7] = np.nextafter(a[1, 4, 6, 7], np.float32(np.inf))
    om.main_step()
    rm.steps(1)
    got = rm.fields()
    assert any(not same_bits(om.cur[q], got[q]).all() for q in range(34))


@pytest.mark.parametrize("cfg", ["tiny", "tiny3"])
def test_reference_reproduces_committed_digests(cfg):
    """The committed golden digests (tests/golden/oracle_digests.json, which
    the library must reproduce on the GPU) are the reference's own results:
    its set-up and main loop from the same seeded state give them."""
    import json
    import os
    from oracle.refmain import RefMain
    from g3m3_gb300.state import make_config
    from golden.make_golden import field_digests, input_digest
    from oracle.oracle import OracleModel
    here = os.path.dirname(os.path.abspath(__file__))
    rec = json.load(open(os.path.join(here, "golden", "oracle_digests.json")))["cases"][cfg]
    st = make_config(cfg)
    assert input_digest(st) == rec["input"]
    om = OracleModel(st)        # only for its starting copies: old = 0, wrk = cur
    rm = RefMain(cfg)
    rm.load_state(om.p, om.cur, om.old, om.wrk, om.b0, om.resistive, om.lists, 0.0, np.zeros(om.p.n_grids))
    rm.init_steps()
    done = 0
    for n in sorted(int(k) for k in rec["steps"]):
        rm.steps(n - done)
        done = n
        want = rec["steps"][str(n)]
        assert field_digests(rm.fields()) == want["fields"], f"{cfg}: fields after {n} step(s)"
        assert rm.get("t") == want["t"]
        assert [float(x) for x in rm.array("t_stepnew")] == want["t_stepnew"]


def test_openmp_build_matches_serial():
    """The reference's OpenMP loops, with the temporaries of each parallel
    loop private (its iterations are independent), give the serial
    reference's bits; this build times the reference on all host cores."""
    import os
    import subprocess
    import sys
    code = r'''
import sys, numpy as np
sys.path[:0] = [sys.argv[2], sys.argv[1]]
from oracle.refmain import RefMain
from g3m3_gb300.state import make_config
from oracle.oracle import OracleModel
om = OracleModel(make_config("tiny3"))
out = []
for omp in (False, True):
    rm = RefMain("tiny3", omp=omp)
    rm.load_state(om.p, om.cur, om.old, om.wrk, om.b0, om.resistive, om.lists, 0.0, np.zeros(3))
    rm.init_steps()
    rm.steps(2)
    out.append(rm.fields().copy())
a, b = out
same = (a == b) | (np.isnan(a) & np.isnan(b))
print("SAME" if same.all() else "DIFF %d" % (~same).sum())
'''
    here = os.path.dirname(os.path.abspath(__file__))
    env = dict(os.environ, OMP_NUM_THREADS="4")
    r = subprocess.run([sys.executable, "-c", code, here, os.path.dirname(here)], env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("SAME"), r.stdout[-500:]


def test_fluid_file_matches_reference_writer(tmp_path):
    """The fluid (restart) file the reference's main loop writes at a
    fluid-file time (3d_main.f90:3305-3349: unformatted records of t, the 34
    fields, b0 and the inner-boundary lists) equals, byte for byte, what
    g3m3_fluid_write makes of the same state."""
    import ctypes
    import os
    from g3m3_gb300 import _lib
    from g3m3_gb300.api import addr
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    probe = OracleModel(make_config("tiny3"))
    probe.init_steps()
    probe.main_step()
    om, rm = _pair("tiny3", divb_at=probe.s.t)
    rm.set(divb_lores=0)           # the file only: no div B pass after it
    rm.set_unit_dir(str(tmp_path))
    rm.steps(1)
    om.main_step()
    _compare(om, rm, "tiny3 after the step that writes the file")
    ref = open(os.path.join(str(tmp_path), "fort.11"), "rb").read()
    li = {k: np.ascontiguousarray(v) for k, v in om.lists.items()}
    path = str(tmp_path / "ours")
    L = _lib.load()
    rc = L.g3m3_fluid_write(None, path.encode(), ctypes.byref(om.p), ctypes.c_double(om.s.t), addr(om.cur),
                            addr(om.b0), addr(li["parm_srf"]), addr(li["parm_mid"]), addr(li["parm_zero"]),
                            addr(li["ijzero"]), addr(li["numzero"]), addr(li["ijmid"]), addr(li["nummid"]),
                            addr(li["ijsrf"]), addr(li["numsrf"]), li["ijsrf"].shape[0], li["ijmid"].shape[0],
                            li["ijzero"].shape[0])
    assert rc == 0
    ours = open(path, "rb").read()
    assert len(ours) == len(ref)
    assert ours == ref
