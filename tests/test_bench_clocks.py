"""bench.py's clock record, against a fake nvidia-smi on PATH (no GPU): only
samples taken after the sampler's start() returned are counted, the median
SM clock and the throttle reasons come from them."""
from __future__ import annotations

import os
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

FAKE = """#!/bin/bash
sleep 0.3
echo "0, 1000, 2070, 300.0, 0x0, Not Active, Active, Not Active, Not Active"
while true; do
  echo "0, 2070, 2070, 900.0, 0x4, Not Active, Not Active, Not Active, Active"
  sleep 0.05
done
"""


@pytest.fixture
def fake_smi(tmp_path, monkeypatch):
    exe = tmp_path / "nvidia-smi"
    exe.write_text(FAKE)
    exe.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    return exe


def test_samples_start_with_the_timed_region(fake_smi):
    import bench
    c = bench.Clocks(0)
    t0 = time.time()
    c.start()
    assert time.time() - t0 >= 0.25          # waited for the first sample
    time.sleep(0.3)
    rec = c.stop()
    assert rec["samples"] >= 2
    # the first sample (before start() returned) is not counted
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"]


def test_no_sampler(monkeypatch, tmp_path):
    import bench
    monkeypatch.setenv("PATH", str(tmp_path))   # no nvidia-smi at all
    c = bench.Clocks(0)
    c.start()
    rec = c.stop()
    assert rec == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
