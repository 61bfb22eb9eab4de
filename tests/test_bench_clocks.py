"""bench.py's clock sampler against a stand-in ``nvidia-smi`` on PATH (a shell script printing the
query's CSV rows every 50 ms): only rows taken after mark() count, throttle reasons are collected
from them, and a missing nvidia-smi gives no clock record.  CPU only."""
import os
import stat
import sys
import time

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402

FAKE = """#!/bin/sh
echo "345, 2070, 90.1, Not Active, Not Active, Not Active, Not Active"
while true; do
  sleep 0.05
  echo "1980, 2070, 900.5, Not Active, Not Active, Not Active, Active"
done
"""


@pytest.fixture
def fake_smi(tmp_path, monkeypatch):
    path = tmp_path / "nvidia-smi"
    path.write_text(FAKE)
    path.chmod(path.stat().st_mode | stat.S_IXUSR)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ.get('PATH', '')}")
    return path


def test_samples_before_the_mark_are_set_aside(fake_smi):
    clk = bench.ClockSampler(0)
    clk.start()
    assert clk.proc is not None and clk._lines()
    clk.mark()
    time.sleep(0.4)
    rec = clk.stop()
    assert rec["samples"] >= 2
    assert rec["sm_mhz"] == 1980.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"]


def test_a_region_without_samples_reports_zero(fake_smi):
    clk = bench.ClockSampler(0)
    clk.start()
    time.sleep(0.2)
    clk.mark()
    clk.proc.kill()                 # no row can arrive after the mark
    clk.proc.wait()
    rec = clk.stop()
    assert rec["samples"] == 0 and rec["sm_mhz"] > 0


def test_no_nvidia_smi_gives_no_record(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    clk = bench.ClockSampler(0)
    clk.start()
    clk.mark()
    assert clk.stop() is None
