"""bench.py's clock sampler on CPU, against a stand-in nvidia-smi that prints
the CSV the real one prints for the sampler's query (index, clocks.sm,
clocks.max.sm, power.draw, active reasons bitmask, then the four throttle
reasons as Active / Not Active)."""
import os
import stat
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

FAKE = """#!/bin/sh
echo "0, 2070, 2070, 812.50, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
echo "0, 2055, 2070, 1391.20, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
echo "0, 2070, 2070, 1380.00, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
exec sleep 30
"""


def _with_fake_smi(tmp_path, monkeypatch, script):
    p = tmp_path / "nvidia-smi"
    p.write_text(script)
    p.chmod(p.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ.get("PATH", ""))


def test_clock_sampler_parses_samples_and_reasons(tmp_path, monkeypatch):
    _with_fake_smi(tmp_path, monkeypatch, FAKE)
    clk = bench.ClockSampler(0)
    clk.start()
    time.sleep(0.5)
    out = clk.stop()
    assert out["samples"] == 3
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))   # an empty directory: no nvidia-smi
    clk = bench.ClockSampler(0)
    clk.start()
    out = clk.stop()
    assert out["sm_mhz"] is None and out["reasons"] == ["nvidia-smi unavailable"]
