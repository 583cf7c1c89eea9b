"""bench.py's clock sampler on CPU, against a stand-in nvidia-smi on PATH that
prints the queried CSV fields every 20 ms."""
import os
import stat
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FAKE = """#!/bin/sh
sleep 0.2
while true; do
  echo "0, 1980, 2070, 900.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
  sleep 0.02
done
"""


def test_sampler_records_clocks_and_reasons(tmp_path, monkeypatch):
    fake = tmp_path / "nvidia-smi"
    fake.write_text(FAKE)
    fake.chmod(fake.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    sys.path.insert(0, ROOT)
    import bench
    with bench.ClockSampler(0) as clk:
        assert clk.lines, "the sampler returns only once the first sample has arrived"
        time.sleep(0.2)
    s = clk.summary()
    assert s["sm_mhz"] == 1980.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] >= 3


def test_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))  # no nvidia-smi anywhere
    sys.path.insert(0, ROOT)
    import bench
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
