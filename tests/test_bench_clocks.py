"""bench.py's clock sampler on CPU, against a stand-in `nvidia-smi` on PATH that
prints one CSV sample (SM clock, max clock, reasons bit mask) every 20 ms: the
sampler is live before the timed region starts, keeps the samples that bracket
a region shorter than the sampling period, and names the active reasons."""
import os
import stat
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FAKE = """#!/usr/bin/env python3
import sys, time
i = 0
while True:
    # 1500 MHz with hw_slowdown (0x8) for the first 5 samples, then 2070 MHz with sw_power_cap (0x4)
    line = "1500, 2070, 0x0000000000000008" if i < 5 else "2070, 2070, 0x0000000000000004"
    print(line, flush=True)
    i += 1
    time.sleep(0.02)
"""


def test_clock_sampler_brackets_a_short_region(tmp_path, monkeypatch):
    exe = tmp_path / "nvidia-smi"
    exe.write_text(FAKE)
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ.get("PATH", ""))
    sys.path.insert(0, ROOT)
    import bench

    c = bench.ClockSampler(0)
    c.start()
    assert c.lines, "the sampler is live before the region starts"
    time.sleep(0.5)  # past the slow samples
    t0 = time.perf_counter()
    time.sleep(0.005)  # a region shorter than the sampling period
    t1 = time.perf_counter()
    clk = c.stop(t0, t1)
    assert clk["samples"] >= 2  # one before the region, one after
    assert clk["sm_mhz"] == 2070.0 and clk["sm_max_mhz"] == 2070.0
    assert clk["reasons"] == ["sw_power_cap"]
    assert any(t > t1 for t, _ in c.lines)

    c = bench.ClockSampler(0)
    c.start()
    t0 = time.perf_counter()
    time.sleep(0.05)
    t1 = time.perf_counter()
    clk = c.stop(t0, t1)
    assert "hw_slowdown" in clk["reasons"]
