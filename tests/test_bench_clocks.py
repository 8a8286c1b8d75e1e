"""CPU: the benchmark's clock record keeps the nvidia-smi samples taken inside
the timed region (host wall clock), with the throttle reasons seen there;
a region shorter than the sampling period falls back to the nearest
samples. Fed a synthetic capture in nvidia-smi's csv,noheader,nounits form."""
from __future__ import annotations

import datetime
import os
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def capture(lines):
    import bench
    fd, path = tempfile.mkstemp(suffix=".csv")
    with os.fdopen(fd, "w") as f:
        f.write("\n".join(lines) + "\n")
    c = bench.Clocks(0)
    c.path = path
    c.proc = object()  # a sampler ran
    return c


def line(t, mhz, power, power_cap="Not Active", thermal="Not Active"):
    ts = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return (f"{ts}, 0, {mhz}, 2070, {power}, 0x0000000000000000, Not Active, Not Active, "
            f"{thermal}, {power_cap}")


def test_samples_inside_the_region_only():
    t0 = 1_800_000_000.0
    lines = [line(t0 - 0.30, 1200, 95.0, thermal="Active"),    # before: idle, throttled
             line(t0 + 0.01, 2070, 900.0),
             line(t0 + 0.03, 2055, 950.0, power_cap="Active"),
             line(t0 + 0.05, 2070, 940.0),
             line(t0 + 0.20, 900, 90.0)]                          # after: idle
    c = capture(lines)
    c.mark(t0, t0 + 0.06)
    s = c.summary()
    assert s["samples_in_region"] == 3 and s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]                      # the thermal flag was outside


def test_short_region_takes_the_nearest_samples():
    t0 = 1_800_000_000.0
    c = capture([line(t0 - 0.5, 1000, 90.0), line(t0 - 0.012, 2070, 800.0), line(t0 + 0.018, 2060, 820.0),
                 line(t0 + 0.4, 990, 90.0)])
    c.mark(t0, t0 + 0.005)
    s = c.summary()
    assert s["samples_in_region"] == 0 and s["samples"] == 2
    assert s["sm_mhz"] == 2065.0 and s["reasons"] == []


def test_no_capture_gives_no_record():
    c = capture(["garbage line"])
    c.mark(0.0, 1.0)
    assert c.summary() is None
