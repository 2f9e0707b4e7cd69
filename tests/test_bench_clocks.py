"""Host-side pieces of bench.py: the clock record attached to every bench line."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def test_clock_summary_reasons_and_median():
    rows = [(2070.0, 2070.0, 900.0, 0x4), (2055.0, 2070.0, 950.0, 0x0), (2070.0, 2070.0, 1000.0, 0x1)]
    s = bench.Clocks.summary(rows, "fake")
    assert s["sm_mhz"] == 2070.0 and s["sm_min_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]  # idle (0x1) is not a slowdown
    assert s["samples"] == 3 and s["power_w_median"] == 950.0


def test_clock_summary_slowdowns_named():
    s = bench.Clocks.summary([(1500.0, 2070.0, 1400.0, 0x8 | 0x40 | 0x20)], "fake")
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_clock_summary_empty():
    s = bench.Clocks.summary([], "none")
    assert s["sm_mhz"] is None and s["reasons"] == ["unavailable"] and s["samples"] == 0
