"""bench.py's clock record: only nvidia-smi samples that arrived inside the
timed loop count, and throttle reasons are collected from those samples."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def _row(sm, mx=2070, hw="Not Active", hwt="Not Active", swt="Not Active", pc="Not Active"):
    return ["0", str(sm), str(mx), "900.0", "0x0", hw, hwt, swt, pc]


def test_samples_outside_the_window_are_dropped():
    rows = [(0.5, _row(900, pc="Active")), (1.1, _row(2070)), (1.5, _row(2055)), (1.9, _row(2070)),
            (2.5, _row(1200, hw="Active"))]
    c = bench.summarize_clocks(rows, 1.0, 2.0)
    assert c["samples"] == 3
    assert c["sm_mhz"] == 2070.0 and c["sm_max_mhz"] == 2070.0
    assert c["reasons"] == []
    assert abs(c["window_s"] - 1.0) < 1e-12


def test_reasons_inside_the_window_are_reported():
    rows = [(1.2, _row(1980, pc="Active")), (1.4, _row(1500, hwt="Active")), (1.6, _row(2070, swt="Active"))]
    c = bench.summarize_clocks(rows, 1.0, 2.0)
    assert c["reasons"] == ["hw_thermal_slowdown", "sw_power_cap", "sw_thermal_slowdown"]
    assert c["sm_mhz"] == 1980.0


def test_empty_window_has_no_clock():
    c = bench.summarize_clocks([(5.0, _row(2070))], 1.0, 2.0)
    assert c["samples"] == 0 and c["sm_mhz"] is None and c["reasons"] == []
