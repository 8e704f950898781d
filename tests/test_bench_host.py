"""Host-side pieces of bench.py that need no GPU: the clock / throttle summary
that every JSON line carries, parsed from nvidia-smi's CSV rows."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_clock_summary_median_max_and_reasons():
    import bench
    rows = "\n".join([
        "0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2055, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ])
    s = bench.ClockSampler.parse(rows)
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3


def test_clock_summary_flags_thermal_and_empty_input():
    import bench
    hot = "0, 1500, 2070, 1400.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active"
    assert bench.ClockSampler.parse(hot)["reasons"] == ["hw_thermal_slowdown"]
    na = "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]"
    s = bench.ClockSampler.parse(na)
    assert s["sm_mhz"] is None and s["sm_max_mhz"] is None and s["reasons"] == []
    assert bench.ClockSampler.parse("")["reasons"] == ["no samples"]


def test_cpu_baseline_timing_mode_is_scoped(port):
    """The CPU baseline's timing mode (vectorised Cosine / L1 / L2 partial
    sums, the reference's Eigen speed) moves a distance by rounding only, is
    off by default, and leaves the numerical contract intact once off."""
    import numpy as np
    rng = np.random.default_rng(3)
    x, y = rng.random(784, dtype=np.float32), rng.random(784, dtype=np.float32)
    x /= np.linalg.norm(x)
    y /= np.linalg.norm(y)
    exact = {k: port.distance(x, y, k) for k in ("Cosine", "L1", "L2", "Chi2")}
    port.set_timing_mode(True)
    try:
        fast = {k: port.distance(x, y, k) for k in exact}
    finally:
        port.set_timing_mode(False)
    for k in ("Cosine", "L1", "L2"):
        assert abs(fast[k] - exact[k]) <= 2e-6 * max(1.0, abs(exact[k])), (k, fast[k], exact[k])
    assert fast["Chi2"] == exact["Chi2"]  # a scalar loop in the reference too
    assert {k: port.distance(x, y, k) for k in exact} == exact
