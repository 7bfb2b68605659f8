"""The bench's clock record from nvidia-smi rows (CPU, canned rows): the
median SM clock under load, the maximum clock, every throttle reason seen
Active, and the samples near the timed steps."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _row(sm, mx, hw="Not Active", hw_th="Not Active", sw_th="Not Active", pcap="Not Active"):
    return ["0", sm, mx, "900.0", "0x0000000000000000", hw, hw_th, sw_th, pcap]


def test_summary_reports_median_clock_and_active_reasons():
    import bench
    cs = bench.ClockSampler()
    cs.rows = [_row("2070", "2070"), _row("1965", "2070", pcap="Active"), _row("2070", "2070"),
               _row("[N/A]", "2070"), _row("1800", "2070", sw_th="Active")]
    cs.times = [0.0, 0.1, 0.2, 0.3, 0.9]
    cs.window = (0.15, 0.25)
    s = cs.summary()
    assert s["sm_mhz"] == 2017.5 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap", "sw_thermal_slowdown"]
    assert s["samples"] == 5 and s["samples_near_timed_steps"] == 3


def test_summary_without_samples_says_so():
    import bench
    s = bench.ClockSampler().summary()
    assert s["reasons"] == ["unsampled"] and s["sm_mhz"] is None


def test_a_clean_run_has_no_reasons():
    import bench
    cs = bench.ClockSampler()
    cs.rows = [_row("2070", "2070") for _ in range(4)]
    cs.times = [0.1 * k for k in range(4)]
    cs.window = (0.0, 0.3)
    s = cs.summary()
    assert s["reasons"] == [] and s["sm_mhz"] == 2070.0
