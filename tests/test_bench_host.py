"""Host-side logic of bench.py that needs no GPU: the clock record taken
during the timed region (median SM clock, throttle reasons), the peak used
as the roofline denominator, and the default run's timing arguments."""
import json

import bench
from conftest import ROOT


def _sampler(lines, mark=0):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    s.mark = mark
    return s


def test_clock_summary_median_and_reasons():
    lines = [
        # sm, max sm, power, active mask, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
        "1200, 2070, 300.0, 0x0, Not Active, Not Active, Not Active, Not Active",  # before the timed region
        "2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "2055, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
        "2070, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbled",
        "[N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = _sampler(lines, mark=1).summary()
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_flags_thermal_slowdown():
    lines = ["1800, 2070, 1000, 0x40, Not Active, Not Active, Active, Not Active",
             "1750, 2070, 1000, 0x48, Active, Not Active, Active, Not Active"]
    s = _sampler(lines).summary()
    assert s["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == 1775.0


def test_clock_summary_without_samples():
    s = _sampler([]).summary()
    assert s == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_roofline_peak_is_the_measured_copy_bandwidth():
    p = bench.measured_peaks()
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        assert p == {"hbm_gbs": json.loads(f.read_text())["hbm_gbs"], "source": "measured"}
    else:
        assert p["source"] == "fallback"


def test_default_run_is_one_gpu_with_three_warmups():
    a = bench.parse_args([])
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert a.impl == "la3g" and a.workload == "plain"
    assert bench.parse_args(["--impl", "reference"]).impl == "reference"
