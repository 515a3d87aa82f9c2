"""The clock record of the benchmarks (`benchmarks/clocks.py`): median SM
clock, maximum clock and the throttle reasons seen active in any sample,
from nvidia-smi's CSV lines; unparsable lines are skipped; without
nvidia-smi the record says so."""
from benchmarks.clocks import ClockSampler, summarize


def test_summary_of_samples():
    lines = [
        "0, 2070, 2070, 900.5, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1390.0, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1000.0, Not Active, Not Active, Not Active, Not Active",
        "garbage",
        "0, [N/A], 2070, 1000.0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = summarize(lines)
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_thermal_reasons_are_reported():
    s = summarize(["0, 1500, 2070, 1400, Active, Active, Not Active, Not Active"])
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"]
    assert s["sm_mhz"] == 1500.0


def test_no_samples():
    assert summarize([]) == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
    c = ClockSampler(0)
    assert c.stop()["reasons"] == ["nvidia-smi unavailable"]
