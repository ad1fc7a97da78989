"""bench.py's host logic without a GPU: the clock record that decides whether
a run is kept (throttle reasons, SM clocks under load) is parsed from
nvidia-smi's CSV lines exactly as sampled."""
import bench


def _sampler(lines):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    return s


def test_clock_summary_reasons_and_median():
    s = _sampler([
        "0, 2070, 2070, 905.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1310.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1200.2, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
    ])
    c = s.summary()
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_clock_summary_flags_every_slowdown():
    s = _sampler(["0, 1500, 2070, 700.0, 0x48, Active, Active, Active, Not Active"])
    assert s.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_clock_summary_skips_unreadable_lines():
    s = _sampler(["", "garbage", "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]",
                  "0, 2070, 2070, 1000, 0x0, Not Active, Not Active, Not Active, Not Active"])
    assert s.summary()["samples"] == 1
    assert _sampler([]).summary() is None
