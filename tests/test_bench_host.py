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


def _run_reference(env_extra=None):
    import json
    import os
    import subprocess
    import sys

    from conftest import ROOT

    env = dict(os.environ, **(env_extra or {}))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--ref-step-s", "0.2"], capture_output=True, text=True, timeout=300,
                       cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_line():
    """--impl reference (the CPU port of the threaded path) prints one line with
    the same metric, unit and direction as the GPU arm, an e2e object with no
    host-device traffic and a cpu_baseline describing the run."""
    (line,) = _run_reference()
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["metric"].startswith("seg-seg pair interactions/s at 65k segs")
    assert line["unit"] == "pair-interactions/s" and line["higher_is_better"] is True
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]


def test_reference_arm_other_ranks_print_nothing():
    """Under torchrun only rank 0 runs and prints; the others exit 0 at once."""
    assert _run_reference({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []
