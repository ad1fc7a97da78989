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


def test_reference_arm_step_time_is_the_sampled_steps():
    """ms_per_step is the wall time of the sampled step that ran, so steps x
    ms_per_step fits inside the run; the full-workload figure is extrapolated
    separately."""
    (line,) = _run_reference()
    assert 0 < line["ms_per_step"] < 60_000
    assert line["config"]["ms_per_full_workload_step_extrapolated"] > line["ms_per_step"]


def test_parity_sample_bound_on_cpu(pkg, synth, oracle):
    """The bench's parity check, given the oracle's own Float64 forces, reports
    no excess over the bound; a planted 1e-6 relative error on one node does."""
    import numpy as np

    p, b = synth.square_loops(20, 4, 20.0, 200.0, 3000.0, 0.5, 0.1)
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    k5 = np.array([1.0, 1 / (4 * np.pi), 1 / (8 * np.pi), 1 / (4 * np.pi) / 0.72, 0.28 / (4 * np.pi) / 0.72])
    F = oracle.segseg_ser(k5, net)
    rows = np.arange(0, net.numSeg, 7)
    par = bench.parity_sample(oracle, k5, net, F, rows)
    assert par["rows"] == len(rows) and par["bound_excess"] <= 0 and par["fp64_max_rel_node"] == 0.0
    G = F.copy(order="F")
    G[:, 0, rows[3]] *= 1 + 1e-6
    assert bench.parity_sample(oracle, k5, net, G, rows)["bound_excess"] > 0


def test_summary_is_short_and_complete():
    """The summary printed at the end of the JSON line holds both halves of the
    metric and fits in the last 1,500 characters of the line."""
    import json

    line = {"value": 2.6e8, "e2e": {"value": 2.6e8},
            "roofline": {"frac": 0.37, "frac_pipe_rate": 0.31, "peak": 1.06, "pipe_rate_peak": 1.26},
            "parity_sample": {"rows": 64, "fp64_max_rel_node": 1e-10, "bound_excess": -1e-9,
                              "accuracy_excess": -1e-9}}
    var = {m: {"value": 1e9, "speedup_vs_fp64": 3.0, "ms_per_step": 1000.0, "error_vs_fp64": {"rel_rms": 1e-7}}
           for m in ("fp64_fma", "fp64_fast", "df64", "f32c")}
    sur = {"kappa": 20.0, "f32c": {"value": 5e9, "speedup_vs_fp64": 20.0, "ms_per_step": 400.0,
                                   "error_vs_fp64": {"rel_rms": 2.5e-5, "max_node_over_max_force": 1e-4},
                                   "network_kernel": {"frac": 0.36}}}
    s32 = {"value": 1.6e9, "frac_fp64_peak": 0.45, "parity_sample": {"bound_excess": -1e-12}}
    bat = {m: {"value": 1e9, "error_vs_fp64": {"rel_rms": 1e-7}} for m in ("f32c", "fp64")}
    s = bench.summary(line, var, sur, s32, bat)
    assert s["sigma_32k_grid128"]["evals_per_s"] == 1.6e9
    assert s["surrogate_f32c"]["x_f32c_exact"] == 2.5 and s["fp64"]["parity"]["rows"] == 64
    assert len(json.dumps({"summary": s})) < 1400
