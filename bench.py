"""Benchmark: seg-seg pair interactions/s on one GB300 (FP64 plain method, and
the FP32 + learned-surrogate form at its stated error).

Workload "gpu65k": 65,536 segments = 8192 closed square loops (shear and
prismatic, BCC {110}<111> slip systems, L ~ U(20, 200) b, centres uniform in a
20,000^3 b cube, 5% shifted / tilted near-parallel neighbours), seed 0.
A step is one all-pairs calcSegSegForce: N(N-1)/2 = 2.147e9 pair interactions.

value: device-resident path (packed segments already in HBM, forces left in
       HBM), CUDA events on the launching stream over K steps, L2 flushed
       (a 512 MB write) before every step.  Arithmetic (--mode): fp64_fast by
       default, the FP64 form with fewer FP64 instructions held to the same
       parity bound as the reference's own rounding (checked on 64 segments of
       the timed result against the oracle in the same run); the strict form
       (every multiply and add rounded as the reference rounds it) is timed
       beside it in `variants`.
e2e:   the reference-facing C-ABI call with host buffers (ddd_segseg_force):
       host -> device copies of the network arrays, compute, device -> host copy
       of the 3 x 2 x N forces, all inside the timed region.
cpu_baseline: the C++/OpenMP port of the reference's threaded path
       (calcSegSegForcePar: contiguous i-chunks, one atomic add per output
       component) on the host's cores, on a bounded sub-network of the workload.

surrogate: the same workload through ddd_surrogate_force (far pairs by the
       tcgen05 MLP, near pairs exact in f32c or strict FP64, 1% audit), value,
       speedup over the strict FP64 kernel, node-force error against the strict
       FP64 result, and the network kernel's tensor throughput; and the same
       path with the far pairs by FP32 Gauss-Legendre quadrature instead of the
       network (quad3_*: f32c, fast FP64 or strict FP64 near pairs).

precision_131k: the precision-form workload (131,072 segments, f32c force and
       mixed-form σ̃ on the 128^3 grid) with errors against the FP64 kernel on
       sampled segments and points.

collision: detectCollision on the workload network moving with the mobility
       step's velocities: pair scans/s of the kernels and of the host call, the
       oracle on a prefix of the network beside it, answers compared.

u_tilde: calc_uTilde of the workload network at the displacement nodes of a
       64^3-element cuboid mesh around its cube (Barnett triangles, FP64):
       evaluations/s of the kernels and of the host call, the OpenMP oracle on a
       sample of points beside it, values compared.

node_rows: calcSelfForce and dlnMobility (BCC) on the workload network through
       their host-array C-ABI calls, node forces from the timed seg-seg step plus
       the self force: e2e and kernel times, the kernel's algorithmic GB/s, the
       single-threaded oracle's time and the largest difference from it.

--impl reference: times that CPU port alone (the reference itself is Julia and
cannot run here), same metric and workload, each step a bounded sub-network.

Multi-GPU (--gpus N under torchrun): independent replicas (the path needs no
exchange between GPUs here); value = all ranks' pairs / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic FLOPs per unit (add/sub/mul/div/sqrt/log/atan = 1 each), from the
# op-counting instantiation of the oracle (oracle/ddd_oracle.cpp, opcount_*):
OPS_GENERAL_PAIR = 1511  # general branch: 626 add, 840 mul, 23 div, 10 sqrt, 8 log, 4 atan
OPS_PARALLEL_PAIR = 985  # near-parallel branch without core corrections
OPS_SIGMA_EVAL = 289  # one (segment, field point) σ̃ evaluation: 101 add, 183 mul, 3 div, 2 sqrt
# Each near-parallel side that needs core corrections adds two general evaluations.


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(value, dist, device):
    """The largest of every rank's `value` (the job's time is its slowest rank's);
    `dist` is torch.distributed or None for one process."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_par_sample(pkg, synth, oracle, p, b, k5, target_s, variant="atomic"):
    """Times an OpenMP port on the first n segments of the workload, n chosen so
    that one run takes about target_s seconds.  variant "atomic": the
    restatement of calcSegSegForcePar (contiguous i-chunks, one atomic add per
    output component); "private": the best-effort form (dynamic rows, per-thread
    accumulators)."""
    threads = cpu_threads()
    fn = oracle.segseg_par_atomic if variant == "atomic" else oracle.segseg_par_private
    coord, bvec, seg = synth.network_arrays(p[:256], b[:256])
    net = pkg.DislocationNetwork(coord, bvec, seg)
    t0 = time.perf_counter()
    fn(k5, net, threads)
    dt = time.perf_counter() - t0
    rate = net.numSeg * (net.numSeg - 1) / 2 / dt
    n_loops = int(min(p.shape[0], max(256, np.sqrt(2 * rate * target_s) / 8)))
    coord, bvec, seg = synth.network_arrays(p[:n_loops], b[:n_loops])
    net = pkg.DislocationNetwork(coord, bvec, seg)
    t0 = time.perf_counter()
    fn(k5, net, threads)
    dt = time.perf_counter() - t0
    n = net.numSeg
    return {"value": n * (n - 1) / 2 / dt, "unit": "pair-interactions/s", "cores": threads, "kind": "port",
            "variant": variant, "seconds": dt,
            "sample": "all %d pairs of the first %d segments (%d loops) of the workload, %.1f s" %
                      (n * (n - 1) // 2, n, n_loops, dt)}


def parity_sample(oracle, k5, net, F, rows):
    """The parity check of the GPU forces F (3 x 2 x numSeg) on the given
    0-based rows: the oracle's Float64 rows (the reference's arithmetic) and the
    same rows in long double.  noise = the largest node-force error of the
    reference's own Float64 arithmetic on these rows (against long double).
    The bound, per node force vector: |F_gpu - F_ref| <= 1e-10 |F_ref| + 4 noise
    + 4 ulps of the largest force; bound_excess = the largest left side minus
    right side (<= 0 when the bound holds); accuracy: the kernel's own error
    against long double <= 3 noise."""
    rows = np.sort(np.asarray(rows))
    nt_ = cpu_threads()
    ref_rows = oracle.segseg_rows(k5, net, rows, nt_)
    ext_rows = oracle.segseg_ser_ld(k5, net, rows, nthreads=nt_)
    nrm = lambda a: np.linalg.norm(a, axis=0)
    G = F[:, :, rows]
    d = nrm(G - ref_rows)
    noise = float(nrm(ref_rows - ext_rows).max())
    ulps = 4 * np.finfo(np.float64).eps * float(nrm(ext_rows).max())
    gpu_err = float(nrm(G - ext_rows).max())
    return {"rows": len(rows), "fp64_max_rel_node": float(np.max(d / nrm(ref_rows))),
            "fp64_err_vs_longdouble": gpu_err, "reference_arith_err_vs_longdouble": noise,
            "bound": "|dF| <= 1e-10 |F| + 4 noise + 4 ulp(max|F|) per node",
            "bound_excess": float(np.max(d - (1e-10 * nrm(ref_rows) + 4 * noise + ulps))),
            "accuracy_excess": gpu_err - (3 * noise + ulps)}


def cpu_sigma_sample(pkg, synth, oracle, p, b, k5, cube, target_s):
    """Times the OpenMP port of _calc_σTilde! (segment-outer order kept per
    point, points split over threads) on all segments of the workload and a
    sample of grid points sized to about target_s seconds."""
    threads = cpu_threads()
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    pts = synth.grid_points(32, cube)
    t0 = time.perf_counter()
    oracle.sigma_tilde(k5, pts[:, :threads], net, nthreads=threads)
    dt = time.perf_counter() - t0
    m = int(min(pts.shape[1], max(threads, threads * target_s / max(dt, 1e-6))))
    t0 = time.perf_counter()
    oracle.sigma_tilde(k5, np.asfortranarray(pts[:, :m]), net, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": net.numSeg * m / dt, "unit": "seg-point evaluations/s", "cores": threads, "kind": "port",
            "sample": "%d segments x %d points of the 32^3 grid, %.1f s" % (net.numSeg, m, dt)}


# DRAM bytes per tile pair of the strict and fast FP64 tile kernels and of the
# network pass, from one ncu capture each at 32,768 segments (32,896 tile
# pairs; the partial slots exceed L2 there, so traffic grows with the tile-pair
# count).
TILE_DRAM_BYTES_PER_TILE_PAIR = (31162112 + 376273664) // 32896
TILE_FX_DRAM_BYTES_PER_TILE_PAIR = (27079168 + 366944512) // 32896
MLP_DRAM_BYTES_PER_TILE_PAIR = (12404992 + 346662144) // 32896

# Tensor-core FLOPs of the surrogate network per pair slot (one row of the
# 128-row MMA tiles): 2 (16*128 + 128*128 + 128*128 + 128*112).
OPS_MLP_PAIR = 98304
SURROGATE_CKPT = os.path.join(ROOT, "ddd.jl_gb300", "data", "surrogate_gpu65k_nu028.bin")


def run_surrogate(args, pkg, ctx, k, soa, ref, pairs, ms_fp64, stream, sptr, flush):
    """The learned far-field surrogate on the same workload: far pairs through the
    tcgen05 MLP, near pairs exact, 1% of tile pairs audited exactly.  Exact passes
    in f32c ("FP32+surrogate") and in strict FP64.  Error: node-force relative
    RMS against the timed FP64 result `ref`."""
    import torch
    sur = pkg.Surrogate(ctx, seed=0)
    if os.path.exists(args.surrogate):
        sur.load(args.surrogate)
        source = "checkpoint %s (ddd.jl_gb300/train_surrogate.py: 4 networks of the generator, seeds 11-14, " \
                 "2.5e6 far pairs each, 20 epochs)" % os.path.relpath(args.surrogate, ROOT)
    else:
        import importlib.util
        spec = importlib.util.spec_from_file_location("train_surrogate",
                                                      os.path.join(ROOT, "ddd.jl_gb300", "train_surrogate.py"))
        ts_mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(ts_mod)
        t0 = time.time()
        sur, info = ts_mod.train(epochs=10)
        source = "trained in this run (%d samples, 10 epochs, %.0f s)" % (info["samples"], time.time() - t0)
    n = soa.shape[1]
    F = torch.empty((n, 6), dtype=torch.float64, device="cuda")
    refv = ref.view(n, 6)
    out = {"source": source, "kappa": sur.kappa, "audit_fraction": 0.01}
    # quad3_*: 3-point rule, switched to 2 points on 32-pair steps beyond QUAD_KAPPA_TWO lengths (the
    # default); quad3_f32c_no_switch: 3 points everywhere.
    for key, xm, far, k2 in (("f32c", "f32c", "network", None), ("fp64", "fp64", "network", None),
                             ("quad3_f32c", "f32c", "quad3", pkg.QUAD_KAPPA_TWO),
                             ("quad3_f32c_no_switch", "f32c", "quad3", 0.0),
                             ("quad3_fp64fast", "fp64_fast", "quad3", pkg.QUAD_KAPPA_TWO),
                             ("quad3_fp64", "fp64", "quad3", pkg.QUAD_KAPPA_TWO)):
        with torch.cuda.stream(stream):
            kap = None if far == "network" else pkg.QUAD_KAPPA  # the network's own kappa, or the quadrature's
            sur.force(k, soa, out=F, exact_mode=xm, stream=sptr, far=far, kappa=kap, kappa_two=k2)  # plan set-up
            ts, rep = [], None
            for _ in range(max(1, min(args.steps, 3))):
                flush.zero_()
                a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_.record(stream)
                _, rep = sur.force(k, soa, out=F, exact_mode=xm, stream=sptr, far=far, kappa=kap, kappa_two=k2)
                b_.record(stream)
                torch.cuda.synchronize()
                ts.append(a_.elapsed_time(b_))
        ms = statistics.mean(ts)
        dn = torch.linalg.norm((F - refv).view(n, 2, 3), dim=2)
        fn = torch.linalg.norm(refv.view(n, 2, 3), dim=2)
        slots = rep["tiles_total"] * 128 * 128
        tfl = slots * OPS_MLP_PAIR / (rep["ms_network"] * 1e-3) / 1e12
        far_pairs = rep["pairs_total"] - rep["pairs_near_general"] - rep["pairs_near_parallel"]
        if far != "network":
            out[key] = {
                "value": pairs / (ms * 1e-3), "unit": "pair-interactions/s", "ms_per_step": ms,
                "speedup_vs_fp64": ms_fp64 / ms,
                "far": "FP32 Gauss-Legendre quadrature, 3 points per segment" + (
                    ", 2 on 32-pair steps whose far pairs all lie beyond %g lengths" % k2 if k2 else ""),
                "kappa": pkg.QUAD_KAPPA, "kappa_two": k2, "exact_passes": xm,
                "error_vs_fp64": {"rel_rms": (torch.linalg.norm(F - refv) / torch.linalg.norm(refv)).item(),
                                  "median_rel_node": (dn / fn).median().item(),
                                  "max_node_over_max_force": (dn.max() / fn.max()).item()},
                "audit_estimate_rel_rms": rep["audit_node_rel_rms"], "fallback": rep["fallback"],
                "pairs_far": far_pairs,
                "ms": {kk: rep[kk] for kk in ("ms_prep", "ms_network", "ms_audit", "ms_near", "ms_reduce")},
                "far_kernel": {"kernel": "quad_far_tiles<3>", "far_pairs_per_s": far_pairs / (rep["ms_network"] * 1e-3),
                               "bound": "fp32"},
            }
            continue
        out[key] = {
            "value": pairs / (ms * 1e-3), "unit": "pair-interactions/s", "ms_per_step": ms,
            "speedup_vs_fp64": ms_fp64 / ms,
            "error_vs_fp64": {"rel_rms": (torch.linalg.norm(F - refv) / torch.linalg.norm(refv)).item(),
                              "median_rel_node": (dn / fn).median().item(),
                              "max_node_over_max_force": (dn.max() / fn.max()).item()},
            "audit_estimate_rel_rms": rep["audit_node_rel_rms"], "fallback": rep["fallback"],
            "pairs_near_exact": rep["pairs_near_general"] + rep["pairs_near_parallel"],
            "pairs_network": far_pairs,
            "ms": {kk: rep[kk] for kk in ("ms_prep", "ms_network", "ms_audit", "ms_near", "ms_reduce")},
            "network_kernel": {"kernel": "mlp_far_tiles", "tensor_tflops": tfl, "bound": "tensor",
                               "peak_tflops": None, "frac": None,
                               "traffic": MLP_DRAM_BYTES_PER_TILE_PAIR * rep["tiles_total"],
                               "flops": "%d pair slots x %d MMA FLOPs (FP16 operands, FP32 accumulation)"
                                        % (slots, OPS_MLP_PAIR)},
        }
    return out


def run_precision_131k(pkg, synth, ctx, k, stream, sptr, flush):
    """The precision-form workload: 131,072 segments of the same generator, the
    f32c all-pairs force and the mixed-form σ̃ on the 128^3-point grid,
    each timed once after a warm-up; errors against the FP64 kernel (the
    correctness oracle of the GPU forms) on 512 sampled segments (the idx form)
    and 4,096 sampled points."""
    import torch
    p, b, cfg = synth.make("prec131k", seed=0)
    n = p.shape[0] * 8
    pairs = n * (n - 1) // 2
    soa = torch.from_numpy(synth.packed_soa(p, b)).cuda()
    force = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(0)
    rows = np.sort(rng.choice(n, 512, replace=False))
    pts = synth.grid_points(cfg["grid"], cfg["cube"])
    M = pts.shape[1]
    x0 = torch.from_numpy(np.ascontiguousarray(pts.T)).cuda()
    sig = torch.zeros(6 * M, dtype=torch.float64, device="cuda")

    def timed(fn):
        with torch.cuda.stream(stream):
            fn()
            torch.cuda.synchronize()
            flush.zero_()
            a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a_.record(stream)
            fn()
            b_.record(stream)
            torch.cuda.synchronize()
        return a_.elapsed_time(b_)

    ctx.mode = "f32c"
    try:
        ms_f = timed(lambda: ctx.segseg_force_device(k, soa.data_ptr(), n, n, force.data_ptr(), stream=sptr))
        ms_s = timed(lambda: ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, sig.data_ptr(),
                                                    stream=sptr))
    finally:
        ctx.mode = "fp64"
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    ref_rows = ctx.segseg_force(k, net, idx=rows + 1)  # FP64, 3 x 2 x 512
    got = force.cpu().numpy().reshape(3, 2, n, order="F")[:, :, rows]
    dn = np.linalg.norm(got - ref_rows, axis=0)
    fn = np.linalg.norm(ref_rows, axis=0)
    sp = np.sort(rng.choice(M, 4096, replace=False))
    xs = torch.from_numpy(np.ascontiguousarray(pts[:, sp].T)).cuda()
    sref = torch.zeros(6 * len(sp), dtype=torch.float64, device="cuda")
    ctx.sigma_tilde_device(k, xs.data_ptr(), len(sp), soa.data_ptr(), n, n, sref.data_ptr())
    torch.cuda.synchronize()
    sg = sig.view(M, 6)[torch.from_numpy(sp).cuda()]
    sr = sref.view(len(sp), 6)
    ds = torch.linalg.norm(sg - sr, dim=1)
    ns = torch.linalg.norm(sr, dim=1)
    return {
        "config": "prec131k: %d segments (%d loops, same generator), sigma on the %d^3 = %d-point grid"
                  % (n, p.shape[0], cfg["grid"], M),
        "force_f32c": {"value": pairs / (ms_f * 1e-3), "unit": "pair-interactions/s", "ms": ms_f,
                       "error_vs_fp64_sampled_512_segments": {
                           "rel_rms": float(np.linalg.norm(got - ref_rows) / np.linalg.norm(ref_rows)),
                           "max_rel_node": float(np.max(dn / fn)),
                           "max_node_over_max_force": float(dn.max() / fn.max())}},
        "sigma_mixed": {"value": n * M / (ms_s * 1e-3), "unit": "seg-point evaluations/s", "ms": ms_s,
                        "error_vs_fp64_sampled_4096_points": {
                            "rel_rms": (torch.linalg.norm(sg - sr) / torch.linalg.norm(sr)).item(),
                            "max_rel_point": (ds / ns).max().item(),
                            "max_point_over_max": (ds.max() / ns.max()).item()}},
    }


def run_sigma_32k(pkg, synth, oracle, ctx, k, stream, sptr, flush, fp64_peak, with_cpu=True):
    """σ̃ of the 32,768-segment GPU workload (same generator, seed 0) at every
    point of the 128^3-point grid over its cube (2,097,152 points: the workload
    names "2^20 points on a 128^3 grid", and the whole grid is evaluated), FP64
    strict and the fast FP64 form: each one warm-up on 4,096 points, then one
    timed full evaluation (CUDA events, L2 flushed before it); 256 sampled
    points checked against the oracle (the reference's segment order per
    point) for both."""
    import torch
    p, b, cfg = synth.make("gpu32k", seed=0)
    n = p.shape[0] * 8
    pts = synth.grid_points(cfg["grid"], cfg["cube"])
    M = pts.shape[1]
    soa = torch.from_numpy(synth.packed_soa(p, b)).cuda()
    x0 = torch.from_numpy(np.ascontiguousarray(pts.T)).cuda()
    sig = torch.zeros(6 * M, dtype=torch.float64, device="cuda")
    sig_fx = torch.zeros(6 * M, dtype=torch.float64, device="cuda")

    def timed(out, mode):
        ctx.mode = mode
        try:
            with torch.cuda.stream(stream):
                ctx.sigma_tilde_device(k, x0.data_ptr(), 4096, soa.data_ptr(), n, n, out.data_ptr(), stream=sptr)
                torch.cuda.synchronize()
                flush.zero_()
                a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_.record(stream)
                ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, out.data_ptr(), stream=sptr)
                b_.record(stream)
                torch.cuda.synchronize()
        finally:
            ctx.mode = "fp64"
        return a_.elapsed_time(b_)

    ms = timed(sig, "fp64")
    ms_fx = timed(sig_fx, "fp64_fast")
    evals = n * M
    out = {"config": "gpu32k: %d segments x %d points (%d^3 grid over the %g^3 b cube), FP64 strict"
                     % (n, M, cfg["grid"], cfg["cube"]),
           "value": evals / (ms * 1e-3), "unit": "seg-point evaluations/s", "points_per_s": M / (ms * 1e-3),
           "ms": ms, "frac_fp64_peak": evals * OPS_SIGMA_EVAL / (ms * 1e-3) / fp64_peak,
           "kernel": "sigma_tilde_f64",
           "fast": {"value": evals / (ms_fx * 1e-3), "ms": ms_fx, "speedup_vs_fp64": ms / ms_fx,
                    "frac_fp64_peak": evals * OPS_SIGMA_EVAL / (ms_fx * 1e-3) / fp64_peak,
                    "kernel": "sigma_tilde_fx"}}
    if with_cpu:
        coord, bvec, seg = synth.network_arrays(p, b)
        net = pkg.DislocationNetwork(coord, bvec, seg)
        pick = np.sort(np.random.default_rng(1).choice(M, 256, replace=False))
        k5 = np.array([k.aSq, k.mu4pi, k.mu8pi, k.mu4pinu, k.nuMu4pinu])
        ref = oracle.sigma_tilde(k5, np.asfortranarray(pts[:, pick]), net, nthreads=cpu_threads())
        S = sig.view(M, 6)[torch.from_numpy(pick).cuda()].cpu().numpy().T
        d = np.linalg.norm(S - ref, axis=0)
        r = np.linalg.norm(ref, axis=0)
        smax = torch.linalg.norm(sig.view(M, 6), dim=1).max().item()
        out["parity_sample"] = {"points": len(pick), "max_rel_point": float(np.max(d / r)),
                                "bound": "|dσ| <= 1e-10 |σ| + 1e-12 max|σ| per point",
                                "bound_excess": float(np.max(d - (1e-10 * r + 1e-12 * smax)))}
        Sf = sig_fx.view(M, 6)[torch.from_numpy(pick).cuda()].cpu().numpy().T
        df = np.linalg.norm(Sf - ref, axis=0)
        out["fast"]["parity_sample"] = {"points": len(pick), "max_rel_point": float(np.max(df / r)),
                                        "bound_excess": float(np.max(df - (1e-10 * r + 1e-12 * smax)))}
    return out


def run_node_rows(pkg, oracle, ctx, net, dln, mat, segseg, reps=5, with_cpu=True):
    """calcSelfForce and dlnMobility (BCC) on the workload network through the
    host-array C-ABI calls (copies in and out included), the node forces built
    from the timed seg-seg step plus the self force.  Beside each, the oracle
    (single-threaded C) on the same inputs: its time and the largest difference
    from the GPU result."""
    k, sp = pkg.consts_of(dln, mat), pkg.self_params_of(dln, mat)
    mp = pkg.mob_params_of(dln, mat)
    n = net.numSeg

    def best(fn):
        fn()
        ts, ks = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            r = fn()
            ts.append(time.perf_counter() - t0)
            ks.append(getattr(ctx, "last_kernel_ms", 0.0))
        return min(ts) * 1e3, min(ks), r

    ms_self, k_self, (F1, F2) = best(lambda: ctx.self_force(k, sp, net))
    net.segForce[:, :, :n] = segseg
    net.segForce[:, 0, :n] += F1
    net.segForce[:, 1, :n] += F2
    ms_mob, k_mob, (Fn, Vn) = best(lambda: ctx.mobility_bcc(mp, net))
    net.nodeVel[:, :net.numNode] = Vn
    # Algorithmic bytes: self force reads two nodes, b and the segment row
    # (6 + 3 doubles, 3 int64) and writes 3 doubles per segment; mobility reads
    # per node its coordinates and connectivity row ((1 + 2 * maxConnect) int64)
    # and per connection the link row, the far node, b and the node's force
    # (2 int64, 9 doubles), and writes 6 doubles.
    ld = net.connectivity.shape[0]
    nconn = int(net.connectivity[0, :net.numNode].sum())
    b_self = n * (9 * 8 + 3 * 8 + 3 * 8)
    b_mob = net.numNode * (3 * 8 + ld * 8 + 6 * 8) + nconn * (2 * 8 + 9 * 8)
    out = {"segments": n, "nodes": net.numNode, "timing": "host arrays, H2D and D2H inside, best of %d calls" % reps,
           "self_force": {"ms_e2e": ms_self, "segments_per_s": n / (ms_self * 1e-3), "kernel_ms": k_self,
                          "kernel_gbs": b_self / (k_self * 1e-3) / 1e9 if k_self > 0 else None,
                          "algorithmic_bytes": b_self},
           "mobility_bcc": {"ms_e2e": ms_mob, "nodes_per_s": net.numNode / (ms_mob * 1e-3), "kernel_ms": k_mob,
                            "kernel_gbs": b_mob / (k_mob * 1e-3) / 1e9 if k_mob > 0 else None,
                            "algorithmic_bytes": b_mob, "drag": dict(dln.dragCoeffs), "sigmaPN": mat.σPN}}
    if with_cpu:
        k5 = np.array([dln.coreRadSq, mat.μ4π, mat.μ8π, mat.μ4πν, mat.νμ4πν])
        sc = np.array([dln.coreRad, dln.coreEnergy, mat.ν])
        mpv = np.array([mat.σPN, *(dln.dragCoeffs[c] for c in ("edge", "screw", "climb", "line"))])
        t0 = time.perf_counter()
        R1, R2 = oracle.self_force(k5, sc, net)
        cpu_self = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        RF, RV = oracle.mobility_bcc(mpv, net.coord, net.bVec, net.links, net.connectivity, net.segForce, net.numNode)
        cpu_mob = (time.perf_counter() - t0) * 1e3
        out["self_force"].update(cpu_ms=cpu_self, cpu_kind="port", cpu_cores=1,
                                 max_rel_diff_vs_oracle=float(np.abs(np.r_[F1 - R1, F2 - R2]).max() /
                                                              np.abs(R2).max()))
        out["mobility_bcc"].update(cpu_ms=cpu_mob, cpu_kind="port", cpu_cores=1,
                                   node_force_bit_equal=bool(np.array_equal(Fn, RF)),
                                   vel_rel_diff_vs_oracle=float(np.linalg.norm(Vn - RV) / np.linalg.norm(RV)))
    return out


def run_collision(pkg, oracle, ctx, net, synth, p, b, cd, reps=5, cpu_target_s=10.0, with_cpu=True):
    """detectCollision on the workload network (node velocities from the
    mobility step) through the host-array call: kernel and e2e time as pair
    scans/s (numSeg (numSeg - 1) / 2 per call, the reference's two-line loop),
    and beside it the oracle (the reference's serial loops) on a prefix of the
    network sized to about cpu_target_s, with the GPU answer on that prefix
    compared field by field."""
    n = net.numSeg
    pairs = n * (n - 1) // 2
    cd2 = cd * cd
    ctx.detect_collision(cd2, net)
    ts, ks = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        res, pair = ctx.detect_collision(cd2, net)
        ts.append(time.perf_counter() - t0)
        ks.append(ctx.last_kernel_ms)
    ms_e2e, ms_k = min(ts) * 1e3, min(ks)
    out = {"segments": n, "collisionDist": cd, "pairs_per_call": pairs,
           "result": [res[0], res[1], *res[2:8], res[8], res[9]], "pair": pair,
           "kernel_ms": ms_k, "value": pairs / (ms_k * 1e-3), "unit": "pair scans/s",
           "e2e": {"ms": ms_e2e, "value": pairs / (ms_e2e * 1e-3),
                   "h2d_bytes": int(net.numNode * (3 * 8 * 2 + 4 + 8 * net.connectivity.shape[0]) +
                                    net.links.shape[1] * 16 + n * 24), "d2h_bytes": 96},
           "timing": "best of %d calls; kernel = CUDA events around all collision kernels" % reps}
    if not with_cpu:
        return out

    def prefix(loops):
        coord, bvec, seg = synth.network_arrays(p[:loops], b[:loops])
        sub = pkg.DislocationNetwork(coord, bvec, seg, nodeVel=net.nodeVel[:, :loops * 8])
        return sub

    def ref(sub):
        return oracle.detect_collision(cd2, sub.coord, sub.nodeVel, sub.label, sub.links, sub.bVec, sub.connectivity,
                                       sub.numNode, sub.numSeg)

    sub = prefix(256)
    t0 = time.perf_counter()
    ref(sub)
    rate = sub.numSeg * (sub.numSeg - 1) / 2 / max(time.perf_counter() - t0, 1e-6)
    loops = int(min(p.shape[0], max(256, np.sqrt(2 * rate * cpu_target_s) / 8)))
    sub = prefix(loops)
    t0 = time.perf_counter()
    rres, rpair = ref(sub)
    dt = time.perf_counter() - t0
    gres, gpair = ctx.detect_collision(cd2, sub)
    m = sub.numSeg
    out["cpu_baseline"] = {"value": m * (m - 1) / 2 / dt, "unit": "pair scans/s", "cores": 1, "kind": "port",
                           "sample": "the first %d segments (%d loops) of the workload, %.1f s" % (m, loops, dt)}
    out["parity_prefix"] = {"segments": m, "equal": bool(tuple(gres) == tuple(rres) and gpair == rpair),
                            "result": [gres[0], gres[1], *gres[2:8], gres[8], gres[9]]}
    return out


def run_u_tilde(pkg, oracle, ctx, net, cube, cells=64, reps=3, cpu_target_s=8.0, with_cpu=True):
    """calc_uTilde on the workload network inside a cube^3 regular cuboid mesh
    of cells^3 elements, at the cantilever's displacement nodes (the x0 face and
    the x1/z1 edge): triangle-point evaluations/s of the kernels and of the host
    call; beside it the oracle (OpenMP over points, all host threads) on a
    sample of the points, its values compared with the GPU's."""
    mesh = pkg.fem.RegularCuboidMesh(cube, cube, cube, cells, cells, cells)
    bnd = pkg.fem.cantilever_boundaries(mesh)
    mat = pkg.MaterialParameters(mu=1.0, nu=0.28)
    pts = np.asfortranarray(mesh.coord[:, bnd.uGammaDln - 1])
    M = pts.shape[1]
    k = (mat.omνInv8π, mat.om2νomνInv8π)
    u = ctx.u_tilde(*k, mesh, pts, net)
    ts, ks = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        u = ctx.u_tilde(*k, mesh, pts, net)
        ts.append(time.perf_counter() - t0)
        ks.append(ctx.last_kernel_ms)
    evals = net.numSeg * M  # every segment is internal: one triangle each
    ms_k, ms_e = min(ks), min(ts) * 1e3
    out = {"segments": net.numSeg, "points": M, "mesh": "%g^3, %d^3 elements, cantilever uGammaDln" % (cube, cells),
           "evals_per_call": evals, "kernel_ms": ms_k, "value": evals / (ms_k * 1e-3),
           "unit": "triangle-point evaluations/s", "form": "strict FP64, the reference's formulas",
           "e2e": {"ms": ms_e, "value": evals / (ms_e * 1e-3)}, "timing": "best of %d calls" % reps}
    # The reformulated FP64 form (one atan2 solid angle, FMA): speed and its
    # difference from the strict result.
    mode = ctx.mode
    ctx.mode = "fp64_fma"
    try:
        uf = ctx.u_tilde(*k, mesh, pts, net)
        kf = []
        for _ in range(reps):
            uf = ctx.u_tilde(*k, mesh, pts, net)
            kf.append(ctx.last_kernel_ms)
    finally:
        ctx.mode = mode
    out["fast"] = {"kernel_ms": min(kf), "value": evals / (min(kf) * 1e-3), "speedup_vs_strict": ms_k / min(kf),
                   "max_abs_diff_over_max": float(np.abs(uf - u).max() / np.abs(u).max()),
                   "rel_rms_vs_strict": float(np.linalg.norm(uf - u) / np.linalg.norm(u))}
    if not with_cpu:
        return out
    md = {"faceNorm": mesh.faceNorm, "faceMidPt": mesh.faceMidPt, "C": mesh.closure, "lo": mesh.lo, "hi": mesh.hi}
    threads = cpu_threads()

    def ref(idx):
        return oracle.u_tilde(k, md, mesh.normals, np.asfortranarray(pts[:, idx]), net.coord, net.label, net.links,
                              net.bVec, net.numNode, net.numSeg, nthreads=threads)[0]

    # Calibrate on a growing probe until it takes ~1/8 of the target (the
    # triangle list is built once per call and dominates tiny probes).
    m = threads
    while True:
        t0 = time.perf_counter()
        ref(np.linspace(0, M - 1, m).astype(np.int64))
        dt = time.perf_counter() - t0
        if dt >= cpu_target_s / 8 or m >= M:
            break
        m = min(M, m * 4)
    m = int(min(M, max(threads, m * cpu_target_s / max(dt, 1e-6))))
    idx = np.linspace(0, M - 1, m).astype(np.int64)
    t0 = time.perf_counter()
    r = ref(idx)
    dt = time.perf_counter() - t0
    g = u.reshape(3, -1, order="F")[:, idx]
    out["cpu_baseline"] = {"value": net.numSeg * m / dt, "unit": "triangle-point evaluations/s", "cores": threads,
                           "kind": "port", "sample": "%d of the %d points, all segments, %.1f s" % (m, M, dt)}
    out["parity_sample"] = {"points": m, "max_abs_diff_over_max": float(np.abs(g - r).max() / np.abs(r).max()),
                            "rel_rms": float(np.linalg.norm(g - r) / np.linalg.norm(r))}
    return out


def _r(x, d=4):
    return None if x is None else float("%.*g" % (d, x))


def summary(line, variants, surrogate, sigma32k, batched):
    """The headline figures in a few hundred characters, printed last on the
    JSON line so that a reader of the line's end sees both halves of the metric
    (FP64 plain and FP32 + surrogate), their errors and roofline fractions."""
    rf = line["roofline"]
    out = {"fp64": {"mode": line.get("mode", "fp64").split(" ")[0],
                    "pairs_per_s": _r(line["value"]), "e2e": _r(line["e2e"]["value"]), "frac_probe": _r(rf["frac"], 3),
                    "frac_pipe_rate": _r(rf["frac_pipe_rate"], 3), "probe_tflops": _r(rf["peak"]),
                    "pipe_rate_tflops": _r(rf["pipe_rate_peak"])}}
    par = line.get("parity_sample")
    if par:
        out["fp64"]["parity"] = {"rows": par["rows"], "max_rel_node": _r(par["fp64_max_rel_node"], 3),
                                 "bound_excess": _r(par["bound_excess"], 3),
                                 "accuracy_excess": _r(par["accuracy_excess"], 3)}
    for m, v in (variants or {}).items():
        out[m] = {"pairs_per_s": _r(v["value"]), "x_fp64": _r(v["speedup_vs_fp64"], 3),
                  "rel_rms": _r(v["error_vs_fp64"]["rel_rms"], 3)}
        if v.get("frac_pipe_rate_algorithmic") is not None:
            out[m]["frac_pipe_rate"] = _r(v["frac_pipe_rate_algorithmic"], 3)
    if surrogate:
        sv = surrogate["f32c"]
        f32c = (variants or {}).get("f32c")
        out["surrogate_f32c"] = {
            "pairs_per_s": _r(sv["value"]), "x_fp64": _r(sv["speedup_vs_fp64"], 3),
            "x_f32c_exact": _r(f32c["ms_per_step"] / sv["ms_per_step"], 3) if f32c else None,
            "rel_rms": _r(sv["error_vs_fp64"]["rel_rms"], 3),
            "max_node_over_max": _r(sv["error_vs_fp64"]["max_node_over_max_force"], 3),
            "tensor_frac": _r(sv["network_kernel"]["frac"], 3), "kappa": surrogate["kappa"],
            "arch": "MLP 16-128-128-128-112 GELU, FP16 fwd / FP32 acc, exact bilinear b contraction"}
    for qk in ("quad3_f32c", "quad3_f32c_no_switch", "quad3_fp64fast"):
        if surrogate and qk in surrogate:
            qv = surrogate[qk]
            out[qk] = {"pairs_per_s": _r(qv["value"]), "x_fp64": _r(qv["speedup_vs_fp64"], 3),
                       "rel_rms": _r(qv["error_vs_fp64"]["rel_rms"], 3),
                       "max_node_over_max": _r(qv["error_vs_fp64"]["max_node_over_max_force"], 3)}
    if sigma32k:
        fx = sigma32k.get("fast", {})
        out["sigma_32k_grid128"] = {"evals_per_s": _r(sigma32k["value"]), "frac_probe": _r(sigma32k["frac_fp64_peak"], 3),
                                 "bound_excess": _r(sigma32k.get("parity_sample", {}).get("bound_excess"), 3),
                                 "fast_evals_per_s": _r(fx.get("value")), "fast_frac_probe": _r(fx.get("frac_fp64_peak"), 3),
                                 "fast_bound_excess": _r(fx.get("parity_sample", {}).get("bound_excess"), 3)}
    if batched:
        out["batched"] = {m: {"pairs_per_s": _r(batched[m]["value"]),
                              "rel_rms": _r(batched[m]["error_vs_fp64"]["rel_rms"], 3)}
                          for m in ("f32c", "fp64", "fp64_fast") if m in batched}
    return out


def run_reference(args, pkg, synth, oracle):
    ws, rank = _dist()
    if rank != 0:
        return
    p, b, cfg = synth.make(args.workload, seed=0, num_loops=args.loops)
    k5 = np.array([1.0, 1 / (4 * np.pi), 1 / (8 * np.pi), 1 / (4 * np.pi) / (1 - synth.NU),
                   synth.NU / (4 * np.pi) / (1 - synth.NU)])
    times, vals = [], []
    info = None
    for it in range(args.warmup + args.steps):
        info = cpu_par_sample(pkg, synth, oracle, p, b, k5, args.ref_step_s)
        if it >= args.warmup:
            vals.append(info["value"])
            times.append(info["seconds"])
    v = statistics.median(vals)
    n = p.shape[0] * 8
    out = {
        "impl": "reference",
        "metric": "seg-seg pair interactions/s at 65k segs (FP64 plain vs FP32+surrogate) at stated error",
        "value": v, "unit": "pair-interactions/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "%s: %d segments, %d loops" % (args.workload, n, p.shape[0]),
                   "step": "all pairs of a prefix of the workload sized to about %g s (%s); ms_per_step is that "
                           "sampled step's wall time" % (args.ref_step_s, info["sample"]),
                   "ms_per_full_workload_step_extrapolated": 1e3 * (n * (n - 1) / 2) / v},
        "cpu_baseline": {"kind": "port", "cores": info["cores"], "sample": info["sample"], "value": v,
                         "unit": "pair-interactions/s",
                         "what": "C++/OpenMP restatement of calcSegSegForcePar (DislocationForces.jl:719-777); "
                                 "the Julia reference cannot run on this box (no Julia runtime)"},
        "e2e": {"value": v, "unit": "pair-interactions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gpu65k")
    ap.add_argument("--loops", type=int, default=None,
                    help="override the loop count of the workload (8 segments per loop), for small profiling runs")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--cpu-target-s", type=float, default=15.0)
    ap.add_argument("--ref-step-s", type=float, default=4.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--parity-rows", type=int, default=64, help="segments of the timed result checked against the "
                    "oracle (and long double)")
    ap.add_argument("--rows-only", action="store_true",
                    help="only the rows around the force (self force, mobility, collision, calc_uTilde) on the "
                         "workload, seg-seg forces from one untimed call; prints their JSON and exits (the command "
                         "the ncu captures of those kernels use)")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--mode", default="fp64_fast", choices=["fp64", "fp64_fast"],
                    help="arithmetic of the timed FP64 steps: fp64_fast (default) = the reformulated FP64 form, "
                         "held to the same parity bound as the reference's rounding, which fp64 (strict) keeps "
                         "exactly; the other form is reported beside it")
    ap.add_argument("--headline-only", action="store_true",
                    help="only the timed steps (no e2e, variants or other rows): the command ncu captures of the "
                         "FP64 tile kernel use")
    ap.add_argument("--no-sigma", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--sigma-grid", type=int, default=32)
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-precision131k", action="store_true")
    ap.add_argument("--profile-surrogate", type=int, default=0, metavar="N",
                    help="only run N surrogate force calls on the workload (no audit) and exit: "
                         "the command the ncu captures of the surrogate kernels use")
    ap.add_argument("--surrogate", default=SURROGATE_CKPT, help="surrogate checkpoint (trained here when missing)")
    ap.add_argument("--kappa-two", type=float, default=None,
                    help="--far quad3: 2-point switch threshold in lengths (default the package's, 0 = off)")
    ap.add_argument("--far", default="network", choices=["network", "quad2", "quad3"],
                    help="far pass of --profile-surrogate: the network or FP32 Gauss-Legendre quadrature")
    ap.add_argument("--exact-mode", default="f32c", choices=["f32c", "fp64_fast", "fp64"],
                    help="arithmetic of the near pass of --profile-surrogate")
    args = ap.parse_args()

    import __graft_entry__ as graft
    pkg = graft.load_package()
    oracle, _ = graft.load_oracle()
    import ddd_gb300.synth as synth

    if args.impl == "reference":
        run_reference(args, pkg, synth, oracle)
        return

    import torch
    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    p, b, cfg = synth.make(args.workload, seed=0, num_loops=args.loops)
    n = p.shape[0] * 8
    pairs = n * (n - 1) // 2
    dln = pkg.DislocationParameters(coreRad=synth.CORE_RAD)
    mat = pkg.MaterialParameters(mu=synth.MU, nu=synth.NU)
    k = pkg.consts_of(dln, mat)
    ctx = pkg.Context(local)

    if args.profile_surrogate:
        sur = pkg.Surrogate(ctx, seed=0).load(args.surrogate)
        segs = torch.from_numpy(synth.packed_soa(p, b)).cuda()
        for _ in range(args.profile_surrogate):
            _, rep = sur.force(k, segs, exact_mode=args.exact_mode, audit_fraction=0.0, far=args.far,
                               kappa_two=args.kappa_two)
        torch.cuda.synchronize()
        print(json.dumps({"profile_surrogate": args.profile_surrogate, "segments": n, "report": rep}), flush=True)
        return

    if args.rows_only:
        coord, bvec, seg = synth.network_arrays(p, b)
        net = pkg.DislocationNetwork(coord, bvec, seg)
        out = ctx.segseg_force(k, net)
        dln_m = pkg.DislocationParameters(coreRad=synth.CORE_RAD, coreEnergy=1.0,
                                          dragCoeffs=dict(edge=1.0, screw=2.0, climb=1e10, line=1e-4))
        mat_m = pkg.MaterialParameters(mu=synth.MU, nu=synth.NU, sigmaPN=1e-4)
        rows = {"node_rows": run_node_rows(pkg, oracle, ctx, net, dln_m, mat_m, out, with_cpu=not args.no_cpu),
                "collision": run_collision(pkg, oracle, ctx, net, synth, p, b, 10.0, with_cpu=not args.no_cpu),
                "u_tilde": run_u_tilde(pkg, oracle, ctx, net, cfg["cube"], with_cpu=not args.no_cpu),
                "segments": n}
        print(json.dumps(rows), flush=True)
        return

    stream = torch.cuda.Stream()
    soa = torch.from_numpy(synth.packed_soa(p, b)).cuda()
    force = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    sptr = stream.cuda_stream

    # One reported call: branch statistics for the algorithmic FLOP count.
    ctx.mode = args.mode
    rep = ctx.segseg_force_device(k, soa.data_ptr(), n, n, force.data_ptr(), stream=sptr, report=True)
    flops_per_step = (rep["pairs_general"] * OPS_GENERAL_PAIR + rep["pairs_parallel"] * OPS_PARALLEL_PAIR
                      + rep["core_sides"] * 2 * OPS_GENERAL_PAIR)
    # FP64 peak, measured: an FMA-chain kernel on every SM, calibrated to run
    # about a second per timing (best of three), clocks sampled meanwhile.
    with ClockSampler(local) as probe_clocks:
        fp64_peak = ctx.probe_fma_peak(64)
    probe_clock = probe_clocks.summary()
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            ctx.segseg_force_device(k, soa.data_ptr(), n, n, force.data_ptr(), stream=sptr)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with ClockSampler(local) as clocks:
            ev0.record(stream)
            for s in range(args.steps):
                flush.zero_()
                kev[s][0].record(stream)
                ctx.segseg_force_device(k, soa.data_ptr(), n, n, force.data_ptr(), stream=sptr)
                kev[s][1].record(stream)
            ev1.record(stream)
            torch.cuda.synchronize()
        ms_total = ev0.elapsed_time(ev1)
        ms_kernel = [a.elapsed_time(b_) for a, b_ in kev]
    ms_step = max_over_ranks(ms_total, dist, "cuda") / args.steps
    if dist:
        dist.barrier()
    value = ws * pairs / (ms_step * 1e-3)
    if args.headline_only:
        if rank == 0:
            print(json.dumps({"mode": args.mode, "value": value, "unit": "pair-interactions/s", "ms_per_step": ms_step,
                              "segments": n, "steps": args.steps}), flush=True)
        return

    # Other arithmetic modes of the same path, same workload and timing: the FMA
    # build of the FP64 kernel and the df64 precision form.  Each reports its
    # error against the strict FP64 result (itself parity-checked).
    variants = {}
    ref_force = force.cpu().numpy().reshape(3, 2, -1, order="F")  # the timed mode's result
    # The strict FP64 result (the reference's rounding): the errors of every
    # other form are taken against it.
    strict = force
    if args.mode != "fp64":
        ctx.mode = "fp64"
        strict = torch.zeros_like(force)
        ctx.segseg_force_device(k, soa.data_ptr(), n, n, strict.data_ptr(), stream=sptr)
        torch.cuda.synchronize()
    strict_force = strict.cpu().numpy().reshape(3, 2, -1, order="F")
    cs_v = clocks.summary()
    pipe_peak_v = 4.0 * n_sm * cs_v["sm_mhz"] * 1e6 if cs_v else None
    if not args.no_variants:
        for mode in [m for m in ("fp64", "fp64_fast", "fp64_fma", "df64", "f32c") if m != args.mode]:
            ctx.mode = mode
            out_v = torch.zeros_like(force)
            with torch.cuda.stream(stream):
                rep_v = ctx.segseg_force_device(k, soa.data_ptr(), n, n, out_v.data_ptr(), stream=sptr, report=True)
                vms = []
                for s_ in range(max(1, min(args.steps, 2))):
                    flush.zero_()
                    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a_.record(stream)
                    ctx.segseg_force_device(k, soa.data_ptr(), n, n, out_v.data_ptr(), stream=sptr)
                    b_.record(stream)
                    torch.cuda.synchronize()
                    vms.append(a_.elapsed_time(b_))
            ctx.mode = args.mode
            Fv = out_v.cpu().numpy().reshape(3, 2, -1, order="F")
            dn = np.linalg.norm(Fv - strict_force, axis=0)
            fn = np.linalg.norm(strict_force, axis=0)
            variants[mode] = {
                "value": pairs / (statistics.mean(vms) * 1e-3), "unit": "pair-interactions/s",
                "ms_per_step": statistics.mean(vms),
                "speedup_vs_fp64": ms_step / statistics.mean(vms),
                "frac_fp64_peak_algorithmic": flops_per_step / (statistics.mean(vms) * 1e-3) / fp64_peak,
                "frac_pipe_rate_algorithmic": (flops_per_step / (statistics.mean(vms) * 1e-3) / pipe_peak_v
                                               if pipe_peak_v else None),
                "error_vs_fp64": {"rel_rms": float(np.linalg.norm(Fv - strict_force) / np.linalg.norm(strict_force)),
                                  "max_node_over_max_force": float(dn.max() / fn.max()),
                                  "max_rel_node": float(np.max(dn / np.maximum(fn, 1e-300)))},
                "branches_match_fp64": (rep_v["pairs_general"], rep_v["pairs_parallel"]) ==
                                       (rep["pairs_general"], rep["pairs_parallel"]),
            }

    # The rows below run in the reference's rounding unless they set a mode.
    ctx.mode = "fp64"
    ms_strict = ms_step if args.mode == "fp64" else variants.get("fp64", {}).get("ms_per_step")

    # Learned far-field surrogate ("FP32+surrogate"), same workload and timing.
    surrogate = None
    if not args.no_surrogate:
        surrogate = run_surrogate(args, pkg, ctx, k, soa, strict, pairs, ms_strict or ms_step, stream, sptr, flush)
        peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(peaks_path):
            tp = json.load(open(peaks_path)).get("bf16_tflops")
            for xm in ("f32c", "fp64"):
                nk = surrogate[xm]["network_kernel"]
                nk["peak_tflops"] = tp
                nk["frac"] = nk["tensor_tflops"] / tp if tp else None
                nk["peak_source"] = "MEASURED_PEAKS.json bf16_tflops (burst; FP16 dense rate is the same)"

    precision131k = None
    if not args.no_precision131k and args.loops is None:
        precision131k = run_precision_131k(pkg, synth, ctx, k, stream, sptr, flush)

    sigma32k = None
    if not args.no_sigma and args.loops is None:
        sigma32k = run_sigma_32k(pkg, synth, oracle, ctx, k, stream, sptr, flush, fp64_peak, with_cpu=not args.no_cpu)

    # Field-point stress σ̃ of the same network on a 32^3 grid over the cube.
    sigma = None
    if not args.no_sigma:
        pts = synth.grid_points(args.sigma_grid, cfg["cube"])
        M = pts.shape[1]
        x0 = torch.from_numpy(np.ascontiguousarray(pts.T)).cuda()
        sig = torch.zeros(6 * M, dtype=torch.float64, device="cuda")
        with torch.cuda.stream(stream):
            ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, sig.data_ptr(), stream=sptr)
            torch.cuda.synchronize()
            sms = []
            for _ in range(2):
                flush.zero_()
                a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_.record(stream)
                ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, sig.data_ptr(), stream=sptr)
                b_.record(stream)
                torch.cuda.synchronize()
                sms.append(a_.elapsed_time(b_))
        ms_sig = statistics.mean(sms)
        evals = n * M
        sigma = {"value": evals / (ms_sig * 1e-3), "unit": "seg-point evaluations/s",
                 "points_per_s": M / (ms_sig * 1e-3), "ms": ms_sig,
                 "config": "%d segments x %d points (%d^3 grid over the cube), FP64 strict" % (n, M, args.sigma_grid),
                 "frac_fp64_peak": evals * OPS_SIGMA_EVAL / (ms_sig * 1e-3) / fp64_peak}
        # The precision form (df64 geometry and endpoint differences, FP32
        # assembly): throughput and error against the FP64 result above.
        sig_ref = sig.clone()
        ctx.mode = "f32c"
        with torch.cuda.stream(stream):
            ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, sig.data_ptr(), stream=sptr)
            torch.cuda.synchronize()
            sms = []
            for _ in range(2):
                flush.zero_()
                a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_.record(stream)
                ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, sig.data_ptr(), stream=sptr)
                b_.record(stream)
                torch.cuda.synchronize()
                sms.append(a_.elapsed_time(b_))
        ctx.mode = "fp64"
        ms_mix = statistics.mean(sms)
        dp = torch.linalg.norm((sig - sig_ref).view(M, 6), dim=1)
        rp = torch.linalg.norm(sig_ref.view(M, 6), dim=1)
        sigma["mixed"] = {"value": evals / (ms_mix * 1e-3), "ms": ms_mix, "speedup_vs_fp64": ms_sig / ms_mix,
                          "error_vs_fp64": {"rel_rms": (torch.linalg.norm(sig - sig_ref) /
                                                        torch.linalg.norm(sig_ref)).item(),
                                            "max_point_over_max": (dp.max() / rp.max()).item()}}
        # The fast FP64 form (sigma_fx.cuh): throughput, and its distance from
        # the strict result against the strict form's per-point bound.
        ctx.mode = "fp64_fast"
        with torch.cuda.stream(stream):
            ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, sig.data_ptr(), stream=sptr)
            torch.cuda.synchronize()
            sms = []
            for _ in range(2):
                flush.zero_()
                a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_.record(stream)
                ctx.sigma_tilde_device(k, x0.data_ptr(), M, soa.data_ptr(), n, n, sig.data_ptr(), stream=sptr)
                b_.record(stream)
                torch.cuda.synchronize()
                sms.append(a_.elapsed_time(b_))
        ctx.mode = "fp64"
        ms_fx = statistics.mean(sms)
        dp = torch.linalg.norm((sig - sig_ref).view(M, 6), dim=1)
        sigma["fast"] = {"value": evals / (ms_fx * 1e-3), "ms": ms_fx, "speedup_vs_fp64": ms_sig / ms_fx,
                         "frac_fp64_peak": evals * OPS_SIGMA_EVAL / (ms_fx * 1e-3) / fp64_peak,
                         "kernel": "sigma_tilde_fx",
                         "error_vs_fp64": {"rel_rms": (torch.linalg.norm(sig - sig_ref) /
                                                       torch.linalg.norm(sig_ref)).item(),
                                           "bound_excess": (dp - (1e-10 * rp + 1e-12 * rp.max())).max().item()}}

    # Batched form: 256 independent networks (segment counts log-uniform in
    # [64, 8192], own seeds, cubes 2000-20000 b, slip-system subsets) in one
    # persistent launch replayed from a CUDA graph.  The f32c plan is autotuned
    # (tile 64/128 x work order); the FP64 plans (strict and fast) use the
    # default tile 128.
    batched = None
    if not args.no_batched:
        nets = synth.batch_networks(256, seed=0)
        sizes = [p_.shape[0] * 8 for p_, _ in nets]
        bsegs = torch.from_numpy(np.ascontiguousarray(np.concatenate([synth.packed_soa(p_, b_) for p_, b_ in nets],
                                                                     axis=1))).cuda()
        bforce = torch.zeros(6 * bsegs.shape[1], dtype=torch.float64, device="cuda")
        bpairs = sum(n_ * (n_ - 1) // 2 for n_ in sizes)
        batched = {"networks": len(sizes), "segments": int(sum(sizes)), "pairs_per_run": int(bpairs)}
        # Reference for the errors: every network through the single-network
        # FP64 kernel (itself parity-checked against the oracle).
        tot = bsegs.shape[1]
        bref = torch.zeros(6 * tot, dtype=torch.float64, device="cuda")
        off_ = 0
        for n_ in sizes:
            ctx.segseg_force_device(k, bsegs.data_ptr() + 8 * off_, tot, n_, bref.data_ptr() + 8 * 6 * off_,
                                    stream=sptr)
            off_ += n_
        torch.cuda.synchronize()
        bref_n = torch.linalg.norm(bref.view(tot, 2, 3), dim=2)
        for mode, tune in (("f32c", True), ("fp64", False), ("fp64_fast", False)):
            plan = pkg.Batch(ctx, sizes, mode=mode, tune=tune)
            with torch.cuda.stream(stream):
                plan.run(k, bsegs.data_ptr(), bforce.data_ptr(), stream=sptr)  # tune (if asked) + graph capture
                torch.cuda.synchronize()
                a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_.record(stream)
                for _ in range(2):
                    plan.run(k, bsegs.data_ptr(), bforce.data_ptr(), stream=sptr)
                b_.record(stream)
                torch.cuda.synchronize()
            ms_b = a_.elapsed_time(b_) / 2
            inf = plan.info()
            dn_ = torch.linalg.norm((bforce - bref).view(tot, 2, 3), dim=2)
            batched[mode] = {"value": bpairs / (ms_b * 1e-3), "unit": "pair-interactions/s", "ms_per_run": ms_b,
                             "tile": inf["tile"], "order": inf["order"], "work_items": inf["work_items"],
                             "tune_ms": inf["tune_ms"] if tune else None, "graph_launches": inf["graph_launches"],
                             "error_vs_fp64": {
                                 "against": "each network through the single-network FP64 kernel",
                                 "rel_rms": (torch.linalg.norm(bforce - bref) / torch.linalg.norm(bref)).item(),
                                 "max_rel_node": (dn_ / bref_n.clamp_min(1e-300)).max().item(),
                                 "max_node_over_max_force": (dn_.max() / bref_n.max()).item(),
                                 "bit_equal": bool(torch.equal(bforce, bref))}}
            plan.close()

    # End to end through the reference-facing C-ABI call with host arrays, in
    # the timed steps' mode.
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    ctx.mode = args.mode
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else max(1, min(args.steps, 3))
    pkg_ctx = ctx
    pkg_ctx.segseg_force(k, net)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        out = pkg_ctx.segseg_force(k, net)
    t_e2e = max_over_ranks((time.perf_counter() - t0) / e2e_steps, dist, "cuda")  # every rank reaches this
    erep = pkg_ctx.last_report
    e2e_value = ws * pairs / t_e2e
    # Same forces as the device-resident path.
    same = bool(np.array_equal(out.ravel(order="F"), force.cpu().numpy()))
    ctx.mode = "fp64"

    if rank != 0:
        return
    # The node rows after the force: self force, then BCC mobility (drag
    # coefficients of the reference's mobility test, line drag 1e-4 so the
    # straight sides' midpoints have a regular drag).
    dln_m = pkg.DislocationParameters(coreRad=synth.CORE_RAD, coreEnergy=1.0,
                                      dragCoeffs=dict(edge=1.0, screw=2.0, climb=1e10, line=1e-4))
    mat_m = pkg.MaterialParameters(mu=synth.MU, nu=synth.NU, sigmaPN=1e-4)
    node_rows = run_node_rows(pkg, oracle, ctx, net, dln_m, mat_m, out, with_cpu=not args.no_cpu)
    # Collision detection on the network moving with those velocities:
    # collisionDist = minSegLen / 2 (the reference's default) with minSegLen =
    # 20 b, the workload's shortest segment.
    collision = run_collision(pkg, oracle, ctx, net, synth, p, b, 10.0, with_cpu=not args.no_cpu)
    # Displacements at the FE boundary of a mesh around the workload's cube.
    u_tilde = run_u_tilde(pkg, oracle, ctx, net, cfg["cube"], with_cpu=not args.no_cpu)
    achieved = flops_per_step / (statistics.mean(ms_kernel) * 1e-3)
    cs = clocks.summary()
    # The FP64 pipe's own rate: 2 DFMA per SM per clock (ncu's FP64 pipe peak:
    # 304 DFMA per cycle on 152 SMs), 2 FLOPs each, at the median SM clock
    # sampled during the timed steps.
    step_mhz = cs["sm_mhz"] if cs else None
    pipe_peak = 4.0 * n_sm * step_mhz * 1e6 if step_mhz else None
    line = {
        "metric": "seg-seg pair interactions/s at 65k segs (FP64 plain vs FP32+surrogate) at stated error",
        "value": value, "unit": "pair-interactions/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded generator, seed 0)",
        "config": {"workload": "%s: %d segments, %d closed 8-segment square loops, L~U(%g,%g) b, %g^3 b cube, "
                               "%d%% near-parallel neighbours" % (args.workload, n, p.shape[0], cfg["lmin"],
                                                                  cfg["lmax"], cfg["cube"],
                                                                  round(100 * cfg["parallel_fraction"])),
                   "pairs_per_step": pairs, "l2": "flushed before every step (512 MB write)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / fp64_peak,
                     "traffic": (TILE_DRAM_BYTES_PER_TILE_PAIR if args.mode == "fp64" else
                                 TILE_FX_DRAM_BYTES_PER_TILE_PAIR) * (n // 128) * (n // 128 + 1) // 2,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at 32,768 "
                                       "segments, scaled by tile pairs",
                     "kernel": "segseg_tile_f64<0>" if args.mode == "fp64" else "segseg_tile_fx<0>",
                     "peak_source": "measured FP64 FMA-chain probe on this GPU (ddd_probe_fma_peak, ~1 s per "
                                    "timing, best of 3); MEASURED_PEAKS.json holds no FP64 figure",
                     "probe_clock": probe_clock,
                     "pipe_rate_peak": pipe_peak / 1e12 if pipe_peak else None,
                     "frac_pipe_rate": achieved / pipe_peak if pipe_peak else None,
                     "pipe_rate_source": "2 DFMA/SM/clock x %d SMs x median SM clock of the timed steps" % n_sm,
                     "flops_per_step": flops_per_step,
                     "branches": {k_: rep[k_] for k_ in ("pairs_general", "pairs_parallel", "core_sides")}},
        "e2e": {"value": e2e_value, "unit": "pair-interactions/s", "h2d_bytes_per_step": erep["h2d_bytes"],
                "d2h_bytes_per_step": erep["d2h_bytes"], "steps": e2e_steps, "matches_device_path": same},
        "gpu_launches": 3 * args.steps,
        "mode": {"fp64": "fp64 (strict: every multiply and add rounded separately, as the reference)",
                 "fp64_fast": "fp64_fast (FP64 throughout, reformulated: one division per corner, log/atan in "
                              "integer fixed point on the integer pipes, explicit FMAs where the reference's terms do not cancel; same parity bound "
                              "as the strict form, checked below)"}[args.mode],
        "variants": variants,
        "surrogate": surrogate,
        "precision_131k": precision131k,
        "sigma_tilde": sigma,
        "sigma_tilde_32k_grid128": sigma32k,
        "batched": batched,
        "node_rows": node_rows,
        "collision": collision,
        "u_tilde": u_tilde,
        "kernel_ms_per_step": statistics.mean(ms_kernel),
    }
    if cs:
        line["clocks"] = cs
    if not args.no_cpu:
        k5 = np.array([dln.coreRadSq, mat.μ4π, mat.μ8π, mat.μ4πν, mat.νμ4πν])
        line["cpu_baseline"] = cpu_par_sample(pkg, synth, oracle, p, b, k5, args.cpu_target_s)
        line["cpu_baseline_private"] = cpu_par_sample(pkg, synth, oracle, p, b, k5, args.cpu_target_s / 2,
                                                      variant="private")
        if sigma is not None:
            sigma["cpu_baseline"] = cpu_sigma_sample(pkg, synth, oracle, p, b, k5, cfg["cube"], 5.0)
        # Parity of the timed result on sampled segments: the oracle's Float64 rows
        # and the same rows in long double (the reference arithmetic's own error).
        line["parity_sample"] = parity_sample(oracle, k5, net, ref_force, np.random.default_rng(0).choice(
            n, args.parity_rows, replace=False))
    line["summary"] = summary(line, variants, surrogate, sigma32k, batched)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
