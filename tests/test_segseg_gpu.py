"""Seg-seg force on the GPU (through the C ABI) against the oracle and the goldens.

Tolerances (FP64 path):
  * golden networks: |Δ| <= 5e-14 elementwise and ||Δ|| <= 1e-11 ||golden||
    (the oracle meets 2e-14 / 1e-11; the kernel adds FMA contraction).
  * against the oracle, per node force vector:
        |F_gpu - F_ref| <= 1e-10 |F_ref| + 4 * noise
    where noise = max over nodes of |F_ref - F_ext|, F_ext being the same
    algorithm evaluated in long double: the worst rounding error of the
    reference's own Float64 arithmetic on this network.  Node forces are sums of
    O(N) contributions that cancel (closed loops), so a node whose force is small
    carries an absolute error set by the large terms, and two correct Float64
    evaluations differ by about that much (up to ~3e-10 relative, measured).
    Over the whole array ||ΔF|| <= 1e-10 ||F||.
  * accuracy: max over nodes of |F_gpu - F_ext| <= 3 * noise: the kernel is as
    accurate as the reference's arithmetic.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, k5_of

pytestmark = pytest.mark.gpu

G_SEG = json.load(open(os.path.join(GOLDEN, "segseg_goldens.json")))


def _params(pkg, core_rad=1.0, mu=1.0, nu=0.28):
    return pkg.DislocationParameters(coreRad=core_rad), pkg.MaterialParameters(mu=mu, nu=nu)


def _synthetic(pkg, synth, num_loops, seed, config="gpu32k", parallel_fraction=None, cube=None):
    cfg = dict(synth.CONFIGS[config])
    if parallel_fraction is not None:
        cfg["parallel_fraction"] = parallel_fraction
    if cube is not None:
        cfg["cube"] = cube
    p, b = synth.square_loops(num_loops, seed, cfg["lmin"], cfg["lmax"], cfg["cube"], cfg["shear_fraction"],
                              cfg["parallel_fraction"])
    coord, bvec, seg = synth.network_arrays(p, b)
    return pkg.DislocationNetwork(coord, bvec, seg)


def check_forces(F, oracle, k5, net, rows=None, ref=None, factor=(4, 3), normwise=1e-10):
    """F: GPU forces of all segments (or of the 0-based `rows`); ref: the oracle's
    Float64 forces for the same columns (computed here when None)."""
    nt = os.cpu_count() or 1
    if ref is None:
        ref = oracle.segseg_ser(k5, net) if rows is None else oracle.segseg_rows(k5, net, rows, nt)
    ext = oracle.segseg_ser_ld(k5, net, rows, nthreads=nt)
    assert F.shape == ref.shape == ext.shape
    norm = lambda a: np.linalg.norm(a, axis=0)
    # A few ulps of the largest force: the floor for tiny networks whose noise is 0.
    ulps = 4 * np.finfo(np.float64).eps * norm(ext).max()
    noise = norm(ref - ext).max()
    d = norm(F - ref)
    gpu_err = norm(F - ext).max()
    if os.environ.get("DDD_TEST_STATS"):
        with open(os.environ["DDD_TEST_STATS"], "a") as fh:
            fh.write("%s n=%d noise=%.3e gpu_err=%.3e max_rel_diff=%.3e\n" % (
                os.environ.get("PYTEST_CURRENT_TEST", "?"), F.shape[2], noise, gpu_err,
                np.max(d / (norm(ref) + 1e-300))))
    assert np.linalg.norm(F - ref) <= normwise * np.linalg.norm(ref) + ulps
    excess = np.max(d - (1e-10 * norm(ref) + factor[0] * noise + ulps))
    assert excess <= 0, "node-force difference exceeds bound by %g (noise %g, max rel %g)" % (
        excess, noise, np.max(d / (norm(ref) + 1e-300)))
    assert gpu_err <= factor[1] * noise + ulps, "kernel error %g vs reference arithmetic %g" % (gpu_err, noise)
    return noise, gpu_err


@pytest.mark.parametrize("name", [c["name"] for c in G_SEG["cases"]])
def test_golden_networks(pkg, fixtures, oracle, name):
    c = next(c for c in G_SEG["cases"] if c["name"] == name)
    p = G_SEG["params"]
    fnet = fixtures.make_network(c["loops"], G_SEG["slipSystems"], c["range"], c["shift"])
    net = pkg.DislocationNetwork(fnet.coord, fnet.bVec, fnet.segIdx)
    dln, mat = _params(pkg, p["coreRad"], p["mu"], p["nu"])
    F = pkg.calcSegSegForce(dln, mat, net)
    for node, key in ((0, "f1"), (1, "f2")):
        gold = np.array(c[key])
        d = F[:, node, :].T - gold
        assert np.abs(d).max() <= 5e-14, np.abs(d).max()
        assert np.linalg.norm(d) <= 1e-11 * np.linalg.norm(gold)
    check_forces(F, oracle, k5_of(dln, mat), net)
    rep = pkg.get_context().last_report
    n = net.numSeg
    assert rep["pairs_general"] + rep["pairs_parallel"] == n * (n - 1) // 2
    if name == "pentagons_coincident":
        assert rep["pairs_parallel"] >= 5  # the coincident segment pairs take the near-parallel branch


@pytest.mark.parametrize("num_loops,seed", [(1, 0), (16, 1), (17, 2), (40, 3), (64, 4), (150, 5)])
def test_random_networks_vs_oracle(pkg, synth, oracle, num_loops, seed):
    net = _synthetic(pkg, synth, num_loops, seed, cube=3000.0)
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    check_forces(F, oracle, k5_of(dln, mat), net)


@pytest.mark.parametrize("n", [1, 2, 3, 127, 129, 255, 257])
def test_ragged_sizes(pkg, synth, oracle, n):
    """numSeg not a multiple of the tile, including 1 and 2 segments."""
    net = _synthetic(pkg, synth, 40, 11, cube=2000.0)
    net.numSeg = n
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    if n == 1:
        assert np.all(F == 0)
    else:
        check_forces(F, oracle, k5_of(dln, mat), net)


def test_empty_network(pkg, synth):
    net = _synthetic(pkg, synth, 2, 0)
    net.numSeg = 0
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    assert F.shape == (3, 2, 0)


def test_near_parallel_heavy(pkg, synth, oracle):
    """Half the loops are shifted / 1e-5-rad-tilted copies of their neighbour."""
    net = _synthetic(pkg, synth, 96, 21, parallel_fraction=0.5, cube=1500.0)
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    rep = pkg.get_context().last_report
    assert rep["pairs_parallel"] > 0.05 * (rep["pairs_parallel"] + rep["pairs_general"])
    check_forces(F, oracle, k5_of(dln, mat), net)


def test_external_segments(pkg, synth, oracle):
    net = _synthetic(pkg, synth, 50, 31, cube=2000.0)
    rng = np.random.default_rng(5)
    net.extSeg[rng.choice(net.numSeg, 37, replace=False)] = 1
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    assert np.all(F[:, :, net.extSeg[:net.numSeg] == 1] == 0)
    check_forces(F, oracle, k5_of(dln, mat), net)


def test_deterministic(pkg, synth):
    net = _synthetic(pkg, synth, 64, 41, parallel_fraction=0.2, cube=2000.0)
    dln, mat = _params(pkg)
    a = pkg.calcSegSegForce(dln, mat, net)
    b = pkg.calcSegSegForce(dln, mat, net)
    assert np.array_equal(a, b)


def test_idx_form(pkg, synth, oracle):
    """SegmentForcesTest.jl:372-380: random idx with repeats, and a scalar idx."""
    net = _synthetic(pkg, synth, 60, 51, parallel_fraction=0.2, cube=2000.0)
    net.extSeg[[3, 100]] = 1
    dln, mat = _params(pkg)
    k5 = k5_of(dln, mat)
    rng = np.random.default_rng(7)
    idx = rng.integers(1, net.numSeg + 1, net.numSeg // 2)
    idx[:3] = [4, 4, 101]  # a repeated index and external segments
    Fi = pkg.calcSegSegForce(dln, mat, net, idx)
    assert np.all(Fi[:, :, 2] == 0)
    check_forces(Fi, oracle, k5, net, rows=idx - 1, ref=oracle.segseg_idx(k5, net, idx))
    Fall = pkg.calcSegSegForce(dln, mat, net)
    assert np.linalg.norm(Fi - Fall[:, :, idx - 1]) <= 1e-10 * np.linalg.norm(Fall[:, :, idx - 1])
    one = pkg.calcSegSegForce(dln, mat, net, 17)
    assert one.shape == (3, 2, 1)
    check_forces(one, oracle, k5, net, rows=[16], ref=oracle.segseg_idx(k5, net, [17]))


def test_inplace_forms(pkg, synth, oracle):
    net = _synthetic(pkg, synth, 40, 61, cube=2000.0)
    dln, mat = _params(pkg)
    base = np.asfortranarray(np.random.default_rng(1).normal(size=net.segForce.shape) * 1e-3)
    net.segForce[...] = base
    pkg.calcSegSegForce_inplace(dln, mat, net)
    F = pkg.calcSegSegForce(dln, mat, net)
    assert np.allclose(net.segForce[:, :, :net.numSeg], base[:, :, :net.numSeg] + F, rtol=1e-13, atol=1e-18)
    idx = np.array([5, 9, 9, 200])
    net.segForce[...] = 0
    pkg.calcSegSegForce_inplace(dln, mat, net, idx)
    Fi = pkg.calcSegSegForce(dln, mat, net, idx)
    expect = np.zeros_like(net.segForce)
    for k, i in enumerate(idx):
        expect[:, :, i - 1] += Fi[:, :, k]
    assert np.array_equal(net.segForce, expect)


def test_large_sampled_rows(pkg, synth, oracle):
    """32,768 segments (4096 shear + prismatic loops, 5% near-parallel neighbours):
    all pairs on the GPU, 24 sampled segments against the oracle's rows."""
    p, b, cfg = synth.make("gpu32k", seed=3)
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    rep = pkg.get_context().last_report
    n = net.numSeg
    assert rep["pairs_general"] + rep["pairs_parallel"] == n * (n - 1) // 2
    rng = np.random.default_rng(9)
    rows = np.sort(rng.choice(n, 24, replace=False))
    check_forces(F[:, :, rows], oracle, k5_of(dln, mat), net, rows=rows)


def test_errors(pkg, synth):
    net = _synthetic(pkg, synth, 4, 71)
    dln, mat = _params(pkg)
    with pytest.raises(IndexError):
        pkg.calcSegSegForce(dln, mat, net, [0])
    with pytest.raises(IndexError):
        pkg.calcSegSegForce(dln, mat, net, [net.numSeg + 1])
    bad = pkg.DislocationNetwork(net.coord.copy(), net.bVec, net.segIdx)
    bad.coord[:, 1] = bad.coord[:, 0]
    with pytest.raises(ValueError):
        pkg.calcSegSegForce(dln, mat, bad)
    bad = pkg.DislocationNetwork(net.coord.copy(), net.bVec, net.segIdx)
    bad.coord[0, 3] = np.nan
    with pytest.raises(ValueError):
        pkg.calcSegSegForce(dln, mat, bad)
    bad = pkg.DislocationNetwork(net.coord, net.bVec, net.segIdx.copy(order="F"))
    bad.segIdx[2, 1] = 10 ** 6
    with pytest.raises(IndexError):
        pkg.calcSegSegForce(dln, mat, bad)
    # The context stays usable after rejected calls.
    assert np.isfinite(pkg.calcSegSegForce(dln, mat, net)).all()


def test_device_resident_form(pkg, synth):
    torch = pytest.importorskip("torch")
    p, b = synth.square_loops(70, 81, 20.0, 200.0, 2000.0, 0.5, 0.1)
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    dln, mat = _params(pkg)
    host = pkg.calcSegSegForce(dln, mat, net)
    soa = torch.from_numpy(synth.packed_soa(p, b)).cuda()
    out = torch.zeros(6 * net.numSeg, dtype=torch.float64, device="cuda")
    ctx = pkg.get_context()
    rep = ctx.segseg_force_device(pkg.consts_of(dln, mat), soa.data_ptr(), soa.shape[1], net.numSeg, out.data_ptr(),
                                  stream=torch.cuda.current_stream().cuda_stream, report=True)
    torch.cuda.synchronize()
    dev = out.cpu().numpy().reshape(3, 2, -1, order="F")
    assert np.array_equal(dev, host)
    assert rep["pairs_general"] + rep["pairs_parallel"] == net.numSeg * (net.numSeg - 1) // 2


@pytest.mark.parametrize("num_loops,seed", [(64, 4), (150, 5)])
def test_fma_mode(pkg, synth, oracle, num_loops, seed):
    """DDD_MODE_FP64_FMA: same formulas with fused multiply-adds.  Its rounding
    differs from the reference's arithmetic by up to ~4x that arithmetic's own
    noise (measured: the same happens to the oracle compiled with FMA on a CPU),
    so the bounds are 8x / 6x the noise."""
    net = _synthetic(pkg, synth, num_loops, seed, cube=3000.0)
    dln, mat = _params(pkg)
    ctx = pkg.get_context()
    ctx.mode = "fp64_fma"
    try:
        F = pkg.calcSegSegForce(dln, mat, net)
    finally:
        ctx.mode = "fp64"
    assert ctx.mode == pkg.MODE_FP64
    check_forces(F, oracle, k5_of(dln, mat), net, factor=(8, 6))
    S = pkg.calcSegSegForce(dln, mat, net)
    assert not np.array_equal(F, S)  # a different kernel ran


@pytest.mark.parametrize("num_loops,seed,pf,cube", [(1, 0, 0.05, 3000.0), (17, 2, 0.05, 3000.0),
                                                    (64, 4, 0.05, 3000.0), (150, 5, 0.05, 3000.0),
                                                    (96, 21, 0.5, 1500.0), (300, 7, 0.05, 20000.0)])
def test_fp64_fast_mode(pkg, synth, oracle, num_loops, seed, pf, cube):
    """DDD_MODE_FP64_FAST (one division per corner, table-driven log/atan,
    explicit FMAs where the terms do not cancel; near-parallel branch strict)
    under the same parity bound as the strict kernel: per node
    |ΔF| <= 1e-10 |F| + 4 noise and kernel error <= 3 noise.  The same
    header built for a CPU measures its error at 1.0-1.1x the reference
    arithmetic's own on these networks.  Also: same branch counts as the
    strict kernel, idx and in-place forms, external segments skipped."""
    net = _synthetic(pkg, synth, num_loops, seed, parallel_fraction=pf, cube=cube)
    net.extSeg[::29] = 1
    dln, mat = _params(pkg)
    ctx = pkg.get_context()
    S = pkg.calcSegSegForce(dln, mat, net)
    rep_s = dict(ctx.last_report)
    idx = np.array([1, 5, 5, net.numSeg])
    ctx.mode = "fp64_fast"
    try:
        F = pkg.calcSegSegForce(dln, mat, net)
        rep_f = dict(ctx.last_report)
        Fi = pkg.calcSegSegForce(dln, mat, net, idx)
        assert np.array_equal(pkg.calcSegSegForce(dln, mat, net), F)
    finally:
        ctx.mode = "fp64"
    assert (rep_f["pairs_general"], rep_f["pairs_parallel"]) == (rep_s["pairs_general"], rep_s["pairs_parallel"])
    assert np.all(F[:, :, net.extSeg[:net.numSeg] == 1] == 0)
    k5 = k5_of(dln, mat)
    check_forces(F, oracle, k5, net)
    check_forces(Fi, oracle, k5, net, rows=idx - 1, ref=oracle.segseg_idx(k5, net, idx))
    if num_loops > 1:
        assert not np.array_equal(F, S)  # a different kernel ran


@pytest.mark.parametrize("num_loops,seed,pf", [(64, 4, 0.05), (150, 5, 0.05), (96, 21, 0.5)])
def test_df64_mode(pkg, synth, oracle, num_loops, seed, pf):
    """DDD_MODE_DF64 (double-float general branch, FP64 near-parallel branch and
    accumulation).  Its per-node error is measured at 20-400x the FP64
    arithmetic's own worst error on these networks (the unit roundoff ratio is
    2^6, inputs are rounded to 48 bits, and cancellation amplifies both); the
    same df64 code compiled for a CPU gives the same errors.  Bounds: per node
    1000 x that noise, normwise relative error <= 1e-8; pairs take the FP64
    kernel's branches."""
    net = _synthetic(pkg, synth, num_loops, seed, parallel_fraction=pf, cube=3000.0)
    dln, mat = _params(pkg)
    ctx = pkg.get_context()
    S = pkg.calcSegSegForce(dln, mat, net)
    rep_s = dict(ctx.last_report)
    ctx.mode = "df64"
    try:
        F = pkg.calcSegSegForce(dln, mat, net)
        rep_d = dict(ctx.last_report)
        Fi = pkg.calcSegSegForce(dln, mat, net, [3, 77, 77])
    finally:
        ctx.mode = "fp64"
    assert (rep_d["pairs_general"], rep_d["pairs_parallel"]) == (rep_s["pairs_general"], rep_s["pairs_parallel"])
    check_forces(F, oracle, k5_of(dln, mat), net, factor=(1000, 1000), normwise=1e-8)
    check_forces(Fi, oracle, k5_of(dln, mat), net, rows=[2, 76, 76], factor=(1000, 1000), normwise=1e-8)
    ext = oracle.segseg_ser_ld(k5_of(dln, mat), net, nthreads=os.cpu_count() or 1)
    assert np.linalg.norm(F - ext) <= 1e-8 * np.linalg.norm(ext)


@pytest.mark.parametrize("num_loops,seed,pf,cube", [(64, 4, 0.05, 3000.0), (150, 5, 0.05, 3000.0),
                                                    (300, 7, 0.05, 20000.0)])
def test_f32c_mode(pkg, synth, oracle, num_loops, seed, pf, cube):
    """DDD_MODE_F32C: df64 corner antiderivatives and moments, FP32 assembly.
    Measured (the same code compiled for a CPU) ~5e-8 normwise relative error
    against the long-double evaluation; bounds: normwise <= 2e-7, per node
    |ΔF_n| <= 1e-4 |F_n| + 1e-6 max|F|; same branches as the FP64 kernel."""
    net = _synthetic(pkg, synth, num_loops, seed, parallel_fraction=pf, cube=cube)
    dln, mat = _params(pkg)
    ctx = pkg.get_context()
    pkg.calcSegSegForce(dln, mat, net)
    rep_s = dict(ctx.last_report)
    ctx.mode = "f32c"
    try:
        F = pkg.calcSegSegForce(dln, mat, net)
        rep_c = dict(ctx.last_report)
        Fi = pkg.calcSegSegForce(dln, mat, net, [5, 9, 9])
    finally:
        ctx.mode = "fp64"
    assert (rep_c["pairs_general"], rep_c["pairs_parallel"]) == (rep_s["pairs_general"], rep_s["pairs_parallel"])
    ext = oracle.segseg_ser_ld(k5_of(dln, mat), net, nthreads=os.cpu_count() or 1)
    nrm = lambda a: np.linalg.norm(a, axis=0)
    if os.environ.get("DDD_TEST_STATS"):
        with open(os.environ["DDD_TEST_STATS"], "a") as fh:
            fh.write("f32c n=%d normwise=%.3e max_node_over_max=%.3e\n" % (
                net.numSeg, np.linalg.norm(F - ext) / np.linalg.norm(ext), nrm(F - ext).max() / nrm(ext).max()))
    assert np.linalg.norm(F - ext) <= 2e-7 * np.linalg.norm(ext)
    assert np.all(nrm(F - ext) <= 1e-4 * nrm(ext) + 1e-6 * nrm(ext).max())
    exti = ext[:, :, [4, 8, 8]]
    assert np.all(nrm(Fi - exti) <= 1e-4 * nrm(exti) + 1e-6 * nrm(ext).max())


@pytest.mark.parametrize("mode", ["fp64", "fp64_fma", "fp64_fast", "df64", "f32c"])
def test_banded_partial_sums(pkg, synth, oracle, mode):
    """A partial-sum limit below the all-pairs slot count (4,800 segments: 38
    tiles, 741 tile pairs of 12,288 bytes) makes the launchers run bands of
    tile columns: 100 slots (bands of 1-14 columns) and the minimum (one column
    of 38 slots, 1 byte asked).  The band sums regroup the same FP64 additions,
    so the forces equal the unbanded ones to rounding, repeat bit for bit, and
    in the reference's arithmetic stay within the oracle bounds; the
    device-resident entry point bands the same way.  The idx form under the
    same limits runs its rows in chunks of row tiles: bit-identical."""
    net = _synthetic(pkg, synth, 600, 7)
    assert net.numSeg == 4800
    dln, mat = _params(pkg)
    ctx = pkg.get_context()
    assert ctx.partial_limit == 16 << 30
    ctx.mode = mode
    idx = np.random.default_rng(2).integers(1, net.numSeg + 1, 700)
    try:
        F = pkg.calcSegSegForce(dln, mat, net)
        Fi = pkg.calcSegSegForce(dln, mat, net, idx)
        for limit in (100 * 12288, 1):
            ctx.partial_limit = limit
            Fb = pkg.calcSegSegForce(dln, mat, net)
            assert np.linalg.norm(Fb - F) <= 1e-13 * np.linalg.norm(F)
            assert np.array_equal(pkg.calcSegSegForce(dln, mat, net), Fb)
            # The idx form in chunks of whole row tiles (5 and 1 of the 6):
            # each row's sum is unchanged, bit for bit.
            assert np.array_equal(pkg.calcSegSegForce(dln, mat, net, idx), Fi)
            if mode == "fp64":
                check_forces(Fb, oracle, k5_of(dln, mat), net)
                torch = pytest.importorskip("torch")
                rows9 = np.r_[net.coord[:, net.segIdx[:, 1] - 1], net.coord[:, net.segIdx[:, 2] - 1], net.bVec]
                soa = torch.from_numpy(np.ascontiguousarray(rows9)).cuda()  # 9 x numSeg, row-major
                out = torch.zeros(6 * net.numSeg, dtype=torch.float64, device="cuda")
                ctx.segseg_force_device(pkg.consts_of(dln, mat), soa.data_ptr(), soa.shape[1], net.numSeg,
                                        out.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
                torch.cuda.synchronize()
                assert np.array_equal(out.cpu().numpy().reshape(3, 2, -1, order="F"), Fb)
    finally:
        ctx.partial_limit = 0
        ctx.mode = "fp64"
    assert ctx.partial_limit == 16 << 30
    with pytest.raises(ValueError):
        ctx.partial_limit = -1


def test_concurrent_host_threads(pkg, synth):
    """Host threads calling at once (ctypes releases the GIL): four threads on
    the shared context (its mutex serialises them) and two on contexts of their
    own, each mixing the all-pairs, idx and σ̃ forms; every result is the
    single-threaded one, bit for bit."""
    import threading

    net = _synthetic(pkg, synth, 300, 31)
    dln, mat = _params(pkg)
    pts = synth.grid_points(8, 20000.0)
    idx = [3, 1, net.numSeg, 3]
    want = (pkg.calcSegSegForce(dln, mat, net), pkg.calcSegSegForce(dln, mat, net, idx),
            pkg.calc_σTilde(pts, dln, mat, net))
    k = pkg.consts_of(dln, mat)
    own = [pkg.Context(0), pkg.Context(0)]
    ctxs = [pkg.get_context()] * 4 + own
    got, errors = [None] * len(ctxs), []

    def work(t):
        try:
            c = ctxs[t]
            res = []
            for _ in range(3):
                res.append((c.segseg_force(k, net), c.segseg_force(k, net, idx), c.sigma_tilde(k, pts, net)))
            got[t] = res
        except Exception as e:  # reported below, on the main thread
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(t,)) for t in range(len(ctxs))]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=300)
    for c in own:
        c.close()
    assert not errors, errors
    for res in got:
        for F, Fi, S in res:
            assert np.array_equal(F, want[0]) and np.array_equal(Fi, want[1]) and np.array_equal(S, want[2])
