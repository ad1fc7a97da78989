"""Surrogate force path (ddd_surrogate_force) on the GPU.

Partition: every unordered pair of active segments is evaluated once, either by
the network (R^2 >= kappa^2 max(L_i, L_j)^2, FP32 test) or exactly (all other
pairs).  Checked three ways:
  * network output forced to zero: the result must be the exact forces of the
    near pairs alone, summed here with the CPU oracle over the pairs that the
    same FP32 test (restated in numpy, identical rounding) calls near;
  * kappa so large that every pair is near: the result must be the exact FP64
    all-pairs forces (the library's FP64 path and the oracle);
  * an untrained network: the audit sees a large error and the call falls back
    to the exact forces.
Accuracy and speed with a trained network: node-force relative RMS error
against the exact FP64 forces below 5e-4 on a 32,768-segment network the
network never saw, and at least 5x faster than the exact FP64 path there.

Tolerances of the exact parts: the near pass computes each pair with the same
FP64 code as the exact kernel (strict rounding), but after the Morton sort a
pair may be evaluated with its two segments' roles swapped, and CUDA's and the C
library's log / atan differ by an ulp; both change the rounding at the level of
the algorithm's own FP64 noise, amplified by the cancellation in node sums.  So
the all-pairs comparison uses the FP64 parity check of test_segseg_gpu (per
node: 1e-10 |F| + 4 x the long-double-measured noise; normwise 3e-10), and the
near-pairs comparison ||dF|| <= 1e-10 ||F||, per node <= 1e-9 max |F|.
"""
import os
import time

import numpy as np
import pytest

from conftest import k5_of
from test_segseg_gpu import check_forces

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _params(pkg):
    return pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28)


def _k(pkg):
    return pkg.consts_of(*_params(pkg))


def _network(pkg, synth, loops, seed, cube=20000.0, config="gpu32k"):
    cfg = synth.CONFIGS[config]
    p, b = synth.square_loops(loops, seed, cfg["lmin"], cfg["lmax"], cube, cfg["shear_fraction"],
                              cfg["parallel_fraction"])
    coord, bvec, seg = synth.network_arrays(p, b)
    return pkg.DislocationNetwork(coord, bvec, seg), synth.packed_soa(p, b)


def _exact_device(pkg, segs, ext=None):
    ctx = pkg.get_context()
    k = _k(pkg)
    n = segs.shape[1]
    d = torch.from_numpy(segs).cuda()
    e = torch.from_numpy(ext).cuda() if ext is not None else None
    out = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.segseg_force_device(k, d.data_ptr(), n, n, out.data_ptr(), e.data_ptr() if e is not None else None)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _near_mask_rows(segs, kappa):
    """Per row i, the columns j > i that the FP32 trust-region test calls near
    (the library's pair_is_far, restated with numpy float32 rounding)."""
    n1, n2 = segs[0:3], segs[3:6]
    m = (0.5 * (n1 + n2)).astype(np.float32)
    t = n2 - n1
    tN = 1.0 / np.sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2])
    L = (1.0 / tN).astype(np.float32)
    k2 = np.float32(kappa) * np.float32(kappa)
    n = segs.shape[1]
    for i in range(n - 1):
        j = np.arange(i + 1, n)
        dx = m[0, j] - m[0, i]
        dy = m[1, j] - m[1, i]
        dz = m[2, j] - m[2, i]
        R2 = (dx * dx + dy * dy) + dz * dz
        Lm = np.maximum(L[j], L[i])
        yield i, j[~(R2 >= k2 * (Lm * Lm))]


def _zero_surrogate(pkg):
    sur = pkg.Surrogate(pkg.get_context(), seed=0)
    sur.set_params(np.zeros(sur.num_params, np.float32))
    return sur


def test_zero_network_leaves_exact_near_pairs(pkg, synth, oracle):
    dln, mat = _params(pkg)
    k5 = k5_of(dln, mat)
    net, segs = _network(pkg, synth, 256, seed=31, cube=8000.0)
    sur = _zero_surrogate(pkg)
    F, rep = sur.force(_k(pkg), segs, kappa=20.0, audit_fraction=0.0)
    F = F.cpu().numpy()
    ref = np.zeros_like(F)
    near = 0
    for i, js in _near_mask_rows(segs, 20.0):
        for j in js:
            f = oracle.pair(k5, segs[6:9, i], segs[0:3, i], segs[3:6, i], segs[6:9, j], segs[0:3, j],
                            segs[3:6, j]).ravel()
            ref[i] += f[0:6]
            ref[j] += f[6:12]
            near += 1
    assert near > 1000  # the network places both near and far pairs
    assert rep["pairs_near_general"] + rep["pairs_near_parallel"] == near
    assert rep["pairs_total"] == segs.shape[1] * (segs.shape[1] - 1) // 2
    assert np.linalg.norm(F - ref) <= 1e-10 * np.linalg.norm(ref)
    assert np.abs(F - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("with_ext", [False, True])
def test_all_pairs_near_is_exact(pkg, synth, oracle, with_ext):
    dln, mat = _params(pkg)
    net, segs = _network(pkg, synth, 300, seed=32, cube=6000.0)  # 2,400 segments: padded last tile
    n = segs.shape[1]
    ext = (np.arange(n) % 7 == 3).astype(np.uint8) if with_ext else None
    sur = _zero_surrogate(pkg)
    F, rep = sur.force(_k(pkg), segs, ext=ext, kappa=1e30, audit_fraction=0.0)
    F = F.cpu().numpy()
    na = n - (int(ext.sum()) if with_ext else 0)
    assert rep["pairs_near_general"] + rep["pairs_near_parallel"] == na * (na - 1) // 2
    ex = _exact_device(pkg, segs, ext)
    assert np.linalg.norm(F - ex) <= 3e-10 * np.linalg.norm(ex)
    if with_ext:
        assert np.all(F[ext == 1] == 0.0)
        net.extSeg[:] = ext
    F3 = np.asfortranarray(F.reshape(n, 2, 3).transpose(2, 1, 0))
    check_forces(F3, oracle, k5_of(dln, mat), net, normwise=3e-10)


@pytest.mark.parametrize("mode", ["f32c", "df64"])
def test_all_pairs_near_precision_forms(pkg, synth, mode):
    # The exact passes in the df64 / f32c arithmetic (the general branch in
    # double-float; branch decision and near-parallel branch FP64): every pair
    # near, against the library's FP64 path.  Bound: those forms' measured error
    # (~5e-8 relative RMS for f32c) with margin.
    net, segs = _network(pkg, synth, 300, seed=35, cube=6000.0)
    sur = _zero_surrogate(pkg)
    F, rep = sur.force(_k(pkg), segs, kappa=1e30, audit_fraction=0.0, exact_mode=mode)
    n = segs.shape[1]
    assert rep["pairs_near_general"] + rep["pairs_near_parallel"] == n * (n - 1) // 2
    ex = _exact_device(pkg, segs)
    assert np.linalg.norm(F.cpu().numpy() - ex) <= 1e-6 * np.linalg.norm(ex)


def test_untrained_network_falls_back_to_exact(pkg, synth, oracle):
    # Sparse network: mostly far pairs, whose FP64 evaluation cancels strongly,
    # so the per-node bound (long-double-calibrated noise) carries the check.
    dln, mat = _params(pkg)
    net, segs = _network(pkg, synth, 512, seed=33, cube=10000.0)
    n = segs.shape[1]
    sur = pkg.Surrogate(pkg.get_context(), seed=5)
    flat = sur.params()
    o4 = pkg._PARAM_OFF["b4"][0]
    flat[o4:o4 + 108] = 10.0  # a network far off the true coefficients
    sur.set_params(flat)
    F, rep = sur.force(_k(pkg), segs, kappa=20.0, audit_fraction=0.05, audit_tol=1e-3)
    assert rep["tiles_audit"] > 0 and rep["audit_node_rel_rms"] > 1e-3
    assert rep["fallback"] == 1
    F3 = np.asfortranarray(F.cpu().numpy().reshape(n, 2, 3).transpose(2, 1, 0))
    check_forces(F3, oracle, k5_of(dln, mat), net, normwise=1e-8)


@pytest.fixture(scope="module")
def trained(pkg, synth):
    sur = pkg.Surrogate(pkg.get_context(), seed=1)
    cfg = synth.CONFIGS["gpu32k"]
    nets = [synth.packed_soa(*synth.square_loops(4096, s, cfg["lmin"], cfg["lmax"], cfg["cube"],
                                                  cfg["shear_fraction"], cfg["parallel_fraction"]))
            for s in (101, 102)]
    info = sur.fit(_k(pkg), nets, pairs_per_network=1 << 20, epochs=10, batch=4096, lr=2e-3, kappa=20.0, seed=3)
    assert np.all(np.isfinite(info["loss"])) and info["loss"][-1] < 0.05 * info["loss"][0]
    return sur


def test_trained_surrogate_accuracy_and_gain(pkg, synth, trained):
    net, segs = _network(pkg, synth, 4096, seed=0)  # 32,768 segments, not in the training set
    k = _k(pkg)
    ctx = pkg.get_context()
    d = torch.from_numpy(segs).cuda()
    n = segs.shape[1]
    ex = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.segseg_force_device(k, d.data_ptr(), n, n, ex.data_ptr())
    torch.cuda.synchronize()
    t_exact = time.perf_counter() - t0
    F, rep = trained.force(k, d)  # first call: plan set-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    F, rep = trained.force(k, d)
    torch.cuda.synchronize()
    t_sur = time.perf_counter() - t0
    err = (torch.linalg.norm(F - ex) / torch.linalg.norm(ex)).item()
    if os.environ.get("DDD_TEST_STATS"):
        with open(os.environ["DDD_TEST_STATS"], "a") as fh:
            fh.write("surrogate 32k: rel rms %.3e audit %.3e/%.3e exact %.3f s surrogate %.3f s %s\n"
                     % (err, rep["audit_rel_rms"], rep["audit_rel_max"], t_exact, t_sur, rep))
    assert rep["fallback"] == 0
    assert err < 5e-4, err
    # The audit's node-level estimate is of the right size.
    assert err / 4 < rep["audit_node_rel_rms"] < 4 * err
    assert t_exact / t_sur > 5.0, (t_exact, t_sur)
    F2, _ = trained.force(k, d)
    assert torch.equal(F, F2)  # deterministic


def test_committed_checkpoint_gain_over_f32c_exact(pkg, synth):
    """What the learned part gains over the method without it.  The committed
    checkpoint (trained on four other networks of the workload's generator)
    on a 32,768-segment network of that generator: the surrogate with f32c
    exact passes must beat the f32c exact kernel alone (the same arithmetic
    for every pair, no network) in device time, at <= 1e-4 node-force relative
    RMS error against the strict FP64 forces (the bench measures ~3x at 65,536
    segments, 2.5e-5)."""
    import ddd_gb300

    path = os.path.join(os.path.dirname(ddd_gb300.__file__), "data", "surrogate_gpu65k_nu028.bin")
    ctx = pkg.get_context()
    sur = pkg.Surrogate(ctx, seed=0).load(path)
    net, segs = _network(pkg, synth, 4096, seed=0)
    k = _k(pkg)
    n = segs.shape[1]
    d = torch.from_numpy(segs).cuda()
    ref = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    ctx.segseg_force_device(k, d.data_ptr(), n, n, ref.data_ptr())
    ex = torch.zeros_like(ref)
    # A stream of its own: torch's default stream has handle 0, which the
    # library reads as "its own stream", and the events would time nothing.
    st = torch.cuda.Stream()
    torch.cuda.synchronize()

    def timed(fn, reps=2):
        with torch.cuda.stream(st):
            fn()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            for _ in range(reps):
                fn()
            b.record(st)
            torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    ctx.mode = "f32c"
    try:
        ms_f32c = timed(lambda: ctx.segseg_force_device(k, d.data_ptr(), n, n, ex.data_ptr(),
                                                        stream=st.cuda_stream))
    finally:
        ctx.mode = "fp64"
    out = {}

    def run_sur():
        out["F"], out["rep"] = sur.force(k, d, exact_mode="f32c", stream=st.cuda_stream)

    ms_sur = timed(run_sur)
    err = (torch.linalg.norm(out["F"] - ref) / torch.linalg.norm(ref)).item()
    err_f32c = (torch.linalg.norm(ex - ref) / torch.linalg.norm(ref)).item()
    if os.environ.get("DDD_TEST_STATS"):
        with open(os.environ["DDD_TEST_STATS"], "a") as fh:
            fh.write("gain over f32c exact: %.1f ms vs %.1f ms, err %.3e (f32c %.3e)\n" % (ms_sur, ms_f32c, err,
                                                                                         err_f32c))
    assert out["rep"]["fallback"] == 0
    assert err <= 1e-4, err
    assert ms_sur < ms_f32c, (ms_sur, ms_f32c)

    # The far pairs by quadrature instead of the network (3 points): faster than
    # f32c exact as well, and closer to the strict FP64 forces.
    def run_quad():
        out["Fq"], out["repq"] = sur.force(k, d, exact_mode="f32c", stream=st.cuda_stream, far="quad3")

    ms_quad = timed(run_quad)
    err_q = (torch.linalg.norm(out["Fq"] - ref) / torch.linalg.norm(ref)).item()
    assert out["repq"]["fallback"] == 0
    assert err_q <= 1e-6, err_q
    assert ms_quad < ms_f32c, (ms_quad, ms_f32c)


@pytest.mark.parametrize("exact_mode,far,kappa,kappa_two,rel_max", [("fp64", "quad3", None, None, 1e-8),
                                                                   ("fp64", "quad3", None, 0.0, 1e-8),
                                                                   ("fp64_fast", "quad3", None, None, 1e-8),
                                                                   ("fp64_fast", "quad3", 20.0, None, 1e-8),
                                                                   ("f32c", "quad3", None, None, 1e-6),
                                                                   ("fp64", "quad2", None, None, 1e-6)])
def test_quadrature_far_field(pkg, synth, oracle, exact_mode, far, kappa, kappa_two, rel_max):
    """far = "quad3" / "quad2": far pairs by FP32 Gauss-Legendre quadrature on
    both segments (no network), near pairs exact; near-parallel far pairs take
    the reference's projected geometry first.  On a 12,000-segment network of
    the workload's generator (mostly far pairs), against the long-double
    evaluation of the reference's formulas on 96 sampled segments: relative
    RMS <= 1e-8 with 3 points and FP64 near pairs, strict or fast (the CPU
    build of the same code measures ~3e-10), <= 1e-6 with f32c near pairs (their own ~2e-7) or 2
    points; per node <= 1e-4 |F| + 1e-6 max|F|.  The default trust factor is
    10 lengths for 3 points and 20 for 2 (the 3-point rule is at its FP32
    noise level from 8); 20 with 3 points is checked too.  "quad3" switches
    32-pair steps whose far pairs all lie beyond 30 lengths to 2 points by
    default (kappa_two); 0 keeps 3 points everywhere.  The result does not
    depend on the network's weights, every pair is counted once, and repeats
    are bit-equal."""
    dln, mat = _params(pkg)
    net, segs = _network(pkg, synth, 1500, seed=41)
    n = segs.shape[1]
    k, k5 = _k(pkg), k5_of(dln, mat)
    sur = pkg.Surrogate(pkg.get_context(), seed=0)  # untrained: not used by the quadrature
    F, rep = sur.force(k, segs, far=far, exact_mode=exact_mode, audit_fraction=0.02, kappa=kappa, kappa_two=kappa_two)
    assert rep["fallback"] == 0 and rep["pairs_total"] == n * (n - 1) // 2
    assert rep["pairs_near_general"] + rep["pairs_near_parallel"] < rep["pairs_total"] // 10
    flat = sur.params()
    sur.set_params(np.full_like(flat, 3.0))
    F2, _ = sur.force(k, segs, far=far, exact_mode=exact_mode, audit_fraction=0.02, kappa=kappa, kappa_two=kappa_two)
    assert torch.equal(F, F2)
    F3 = np.asfortranarray(F.cpu().numpy().reshape(n, 2, 3).transpose(2, 1, 0))
    rows = np.sort(np.random.default_rng(5).choice(n, 96, replace=False))
    ext = oracle.segseg_ser_ld(k5, net, rows, nthreads=os.cpu_count() or 1)
    G = F3[:, :, rows]
    nrm = lambda a: np.linalg.norm(a, axis=0)
    rel = np.linalg.norm(G - ext) / np.linalg.norm(ext)
    if os.environ.get("DDD_TEST_STATS"):
        with open(os.environ["DDD_TEST_STATS"], "a") as fh:
            fh.write("quadrature %s %s: rel rms %.3e max node %.3e audit %.3e %s\n" % (
                far, exact_mode, rel, (nrm(G - ext) / nrm(ext)).max(), rep["audit_node_rel_rms"], rep))
    assert rel <= rel_max, rel
    assert np.all(nrm(G - ext) <= 1e-4 * nrm(ext) + 1e-6 * nrm(ext).max())


def test_quadrature_two_point_switch(pkg, synth):
    """The 3-point far pass's switch to 2 points (kappa_two): with the default
    30 lengths it changes the forces (some 32-pair steps lie that far out on
    this 12,000-segment network) by far less than the quadrature's own error
    (relative RMS <= 1e-8 against kappa_two = 0); a threshold no pair reaches
    gives the 3-point result bit for bit, and 2-point-only runs (far_mode 2)
    do not depend on it.  A negative or non-finite kappa_two is refused."""
    net, segs = _network(pkg, synth, 1500, seed=41)
    k = _k(pkg)
    sur = pkg.Surrogate(pkg.get_context(), seed=0)
    F0, _ = sur.force(k, segs, far="quad3", exact_mode="fp64", audit_fraction=0.0, kappa_two=0.0)
    F30, _ = sur.force(k, segs, far="quad3", exact_mode="fp64", audit_fraction=0.0, kappa_two=30.0)
    Fbig, _ = sur.force(k, segs, far="quad3", exact_mode="fp64", audit_fraction=0.0, kappa_two=1e12)
    assert torch.equal(F0, Fbig)
    assert not torch.equal(F0, F30)
    assert (torch.linalg.norm(F30 - F0) / torch.linalg.norm(F0)).item() <= 1e-8
    G0, _ = sur.force(k, segs, far="quad2", exact_mode="fp64", audit_fraction=0.0, kappa_two=0.0)
    G1, _ = sur.force(k, segs, far="quad2", exact_mode="fp64", audit_fraction=0.0, kappa_two=30.0)
    assert torch.equal(G0, G1)
    for bad in (-1.0, float("inf"), float("nan")):
        with pytest.raises(pkg.DDDError):
            sur.force(k, segs, far="quad3", exact_mode="fp64", audit_fraction=0.0, kappa_two=bad)


def test_host_array_entry_matches_device_form(pkg, synth, trained):
    # ddd_surrogate_force_host takes the network's own arrays (the
    # ddd_segseg_force layout, extSeg per segment row): same result, bit for bit.
    dln, mat = _params(pkg)
    net, segs = _network(pkg, synth, 700, seed=36)
    n = segs.shape[1]
    ext = (np.arange(n) % 11 == 5).astype(np.uint8)
    net.extSeg[:] = ext
    Fh, rep_h = trained.force_network(dln, mat, net)
    Fd, rep_d = trained.force(_k(pkg), segs, ext=ext)
    assert np.array_equal(Fh, np.asfortranarray(Fd.cpu().numpy().reshape(n, 2, 3).transpose(2, 1, 0)))
    assert rep_h["pairs_total"] == rep_d["pairs_total"] == (n - int(ext.sum())) * (n - int(ext.sum()) - 1) // 2
    assert np.all(Fh[:, :, ext == 1] == 0.0)
    bad = pkg.DislocationNetwork(net.coord, net.bVec, net.segIdx.copy())
    bad.segIdx[3, 1] = 10 ** 7
    with pytest.raises(pkg.DDDError):
        trained.force_network(dln, mat, bad)


def test_checkpoint_round_trip(pkg, synth, trained, tmp_path):
    path = str(tmp_path / "sur.bin")
    trained.save(path)
    other = pkg.Surrogate(pkg.get_context(), seed=9).load(path)
    assert np.array_equal(other.params(), trained.params())
    assert other.kappa == trained.kappa and other.nu == trained.nu
    net, segs = _network(pkg, synth, 512, seed=34)
    a, _ = trained.force(_k(pkg), segs)
    b, _ = other.force(_k(pkg), segs)
    assert torch.equal(a, b)
    raw = bytearray(open(path, "rb").read())
    raw[100] ^= 1
    open(path, "wb").write(bytes(raw))
    with pytest.raises(pkg.DDDError):
        pkg.Surrogate(pkg.get_context(), seed=9).load(path)
    # A network trained for another Poisson ratio is refused.
    k = pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.3))
    with pytest.raises(pkg.DDDError):
        trained.force(k, segs)


def test_quadrature_many_near_parallel_far_pairs(pkg, oracle):
    """256 exactly parallel 20 b segments on two ladders (y = 300 b k, z = 0
    and 400 b): every pair is far (R >= 15 L) and near-parallel, so every
    force comes from the quadrature of the reference's projected geometry, and
    the tile pair between the two sorted tiles holds 16,384 such pairs, more
    than one round of the far pass's near-parallel list (8,192).  Against the
    oracle's FP64 forces: relative RMS <= 1e-6, per node <= 1e-4 |F| + 1e-6
    max |F|, no near pair, every pair counted once."""
    n = 256
    coord = np.zeros((3, 2 * n))
    for s in range(n):
        y, z = 300.0 * (s % 128), (0.0 if s < 128 else 400.0)
        coord[:, 2 * s] = [0.0, y, z]
        coord[:, 2 * s + 1] = [20.0, y, z]
    bv = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0)
    bvec = np.asfortranarray(np.tile(bv[:, None], (1, n)))
    seg = np.asfortranarray(np.array([[s + 1, 2 * s + 1, 2 * s + 2] for s in range(n)], dtype=np.int64))
    net = pkg.DislocationNetwork(np.asfortranarray(coord), bvec, seg)
    segs = np.zeros((9, n))
    for s in range(n):
        segs[0:3, s] = coord[:, 2 * s]
        segs[3:6, s] = coord[:, 2 * s + 1]
        segs[6:9, s] = bv
    dln, mat = _params(pkg)
    sur = pkg.Surrogate(pkg.get_context(), seed=0)
    F, rep = sur.force(_k(pkg), np.ascontiguousarray(segs), far="quad3", exact_mode="fp64", audit_fraction=0.0)
    assert rep["pairs_total"] == n * (n - 1) // 2
    assert rep["pairs_near_general"] + rep["pairs_near_parallel"] == 0
    G = np.asfortranarray(F.cpu().numpy().reshape(n, 2, 3).transpose(2, 1, 0))
    ref = oracle.segseg_ser(k5_of(dln, mat), net)
    nrm = lambda a: np.linalg.norm(a, axis=0)
    assert np.linalg.norm(G - ref) <= 1e-6 * np.linalg.norm(ref)
    assert np.all(nrm(G - ref) <= 1e-4 * nrm(ref) + 1e-6 * nrm(ref).max())
