"""Batched form: many networks in one persistent launch replayed from a CUDA graph.

With the default configuration (tile 128, no tuning) the batched forces equal
the per-network calls bit for bit (same tile body, same reduction order, same
arithmetic).  With the autotuner the tile size may change, which changes only
the summation blocking: the result must stay within the FP64 parity bound.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES_LOOPS = [0, 1, 3, 17, 90, 40, 8, 30]  # loops per network (8 segments each); includes an empty network


def _batch(pkg, synth, seed=0):
    torch = pytest.importorskip("torch")
    nets = [synth.square_loops(max(nl, 1), seed * 100 + i, 20.0, 200.0, 3000.0, 0.5, 0.1) for i, nl in
            enumerate(SIZES_LOOPS)]
    sizes = [8 * nl for nl in SIZES_LOOPS]
    packed = [synth.packed_soa(p, b)[:, :8 * nl] for (p, b), nl in zip(nets, SIZES_LOOPS)]
    segs = np.ascontiguousarray(np.concatenate(packed, axis=1))
    ext = np.zeros(segs.shape[1], np.uint8)
    ext[::11] = 1
    return torch, sizes, segs, ext


def _per_network(pkg, ctx, k, torch, sizes, segs, ext):
    out, off = [], 0
    for n in sizes:
        if n == 0:
            out.append(np.zeros(0))
            continue
        s = torch.from_numpy(np.ascontiguousarray(segs[:, off:off + n])).cuda()
        e = torch.from_numpy(np.ascontiguousarray(ext[off:off + n])).cuda()
        f = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
        ctx.segseg_force_device(k, s.data_ptr(), n, n, f.data_ptr(), ext_ptr=e.data_ptr())
        torch.cuda.synchronize()
        out.append(f.cpu().numpy())
        off += n
    return np.concatenate(out)


@pytest.mark.parametrize("mode", ["fp64", "fp64_fast", "df64", "f32c"])
def test_batched_equals_per_network(pkg, synth, mode):
    ctx = pkg.get_context()
    k = pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))
    torch, sizes, segs, ext = _batch(pkg, synth)
    ctx.mode = mode
    try:
        ref = _per_network(pkg, ctx, k, torch, sizes, segs, ext)
    finally:
        ctx.mode = "fp64"
    b = pkg.Batch(ctx, sizes, mode=mode, tune=False)
    dsegs = torch.from_numpy(segs).cuda()
    dext = torch.from_numpy(ext).cuda()
    force = torch.full((6 * segs.shape[1],), float("nan"), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    b.run(k, dsegs.data_ptr(), force.data_ptr(), ext_ptr=dext.data_ptr(), stream=st)
    b.run(k, dsegs.data_ptr(), force.data_ptr(), ext_ptr=dext.data_ptr(), stream=st)  # graph replay
    torch.cuda.synchronize()
    got = force.cpu().numpy()
    assert np.array_equal(got, ref)
    info = b.info()
    assert info["tile"] == 128 and info["graph_launches"] == 2 and info["total_segments"] == segs.shape[1]


def test_batched_autotune(pkg, synth):
    ctx = pkg.get_context()
    k = pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))
    torch, sizes, segs, ext = _batch(pkg, synth, seed=3)
    ref = _per_network(pkg, ctx, k, torch, sizes, segs, ext)
    b = pkg.Batch(ctx, sizes, mode="fp64", tune=True)
    dsegs = torch.from_numpy(segs).cuda()
    dext = torch.from_numpy(ext).cuda()
    force = torch.zeros(6 * segs.shape[1], dtype=torch.float64, device="cuda")
    b.run(k, dsegs.data_ptr(), force.data_ptr(), ext_ptr=dext.data_ptr())
    torch.cuda.synchronize()
    info = b.info()
    assert info["tile"] in (64, 128)
    assert all(t > 0 for t in info["tune_ms"])
    got = force.cpu().numpy().reshape(3, 2, -1, order="F")
    want = ref.reshape(3, 2, -1, order="F")
    d = np.linalg.norm(got - want, axis=0)
    n = np.linalg.norm(want, axis=0)
    assert np.all(d <= 1e-10 * n + 1e-12 * n.max())
    # A second plan for the same sizes and mode reuses the tuned choice.
    b2 = pkg.Batch(ctx, sizes, mode="fp64", tune=True)
    b2.run(k, dsegs.data_ptr(), force.data_ptr(), ext_ptr=dext.data_ptr())
    torch.cuda.synchronize()
    assert b2.info()["tile"] == info["tile"] and b2.info()["tune_ms"][0] == -1.0
