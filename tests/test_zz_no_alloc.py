"""The allocation-free entry point ddd_segseg_force_device_noalloc.

It serves callers that cannot let this library allocate device memory (an
application whose GPU memory belongs to its own pool allocator, or a
time-stepping loop that cannot afford cudaMalloc/cudaFree's device-wide
synchronisation).  Its scratch is a fixed device array shared by every call,
so this test calls it twice in a row — a large network and then a smaller
one, so stale scratch from the first call would show — and compares each
result with the existing entry point's (ddd_segseg_force_device) within the
parity tolerance of the other GPU tests: per node force
|ΔF| <= 1e-10 |F| + 1e-12 max|F|.  It also checks the size limit.

This file is collected last so a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(a, b):
    a = a.reshape(3, 2, -1, order="F")
    b = b.reshape(3, 2, -1, order="F")
    d = np.linalg.norm(a - b, axis=0)
    n = np.linalg.norm(b, axis=0)
    assert np.all(d <= 1e-10 * n + 1e-12 * n.max()), np.max(d / (n + 1e-300))


def test_noalloc_matches_device_entry_point_twice(pkg, synth):
    torch = pytest.importorskip("torch")
    L = pkg.library()
    ctx = pkg.get_context()
    dln = pkg.DislocationParameters(coreRad=1.0)
    mat = pkg.MaterialParameters(mu=1.0, nu=0.28)
    k = pkg.consts_of(dln, mat)
    stream = torch.cuda.current_stream()
    for loops, seed in ((512, 11), (37, 12)):  # 4096 segments (the limit), then 296
        p, b = synth.square_loops(loops, seed, 20.0, 200.0, 3000.0, 0.5, 0.1)
        n = loops * 8
        soa = torch.from_numpy(synth.packed_soa(p, b)).cuda()
        ext = torch.zeros(n, dtype=torch.uint8, device="cuda")
        ext[::13] = 1
        ref = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
        ctx.segseg_force_device(k, soa.data_ptr(), n, n, ref.data_ptr(), ext_ptr=ext.data_ptr(),
                                stream=stream.cuda_stream)
        out = torch.full((6 * n,), float("nan"), dtype=torch.float64, device="cuda")
        rc = L.ddd_segseg_force_device_noalloc(ctypes.byref(k), soa.data_ptr(), n, ext.data_ptr(), n, out.data_ptr(),
                                               stream.cuda_stream)
        assert rc == pkg.DDD_OK
        torch.cuda.synchronize()
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all()
        _close(got, want)


def test_noalloc_rejects_sizes_beyond_limit(pkg):
    torch = pytest.importorskip("torch")
    L = pkg.library()
    k = pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))
    n = pkg.NOALLOC_MAX_SEGMENTS + 1
    segs = torch.zeros((9, n), dtype=torch.float64, device="cuda")
    out = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    rc = L.ddd_segseg_force_device_noalloc(ctypes.byref(k), segs.data_ptr(), n, None, n, out.data_ptr(), None)
    assert rc == pkg.DDD_ETOOBIG
