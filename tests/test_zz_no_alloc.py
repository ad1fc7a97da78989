"""The allocation-free entry point ddd_segseg_force_device_noalloc.

It serves callers that cannot let this library allocate device memory (an
application whose GPU memory belongs to its own pool allocator, or a
time-stepping loop that cannot afford cudaMalloc/cudaFree's device-wide
synchronisation).  Its scratch is a fixed device array shared by every call,
so this test calls it twice in a row — a large network and then a smaller
one, so stale scratch from the first call would show — and compares each
result with the existing entry point's (ddd_segseg_force_device).  Both run
the same strict FP64 kernels in the same order on the same inputs, with the
context in its default FP64 mode, so the results must be equal bit for bit.
It also checks the set-up call (numSeg = 0), the NULL ext / NULL (legacy
default) stream form, that a second call leaves the device's free memory
unchanged, the size limit and the constants' checks.

This file is collected last so a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _consts(pkg):
    return pkg.consts_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))


def test_noalloc_matches_device_entry_point_twice(pkg, synth):
    torch = pytest.importorskip("torch")
    L = pkg.library()
    ctx = pkg.get_context()
    assert ctx.mode == pkg.MODE_FP64
    k = _consts(pkg)
    stream = torch.cuda.current_stream()
    # Set-up call: loads the scratch and the kernels on this device, launches nothing.
    assert L.ddd_segseg_force_device_noalloc(ctypes.byref(k), None, 0, None, 0, None, None) == pkg.DDD_OK
    cases = []
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
        cases.append((n, soa, ext, ref, out))
    torch.cuda.synchronize()
    free_before = None
    for call, (n, soa, ext, ref, out) in enumerate(cases):
        rc = L.ddd_segseg_force_device_noalloc(ctypes.byref(k), soa.data_ptr(), n, ext.data_ptr(), n, out.data_ptr(),
                                               stream.cuda_stream)
        assert rc == pkg.DDD_OK
        torch.cuda.synchronize()
        if call == 0:
            free_before = torch.cuda.mem_get_info()[0]
        else:  # the second call reserved no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.array_equal(got, want)


def test_noalloc_null_ext_and_default_stream(pkg, synth):
    """ext = NULL (no external segments) on the legacy default stream (NULL)."""
    torch = pytest.importorskip("torch")
    L = pkg.library()
    ctx = pkg.get_context()
    k = _consts(pkg)
    p, b = synth.square_loops(90, 13, 20.0, 200.0, 3000.0, 0.5, 0.1)
    n = 720
    soa = torch.from_numpy(synth.packed_soa(p, b)).cuda()
    ref = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    ctx.segseg_force_device(k, soa.data_ptr(), n, n, ref.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    out = torch.full((6 * n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = L.ddd_segseg_force_device_noalloc(ctypes.byref(k), soa.data_ptr(), n, None, n, out.data_ptr(), None)
    assert rc == pkg.DDD_OK
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref.cpu().numpy())


def test_noalloc_rejects_sizes_beyond_limit_and_bad_constants(pkg):
    torch = pytest.importorskip("torch")
    L = pkg.library()
    k = _consts(pkg)
    n = pkg.NOALLOC_MAX_SEGMENTS + 1
    segs = torch.zeros((9, n), dtype=torch.float64, device="cuda")
    out = torch.zeros(6 * n, dtype=torch.float64, device="cuda")
    rc = L.ddd_segseg_force_device_noalloc(ctypes.byref(k), segs.data_ptr(), n, None, n, out.data_ptr(), None)
    assert rc == pkg.DDD_ETOOBIG
    for field in ("aSq", "mu4pi", "nuMu4pinu"):
        bad = _consts(pkg)
        setattr(bad, field, float("nan"))
        rc = L.ddd_segseg_force_device_noalloc(ctypes.byref(bad), segs.data_ptr(), 8, None, 8, out.data_ptr(), None)
        assert rc == pkg.DDD_ENONFINITE
    bad = _consts(pkg)
    bad.aSq = 0.0
    assert L.ddd_segseg_force_device_noalloc(ctypes.byref(bad), segs.data_ptr(), 8, None, 8, out.data_ptr(),
                                             None) == pkg.DDD_EINVAL
