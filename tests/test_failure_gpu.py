"""Failure detection on the GPU without a GPU fault.

Every wait inside this library's tensor-core kernels is an mbarrier wait
bounded by an SM-clock deadline; on expiry the kernel records a flag, leaves
its loops and returns, and the call reports DDD_ETIMEOUT.  The self-test entry
point runs that same bounded wait in a one-warp kernel that issues no MMA and
holds no tensor memory, on a barrier that nothing arrives on, so the wait runs
out after about half a millisecond.  The test checks the status, that the same
wait succeeds when the arrival happens, and that the context still computes
correct forces afterwards.
"""
import numpy as np
import pytest

from conftest import k5_of

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_stays_usable(pkg, synth, oracle):
    ctx = pkg.get_context()
    assert ctx.selftest_bounded_wait(1_000_000, arrive=True) == pkg.DDD_OK
    assert ctx.selftest_bounded_wait(1_000_000, arrive=False) == pkg.DDD_ETIMEOUT
    assert "timed out" in ctx.last_error
    # Out-of-range limits are refused before any launch.
    assert ctx.selftest_bounded_wait(0, arrive=False) == pkg.DDD_EINVAL
    assert ctx.selftest_bounded_wait(3_000_000_000, arrive=False) == pkg.DDD_EINVAL
    # The context is usable: a seg-seg force matching the oracle, and the wait again.
    p, b = synth.square_loops(12, 3, 20.0, 200.0, 2000.0, 0.5, 0.1)
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    dln, mat = pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28)
    F = pkg.calcSegSegForce(dln, mat, net)
    ref = oracle.segseg_ser(k5_of(dln, mat), net)
    assert np.abs(F - ref).max() <= 1e-10 * np.abs(ref).max()
    assert ctx.selftest_bounded_wait(1_000_000, arrive=False) == pkg.DDD_ETIMEOUT
    assert ctx.selftest_bounded_wait(1_000_000, arrive=True) == pkg.DDD_OK
