"""The fast FP64 form's arithmetic on a CPU.

tests/f64fast_host/pair_fast_host.cpp compiles ddd.jl_gb300/csrc/pair_f64fast.cuh
(the general branch DDD_MODE_FP64_FAST runs on the GPU: one division per
corner, table-driven logarithm and arctangent, explicit fused multiply-adds)
as plain C++ without contraction, so its general-branch values are the GPU's
bit for bit; near-parallel pairs take the oracle's strict branch, as on the
GPU.  All pairs are summed in calcSegSegForceSer!'s order.

On seeded networks the form's largest node-force error against the long-double
evaluation must stay within 1.5x the reference arithmetic's own (measured
1.00-1.08x), and the parity bound of the GPU tests must hold against the
oracle.  The table-driven log and atan are checked against long double at
<= 2 ulp over wide argument ranges.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, k5_of

SRC = os.path.join(ROOT, "tests", "f64fast_host", "pair_fast_host.cpp")


@pytest.fixture(scope="module")
def fasthost(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("fasthost") / "libfasthost.so")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-Wno-unknown-pragmas",
           "-I", os.path.join(ROOT, "ddd.jl_gb300", "csrc"), SRC, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    dp, ip, up = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint8)
    lib.fast_segseg_ser.argtypes = [ctypes.c_int, dp, dp, dp, ip, ctypes.c_int64, up, ctypes.c_int64, dp]
    lib.fast_segseg_ser.restype = None
    lib.fast_log_atan.argtypes = [ctypes.c_int, dp, ctypes.c_int64, dp, dp]
    lib.fast_sigma.argtypes = [dp, dp, ctypes.c_int64, dp, dp, ip, ctypes.c_int64, ctypes.c_int64, dp]
    lib.fast_sigma.restype = None
    lib.fast_log_atan.restype = None

    def forces(k5, net, fmath=1):
        F = np.zeros((3, 2, net.numSeg), order="F")
        lib.fast_segseg_ser(fmath, np.ascontiguousarray(k5).ctypes.data_as(dp), net.coord.ctypes.data_as(dp),
                            net.bVec.ctypes.data_as(dp), net.segIdx.ctypes.data_as(ip), net.segIdx.shape[0],
                            net.extSeg.ctypes.data_as(up), net.numSeg, F.ctypes.data_as(dp))
        return F

    def log_atan(x, kind=1):
        x = np.ascontiguousarray(x, np.float64)
        lo, at = np.zeros_like(x), np.zeros_like(x)
        lib.fast_log_atan(kind, x.ctypes.data_as(dp), len(x), lo.ctypes.data_as(dp), at.ctypes.data_as(dp))
        return lo, at

    def sigma(k5, pts, net):
        pts = np.asfortranarray(pts, np.float64)
        S = np.zeros((6, pts.shape[1]), order="F")
        lib.fast_sigma(np.ascontiguousarray(k5).ctypes.data_as(dp), pts.ctypes.data_as(dp), pts.shape[1],
                       net.coord.ctypes.data_as(dp), net.bVec.ctypes.data_as(dp), net.segIdx.ctypes.data_as(ip),
                       net.segIdx.shape[0], net.numSeg, S.ctypes.data_as(dp))
        return S

    forces.log_atan = log_atan
    forces.sigma = sigma
    return forces


@pytest.mark.parametrize("fmath", [2, 1])
@pytest.mark.parametrize("num_loops,seed,cube,pf", [(16, 1, 3000.0, 0.05), (64, 4, 3000.0, 0.05),
                                                    (96, 21, 1500.0, 0.5), (300, 7, 20000.0, 0.05)])
def test_fast_form_within_reference_noise(pkg, synth, oracle, fasthost, num_loops, seed, cube, pf, fmath):
    p, b = synth.square_loops(num_loops, seed, 20.0, 200.0, cube, 0.5, pf)
    net = pkg.DislocationNetwork(*synth.network_arrays(p, b))
    dln, mat = pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28)
    k5 = k5_of(dln, mat)
    ref = oracle.segseg_ser(k5, net)
    ext = oracle.segseg_ser_ld(k5, net, nthreads=os.cpu_count() or 1)
    nrm = lambda a: np.linalg.norm(a, axis=0)
    ulps = 4 * np.finfo(np.float64).eps * nrm(ext).max()
    noise = nrm(ref - ext).max()
    F = fasthost(k5, net, fmath)
    if os.environ.get("DDD_TEST_STATS"):
        with open(os.environ["DDD_TEST_STATS"], "a") as fh:
            fh.write("fast host fmath=%d loops=%d: normwise %.3e, err/noise %.3f\n"
                     % (fmath, num_loops, np.linalg.norm(F - ref) / np.linalg.norm(ref), nrm(F - ext).max() / noise))
    assert np.linalg.norm(F - ref) <= 1e-10 * np.linalg.norm(ref) + ulps
    assert nrm(F - ext).max() <= 1.5 * noise + ulps
    assert np.max(nrm(F - ref) - (1e-10 * nrm(ref) + 4 * noise + ulps)) <= 0
    assert not np.array_equal(F, ref)


def test_table_log_atan_ulps(fasthost):
    rng = np.random.default_rng(3)
    x = np.concatenate([np.exp2(rng.uniform(-60, 60, 200000)), 1 + rng.uniform(-1e-3, 1e-3, 50000),
                        rng.uniform(0.5, 2.0, 50000)])
    lo, at = fasthost.log_atan(x)
    ln, an = np.log(x.astype(np.longdouble)), np.arctan(x.astype(np.longdouble))
    ulp = lambda v: np.spacing(np.abs(v.astype(np.float64)))
    assert np.max(np.abs(lo - ln) / ulp(ln)) <= 2.0
    assert np.max(np.abs(at - an) / ulp(an)) <= 2.0
    lo_n, at_n = fasthost.log_atan(-x)
    assert np.all(np.isnan(lo_n)) and np.array_equal(at_n, -at)
    lo_s, at_s = fasthost.log_atan(np.array([0.0, np.inf, 1.0, 5e-320]))
    assert lo_s[0] == -np.inf and lo_s[1] == np.inf and lo_s[2] == 0.0 and np.isclose(lo_s[3], np.log(5e-320))
    assert at_s[1] == np.pi / 2 and at_s[0] == 0.0


def test_integer_log_atan_ulps(fasthost):
    """The integer-pipe log and atan (intmath_f64.cuh): one rounding of a
    fixed-point result carried to 2^-60 relative or better, so within 0.51 ulp
    of the long-double value over the whole range, next to 1 (log), below
    1/128 and above 1 (atan), with the standard functions' answers for 0,
    infinities, NaN and subnormals."""
    rng = np.random.default_rng(4)
    x = np.concatenate([np.exp2(rng.uniform(-1020, 1020, 100000)), np.exp2(rng.uniform(-30, 30, 100000)),
                        1 + rng.choice([-1, 1], 50000) * np.exp2(rng.uniform(-52, -6, 50000)),
                        1 + np.arange(-2000, 2000) * 2.0 ** -52, rng.uniform(0.5, 2.0, 50000),
                        np.arange(1, 129) / 128.0, np.arange(1, 65) / 64.0 * (1 + 2.0 ** -52)])
    lo, at = fasthost.log_atan(x, 2)
    xl = x.astype(np.longdouble)
    ln, an = np.log(xl), np.arctan(xl)
    ulp = lambda v: np.spacing(np.abs(v.astype(np.float64)))
    nz = ln != 0
    assert np.all(lo[~nz] == 0.0)
    assert np.max(np.abs(lo[nz] - ln[nz]) / ulp(ln[nz])) <= 0.51
    assert np.max(np.abs(at - an) / ulp(an)) <= 0.51
    lo_n, at_n = fasthost.log_atan(-x, 2)
    assert np.all(np.isnan(lo_n)) and np.array_equal(at_n, -at)
    lo_s, at_s = fasthost.log_atan(np.array([0.0, np.inf, 1.0, 5e-320, -np.inf, np.nan, 1e-30]), 2)
    assert lo_s[0] == -np.inf and lo_s[1] == np.inf and lo_s[2] == 0.0 and np.isclose(lo_s[3], np.log(5e-320))
    assert at_s[1] == np.pi / 2 and at_s[0] == 0.0 and at_s[4] == -np.pi / 2 and np.isnan(at_s[5])
    assert at_s[6] == 1e-30


@pytest.mark.parametrize("num_loops,cube", [(64, 2000.0), (300, 20000.0), (96, 1500.0)])
def test_fast_sigma_within_bound(pkg, synth, oracle, fasthost, num_loops, cube):
    """The fast σ̃ form (sigma_fx.cuh, the header the GPU runs) against long
    double: normwise within 4x the reference arithmetic's own error (measured
    2-2.3x; both ~1e-15), and the strict form's per-point bound
    |Δσ| <= 1e-10 |σ| + 1e-12 max|σ| against the reference arithmetic."""
    p, b = synth.square_loops(num_loops, 3, 20.0, 200.0, cube, 0.5, 0.1)
    net = pkg.DislocationNetwork(*synth.network_arrays(p, b))
    k5 = k5_of(pkg.DislocationParameters(coreRad=1.0), pkg.MaterialParameters(mu=1.0, nu=0.28))
    pts = np.asfortranarray(np.random.default_rng(1).uniform(0, cube, (3, 1500)))
    ref = oracle.sigma_tilde(k5, pts, net, nthreads=os.cpu_count() or 1)
    ld = oracle.sigma_tilde_ld(k5, pts, net, nthreads=os.cpu_count() or 1)
    F = fasthost.sigma(k5, pts, net)
    assert np.linalg.norm(F - ld) <= 4 * np.linalg.norm(ref - ld) + 1e-16 * np.linalg.norm(ld)
    d, n = np.linalg.norm(F - ref, axis=0), np.linalg.norm(ref, axis=0)
    assert np.all(d <= 1e-10 * n + 1e-12 * n.max())
