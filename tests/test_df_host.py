"""The precision forms' pair arithmetic on a CPU.

tests/df_host/df_pair_host.cpp compiles ddd.jl_gb300/csrc/pair_df.cuh (the
df64 and f32c general-branch formulas the GPU runs) as plain C++, with every
FP32 operation rounded on its own.  The only host/device difference is the
first-step quotient estimate of a double-float division, exact here and
approximate on the GPU; the algorithm allows any error below 2^-20 there.

Per pair, against long double (the oracle's long-double evaluation of the
same formulas), with errors relative to each pair's largest force, at centre
distances R ~ 50, 1,000 and 20,000 (lengths 20-200):
* the reference's own FP64 result has errors that grow with R/L as its terms
  cancel. Measured median / max: 6e-15 / 5e-11 near, 6e-12 / 7e-7 at R/L ~ 10,
  7e-8 / 6e-4 at R/L ~ 200;
* df64 (unit roundoff 2^-48, 32x FP64's) tracks it at 25-40x, and is bounded
  here by 128x FP64's error, median and max;
* f32c adds its FP32 assembly's ~2e-7. It is bounded by 1e-6 + 128x FP64's
  median, and 2e-5 + 128x FP64's max;
* plain FP32 (the oracle's FP32 restatement) is 13x worse than f32c near and
  1e4 to 1e7 times worse beyond. The compensated terms carry the accuracy.

The mixed σ̃ form (sigma_point_mixed, same header) against the FP64 oracle
per point: its error is flat in distance, ~1e-7.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "df_host", "df_pair_host.cpp")
K4 = np.array([1.0, 1 / (4 * np.pi), 1 / (8 * np.pi), 1 / (4 * np.pi) / (1 - 0.28)])
K5 = np.r_[K4, 0.28 / (4 * np.pi) / (1 - 0.28)]


@pytest.fixture(scope="module")
def dfhost(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("dfhost") / "libdfhost.so")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-Wno-unknown-pragmas",
           "-I", os.path.join(ROOT, "ddd.jl_gb300", "csrc"), SRC, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)
    lib.df_pair_forces.argtypes = [ctypes.c_int, dp, dp, ip, ctypes.c_int64, dp]
    lib.df_pair_forces.restype = None
    lib.df_sigma_points.argtypes = [dp, dp, ctypes.c_int64, dp, ctypes.c_int64, dp]
    lib.df_sigma_points.restype = None
    lib.df_pair_quad_forces.argtypes = [dp, dp, ip, ctypes.c_int64, ctypes.c_int, dp]
    lib.df_pair_quad_forces.restype = None

    def forces(form, n1, n2, b):
        """Forces (m × 4 × 3) of the pairs (segment 2q, segment 2q+1)."""
        t = n2 - n1
        tN = 1.0 / np.sqrt(t[:, 0] * t[:, 0] + t[:, 1] * t[:, 1] + t[:, 2] * t[:, 2])
        segs = np.ascontiguousarray(np.c_[n1, n2, b, t * tN[:, None], tN])
        m = len(n1) // 2
        p = np.arange(2 * m, dtype=np.int64)
        out_ = np.zeros(12 * m)
        lib.df_pair_forces(form, K4.ctypes.data_as(dp), segs.ctypes.data_as(dp), p.ctypes.data_as(ip), m,
                           out_.ctypes.data_as(dp))
        return out_.reshape(m, 4, 3)

    def sigma(n1, n2, b, x):
        """Mixed-form σ̃ (6 × M) of one segment at the points x (M × 3)."""
        t = n2 - n1
        tN = 1.0 / np.sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2])
        segs = np.ascontiguousarray(np.r_[n1, n2, b, t * tN, tN][None, :])
        xs = np.ascontiguousarray(x)
        out_ = np.zeros(6 * len(x))
        lib.df_sigma_points(K5.ctypes.data_as(dp), segs.ctypes.data_as(dp), 1, xs.ctypes.data_as(dp), len(x),
                            out_.ctypes.data_as(dp))
        return out_.reshape(-1, 6).T

    def quad(nq, n1, n2, b):
        """The planned far-field form on the mixed arithmetic (m × 4 × 3)."""
        t = n2 - n1
        tN = 1.0 / np.sqrt(t[:, 0] * t[:, 0] + t[:, 1] * t[:, 1] + t[:, 2] * t[:, 2])
        segs = np.ascontiguousarray(np.c_[n1, n2, b, t * tN[:, None], tN])
        m = len(n1) // 2
        p = np.arange(2 * m, dtype=np.int64)
        out_ = np.zeros(12 * m)
        lib.df_pair_quad_forces(K5.ctypes.data_as(dp), segs.ctypes.data_as(dp), p.ctypes.data_as(ip), m, nq,
                                out_.ctypes.data_as(dp))
        return out_.reshape(m, 4, 3)

    forces.sigma = sigma
    forces.quad = quad
    return forces


def _pairs(m, dist, seed):
    """m pairs of segments (lengths 20-200, random directions and unit b), the
    second segment's start ~dist from the first's."""
    rng = np.random.default_rng(seed)
    n1 = rng.normal(size=(2 * m, 3)) * 100
    d = rng.normal(size=(2 * m, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    n1[1::2] = n1[0::2] + rng.normal(size=(m, 3)) / np.sqrt(3) * dist
    n2 = n1 + d * rng.uniform(20, 200, 2 * m)[:, None]
    b = rng.normal(size=(2 * m, 3))
    b /= np.linalg.norm(b, axis=1)[:, None]
    t = (n2 - n1) / np.linalg.norm(n2 - n1, axis=1)[:, None]
    c = np.sum(t[0::2] * t[1::2], axis=1)
    assert np.all(1 - c * c > 1e-6)  # all general-branch pairs
    return n1, n2, b


def _oracle(oracle, n1, n2, b, f32=False):
    m = len(n1) // 2
    return np.array([oracle.pair(K5, b[2 * q], n1[2 * q], n2[2 * q], b[2 * q + 1], n1[2 * q + 1], n2[2 * q + 1],
                                 f32=f32) for q in range(m)])


def _rel(F, ref):
    """Per pair: the largest force-component error over the pair's largest force."""
    m = len(ref)
    return np.abs(F - ref).reshape(m, -1).max(axis=1) / np.abs(ref).reshape(m, -1).max(axis=1)


def _long_double(pkg, oracle, n1, n2, b):
    m = len(n1) // 2
    ld = np.zeros((m, 4, 3))
    for q in range(m):
        coord = np.asfortranarray(np.c_[n1[2 * q], n2[2 * q], n1[2 * q + 1], n2[2 * q + 1]])
        net = pkg.DislocationNetwork(coord, np.asfortranarray(np.c_[b[2 * q], b[2 * q + 1]]),
                                     np.array([[1, 1, 2], [2, 3, 4]], np.int64))
        F = oracle.segseg_ser_ld(K5, net)  # 3 × 2 × 2, long double
        ld[q] = np.array([F[:, 0, 0], F[:, 1, 0], F[:, 0, 1], F[:, 1, 1]])
    return ld


@pytest.mark.parametrize("dist,seed,f32_factor", [(50.0, 1, 5.0), (1000.0, 2, 1e3), (20000.0, 3, 1e3)])
def test_precision_forms_vs_long_double(pkg, dfhost, oracle, dist, seed, f32_factor):
    n1, n2, b = _pairs(300, dist, seed)
    ld = _long_double(pkg, oracle, n1, n2, b)
    e64 = _rel(_oracle(oracle, n1, n2, b), ld)
    e_df = _rel(dfhost(0, n1, n2, b), ld)
    e_c = _rel(dfhost(1, n1, n2, b), ld)
    e_32 = _rel(_oracle(oracle, n1, n2, b, f32=True), ld)
    med = np.median
    assert med(e_df) <= 128 * med(e64) and e_df.max() <= 128 * e64.max(), (med(e_df), e_df.max(), med(e64),
                                                                              e64.max())
    assert med(e_c) <= 1e-6 + 128 * med(e64), (med(e_c), med(e64))
    assert e_c.max() <= 2e-5 + 128 * e64.max(), (e_c.max(), e64.max())
    assert med(e_32) >= f32_factor * med(e_c), (med(e_32), med(e_c))


@pytest.mark.parametrize("dist", [50.0, 1000.0, 20000.0])
def test_mixed_sigma_per_point(pkg, dfhost, oracle, dist):
    """The mixed σ̃ form (endpoint terms and their differences in df64,
    assembly in FP32) against the FP64 oracle, per point relative to the
    point's largest component: flat in distance (measured median 1.2e-7, max
    5.9e-7 at R/L from 0.5 to 200), where the endpoint terms cancel as
    (L/R)^2."""
    rng = np.random.default_rng(int(dist))
    errs = []
    for _ in range(30):
        n1 = rng.normal(size=3) * 100
        d = rng.normal(size=3)
        n2 = n1 + d / np.linalg.norm(d) * rng.uniform(20, 200)
        b = rng.normal(size=3)
        b /= np.linalg.norm(b)
        x = n1 + rng.normal(size=(20, 3)) / np.sqrt(3) * dist
        net = pkg.DislocationNetwork(np.asfortranarray(np.c_[n1, n2]), np.asfortranarray(b[:, None]),
                                     np.array([[1, 1, 2]], np.int64))
        ref = oracle.sigma_tilde(K5, np.asfortranarray(x.T), net)
        S = dfhost.sigma(n1, n2, b, x)
        errs.append(np.abs(S - ref).max(axis=0) / np.abs(ref).max(axis=0))
    e = np.concatenate(errs)
    assert np.median(e) <= 5e-7 and e.max() <= 5e-6, (np.median(e), e.max())


def _pairs_rl(m, rl, seed):
    """m pairs at centre distance R = rl (L1 + L2) / 2, lengths 20-200."""
    rng = np.random.default_rng(seed)
    n1, n2, b = np.zeros((2 * m, 3)), np.zeros((2 * m, 3)), np.zeros((2 * m, 3))
    for q in range(m):
        L1, L2 = rng.uniform(20, 200, 2)
        d1, d2, off, b1, b2 = (v / np.linalg.norm(v) for v in rng.normal(size=(5, 3)))
        a = rng.normal(size=3) * 10
        n1[2 * q], n2[2 * q] = a, a + d1 * L1
        n1[2 * q + 1] = a + off * rl * 0.5 * (L1 + L2)
        n2[2 * q + 1] = n1[2 * q + 1] + d2 * L2
        b[2 * q], b[2 * q + 1] = b1, b2
    return n1, n2, b


@pytest.mark.parametrize("rl", [30, 300])
def test_far_field_quadrature_on_mixed_arithmetic(pkg, dfhost, oracle, rl):
    """The planned far-field form (Gauss quadrature of the partner's mixed σ̃,
    FP32 assembly) against long double.  The 3-point rule is within 5e-6 of
    each pair's largest force from R/L = 30 (measured median 1.5e-7, max
    5.2e-7).  At R/L = 300 both rules are, where the reference formula's own
    FP64 result is off by more (measured max 1.4e-3; the rules 8e-7)."""
    n1, n2, b = _pairs_rl(150, rl, seed=rl)
    ld = _long_double(pkg, oracle, n1, n2, b)
    e3 = _rel(dfhost.quad(3, n1, n2, b), ld)
    assert np.median(e3) <= 5e-7 and e3.max() <= 5e-6, (np.median(e3), e3.max())
    if rl >= 300:
        e2 = _rel(dfhost.quad(2, n1, n2, b), ld)
        e64 = _rel(_oracle(oracle, n1, n2, b), ld)
        assert e2.max() <= 5e-6 and e64.max() > max(e2.max(), e3.max()), (e2.max(), e3.max(), e64.max())
