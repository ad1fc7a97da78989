"""The far-field quadrature's arithmetic on a CPU.

tests/quad_host/quad_host.cpp compiles ddd.jl_gb300/csrc/farfield_quad.cuh
(the FP32 Gauss-Legendre form of the far-pair force that ddd_surrogate_force
runs with far_mode 2 or 3) as plain C++, with inputs rounded to FP32 as the GPU
pass rounds them.  Against the long-double evaluation of the reference's
analytic pair force (the oracle on two-segment networks), relative to each
pair's largest node force, at midpoint separations R = 20-1000 max(L):
* 3 points: median ~2e-7, max < 1e-6 (the FP32 arithmetic; the quadrature
  itself is ~1e-9 at R/L = 20);
* 2 points: ~5e-6 at R/L = 20 (quadrature error), ~2e-7 from R/L = 100.
The analytic FP64 formula of the reference is off by up to ~3e-2 at
R/L = 1000 on the same pairs (its four-corner cancellation), which the test
records as the comparison.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "quad_host", "quad_host.cpp")
K5 = np.array([1.0, 1 / (4 * np.pi), 1 / (8 * np.pi), 1 / (4 * np.pi) / 0.72, 0.28 / (4 * np.pi) / 0.72])


@pytest.fixture(scope="module")
def quadhost(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("quadhost") / "libquadhost.so")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
           os.path.join(ROOT, "ddd.jl_gb300", "csrc"), SRC, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)
    lib.quad_pair_forces.argtypes = [dp, dp, ip, ctypes.c_int64, ctypes.c_int, dp]
    lib.quad_pair_forces.restype = None
    return lib


def _pairs(rng, RL, n):
    def unit():
        v = rng.normal(size=3)
        return v / np.linalg.norm(v)
    out = []
    for _ in range(n):
        L1, L2 = rng.uniform(20, 200, 2)
        c1 = rng.uniform(0, 20000, 3)
        c2 = c1 + unit() * RL * max(L1, L2)
        t1, t2, b1, b2 = unit(), unit(), unit(), unit()
        out.append((c1 - t1 * L1 / 2, c1 + t1 * L1 / 2, b1, c2 - t2 * L2 / 2, c2 + t2 * L2 / 2, b2))
    return out


@pytest.mark.parametrize("RL,nq,med,mx", [(20, 3, 5e-7, 2e-6), (30, 3, 5e-7, 2e-6), (100, 3, 5e-7, 2e-6),
                                          (1000, 3, 5e-7, 2e-6), (20, 2, 1e-5, 5e-5), (100, 2, 5e-7, 5e-6)])
def test_quadrature_against_long_double(pkg, oracle, quadhost, RL, nq, med, mx):
    rng = np.random.default_rng(RL + nq)
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)
    errs = []
    for n11, n12, b1, n21, n22, b2 in _pairs(rng, RL, 30):
        segs = np.ascontiguousarray(np.r_[n11, n12, b1, n21, n22, b2])
        out = np.zeros(12)
        pr = np.array([0, 1], dtype=np.int64)
        quadhost.quad_pair_forces(K5.ctypes.data_as(dp), segs.ctypes.data_as(dp), pr.ctypes.data_as(ip), 1, nq,
                                  out.ctypes.data_as(dp))
        net = pkg.DislocationNetwork(np.asfortranarray(np.stack([n11, n12, n21, n22], 1)),
                                     np.asfortranarray(np.stack([b1, b2], 1)),
                                     np.asfortranarray(np.array([[1, 1, 2], [2, 3, 4]], dtype=np.int64)))
        ext = oracle.segseg_ser_ld(K5, net)
        q = out.reshape(2, 2, 3).transpose(2, 1, 0)  # (xyz, node, segment)
        errs.append(np.abs(q - ext).max() / np.abs(ext).max())
    assert np.median(errs) <= med and np.max(errs) <= mx, (np.median(errs), np.max(errs))


@pytest.mark.parametrize("kappa,kappa_two", [(20.0, 0.0), (10.0, 0.0), (10.0, 30.0)])
@pytest.mark.parametrize("loops,seed,cube,pf", [(600, 41, 20000.0, 0.05), (300, 7, 3000.0, 0.2)])
def test_network_rows_against_long_double(pkg, synth, oracle, quadhost, loops, seed, cube, pf, kappa, kappa_two):
    """A whole network as the far-field mode computes it (quad_network_rows:
    the kernel's own decisions and near-parallel construction, near pairs from
    the oracle), 48 sampled segments against the long-double evaluation of the
    reference's formulas.  Near-parallel far pairs take the reference's
    projected geometry (calcParSegSegForce), which the quadrature then
    integrates: without it these pairs alone put ~1e-6 into the node forces.
    Measured with 3 points: normwise ~3e-10, worst node ~4e-9 relative (far
    pairs' forces are small beside the near pairs', so their FP32 error of
    ~2e-7 each stays small in the node sums), at the trust factor 20 and at
    10 (the quadrature's default).  kappa_two > 0: every pair beyond
    kappa_two max(L_i, L_j) takes the 2-point rule, more pairs than the GPU
    pass's switch (a 32-pair step only when all its far pairs are that far);
    at 30 the errors stay where they are (measured ~7.5e-10 normwise with 96 %
    of the pairs on 2 points on 32,768 segments of the workload).  Bounds:
    normwise 1e-8, per node 1e-6 |F| + 1e-8 max |F|."""
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)
    quadhost.quad_network_rows.argtypes = [dp, dp, ctypes.c_int64, ctypes.c_double, ctypes.c_int, ip, ctypes.c_int64,
                                           ctypes.c_void_p, dp]
    quadhost.quad_network_rows.restype = None
    p, b = synth.square_loops(loops, seed, 20.0, 200.0, cube, 0.5, pf)
    net = pkg.DislocationNetwork(*synth.network_arrays(p, b))
    n = net.numSeg
    segs = np.ascontiguousarray(synth.packed_soa(p, b).T)
    rows = np.sort(np.random.default_rng(seed).choice(n, 48, replace=False)).astype(np.int64)
    two = None
    if kappa_two > 0:
        m = 0.5 * (segs[:, 0:3] + segs[:, 3:6])
        L = np.linalg.norm(segs[:, 3:6] - segs[:, 0:3], axis=1)
        R = np.linalg.norm(m[rows][:, None] - m[None], axis=2)
        two = np.ascontiguousarray(R >= kappa_two * np.maximum(L[rows][:, None], L[None]), dtype=np.uint8)
        assert two.mean() > 0.05
    out = np.zeros((len(rows), 6))
    quadhost.quad_network_rows(K5.ctypes.data_as(dp), segs.ctypes.data_as(dp), n, kappa, 3, rows.ctypes.data_as(ip),
                               len(rows), None if two is None else two.ctypes.data_as(ctypes.c_void_p),
                               out.ctypes.data_as(dp))
    ext = oracle.segseg_ser_ld(K5, net, rows, nthreads=os.cpu_count() or 1)
    G = out.reshape(-1, 2, 3).transpose(2, 1, 0)
    nrm = lambda a: np.linalg.norm(a, axis=0)
    rel = np.linalg.norm(G - ext) / np.linalg.norm(ext)
    if os.environ.get("DDD_TEST_STATS"):
        with open(os.environ["DDD_TEST_STATS"], "a") as fh:
            fh.write("quad network rows %d loops cube %g kappa %g kappa_two %g: rel %.3e max node rel %.3e\n" % (
                loops, cube, kappa, kappa_two, rel, np.max(nrm(G - ext) / nrm(ext))))
    assert rel <= 1e-8, rel
    assert np.all(nrm(G - ext) <= 1e-6 * nrm(ext) + 1e-8 * nrm(ext).max())


@pytest.mark.parametrize("side", [1, 2])
def test_near_parallel_connector_test_matches_fp64(quadhost, side):
    """The near-parallel construction decides the reference's connector test
    (magDiffSq > sqrt(eps) (|nbm1|^2 + |nbm2|^2), DislocationForces.jl:1204-1317
    and :1319-1433) in FP32 from approximate node positions, and in FP64 within
    1e-5 of the threshold.  Over 20,000 near-parallel configurations (tilts
    1e-7 to 1.2e-4 rad, segment lengths 20-200, positions 1 to 3e4 from the
    origin, a third of them placed within 1e-3 relative of the threshold, half
    of those within 5e-6), the decision equals the FP64 formula's evaluated in
    the reference's order."""
    dp = ctypes.POINTER(ctypes.c_double)
    quadhost.quad_par_sources.argtypes = [ctypes.c_int, dp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]
    quadhost.quad_par_sources.restype = None
    rng = np.random.default_rng(11 + side)
    eps, hcot = 1.4901161193847656e-08, 4075.672300430329
    n = 20000

    def unit(v):
        return v / np.linalg.norm(v, axis=-1, keepdims=True)

    L = rng.uniform(20, 200, n)
    u = unit(rng.normal(size=(n, 3)))
    w = unit(np.cross(u, rng.normal(size=(n, 3))))
    th = np.exp(rng.uniform(np.log(1e-7), np.log(1.2e-4), n))
    ta = unit(np.cos(th)[:, None] * u + np.sin(th)[:, None] * w)
    lb = L[:, None] * u
    pos = unit(rng.normal(size=(n, 3))) * np.exp(rng.uniform(0, np.log(3e4), n))[:, None]

    def ref_conn(ta, lb, na):
        tmp = lb[:, 0] * ta[:, 0] + lb[:, 1] * ta[:, 1] + lb[:, 2] * ta[:, 2]
        proj = tmp[:, None] * ta
        diff = lb - proj
        dd = diff[:, 0] * diff[:, 0] + diff[:, 1] * diff[:, 1] + diff[:, 2] * diff[:, 2]
        mag = np.sqrt(dd)
        tv1 = 0.5 * diff
        tv2 = (hcot * mag)[:, None] * ta
        e1 = na + tv1 + tv2
        e2 = na + proj + tv1 - tv2
        s1 = e1[:, 0] * e1[:, 0] + e1[:, 1] * e1[:, 1] + e1[:, 2] * e1[:, 2]
        s2 = e2[:, 0] * e2[:, 0] + e2[:, 1] * e2[:, 1] + e2[:, 2] * e2[:, 2]
        msq = dd if side == 1 else mag * mag
        return msq > eps * (s1 + s2), msq, s1 + s2

    # A third placed within 1e-3, relative, of the threshold: tilts of 9e-5 to
    # 1.2e-4 rad (below ~8.6e-5 no position reaches it) and the node at
    # -lb/2 + r v, r solving |r v + a|^2 + |r v + b|^2 = magDiffSq / (eps target)
    # for the offsets a, b of nbm1 and nbm2 from that point.
    k = np.arange(n) % 3 == 0
    th[k] = rng.uniform(9e-5, 1.2e-4, k.sum())
    ta = unit(np.cos(th)[:, None] * u + np.sin(th)[:, None] * w)
    target = 1 + np.where(np.arange(n) % 2 == 0, rng.uniform(-1e-3, 1e-3, n), rng.uniform(-5e-6, 5e-6, n))
    tmp = np.sum(lb * ta, axis=1)
    diff = lb - tmp[:, None] * ta
    dd = np.sum(diff * diff, axis=1)
    h = (hcot * np.sqrt(dd))[:, None] * ta
    a = -0.5 * lb + 0.5 * diff + h
    b = -0.5 * lb + tmp[:, None] * ta + 0.5 * diff - h
    v = unit(rng.normal(size=(n, 3)))
    T = dd / (eps * target)
    pb = np.sum(v * (a + b), axis=1)
    disc = pb ** 2 - 2 * (np.sum(a * a, axis=1) + np.sum(b * b, axis=1) - T)
    ok = k & (disc > 0)
    r = (-pb + np.sqrt(np.where(disc > 0, disc, 0))) / 2
    pos[ok] = -0.5 * lb[ok] + r[ok, None] * v[ok]
    _, msq, ssum = ref_conn(ta, lb, pos)
    close = ok & (np.abs(msq / (eps * ssum) - 1) < 2e-3)
    want, _, _ = ref_conn(ta, lb, pos)
    cfg = np.ascontiguousarray(np.concatenate([ta, lb, pos], axis=1))
    got = np.zeros(n, dtype=np.int32)
    quadhost.quad_par_sources(side, cfg.ctypes.data_as(dp), n, got.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    band = close & (np.abs(msq / (eps * ssum) - 1) < 1e-5)  # decided by the FP64 evaluation
    assert close.sum() > n // 5 and band.sum() > n // 20 and 0.3 < want[close].mean() < 0.7
    assert np.array_equal(got >= 2, want)
