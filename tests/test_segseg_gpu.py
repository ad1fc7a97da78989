"""Seg-seg force on the GPU (through the C ABI) against the oracle and the goldens.

Tolerances (FP64 path):
  * golden networks: |Δ| <= 5e-14 elementwise and ||Δ|| <= 1e-11 ||golden||
    (the oracle meets 2e-14 / 1e-11; the kernel adds FMA contraction);
  * against the oracle: ||Δ|| <= 1e-10 ||F|| over the whole array, and per node
    force vector |ΔF_n| <= 1e-10 |F_n| + 1e-12 max_n |F_n| — node forces are
    sums of O(N) contributions that cancel (closed loops), so the absolute
    floor is set by the largest force in the network, not by the node itself.
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


def assert_forces_close(F, ref, rel=1e-10, floor=1e-12, fmax=None):
    """fmax: the largest node force of the whole network (default: of ref)."""
    assert F.shape == ref.shape
    d = F - ref
    scale = np.linalg.norm(ref)
    assert np.linalg.norm(d) <= rel * scale + 1e-300, np.linalg.norm(d) / scale
    dn = np.linalg.norm(d, axis=0)
    fn = np.linalg.norm(ref, axis=0)
    bound = rel * fn + floor * (fn.max() if fmax is None else fmax)
    worst = np.max(dn - bound)
    assert worst <= 0, "node-force error exceeds bound by %g (max rel %g)" % (worst, np.max(dn / (fn + 1e-300)))


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
    assert_forces_close(F, oracle.segseg_ser(k5_of(dln, mat), net))
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
    assert_forces_close(F, oracle.segseg_ser(k5_of(dln, mat), net))


@pytest.mark.parametrize("n", [1, 2, 3, 127, 129, 255, 257])
def test_ragged_sizes(pkg, synth, oracle, n):
    """numSeg not a multiple of the tile, including 1 and 2 segments."""
    net = _synthetic(pkg, synth, 40, 11, cube=2000.0)
    net.numSeg = n
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    ref = oracle.segseg_ser(k5_of(dln, mat), net)
    if n == 1:
        assert np.all(F == 0)
    else:
        assert_forces_close(F, ref)


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
    assert_forces_close(F, oracle.segseg_ser(k5_of(dln, mat), net))


def test_external_segments(pkg, synth, oracle):
    net = _synthetic(pkg, synth, 50, 31, cube=2000.0)
    rng = np.random.default_rng(5)
    net.extSeg[rng.choice(net.numSeg, 37, replace=False)] = 1
    dln, mat = _params(pkg)
    F = pkg.calcSegSegForce(dln, mat, net)
    assert np.all(F[:, :, net.extSeg[:net.numSeg] == 1] == 0)
    assert_forces_close(F, oracle.segseg_ser(k5_of(dln, mat), net))


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
    ref = oracle.segseg_idx(k5, net, idx)
    assert np.all(Fi[:, :, 2] == 0)
    assert_forces_close(Fi, ref)
    Fall = pkg.calcSegSegForce(dln, mat, net)
    assert np.linalg.norm(Fi - Fall[:, :, idx - 1]) <= 1e-10 * np.linalg.norm(Fall[:, :, idx - 1])
    one = pkg.calcSegSegForce(dln, mat, net, 17)
    assert one.shape == (3, 2, 1)
    assert_forces_close(one, oracle.segseg_idx(k5, net, [17]))


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
    ref = oracle.segseg_rows(k5_of(dln, mat), net, rows, nthreads=os.cpu_count() or 1)
    assert_forces_close(F[:, :, rows], ref, fmax=np.linalg.norm(F, axis=0).max())


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
