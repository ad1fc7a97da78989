"""Self force and total segment force on the GPU (through the C ABI).

calcSelfForce's formula is per segment with no sums, so the GPU (strict FP64)
and the oracle differ only where CUDA's and the C library's log differ by an
ulp: bound 1e-14 relative to the largest component.  Goldens: the reference's
test/SegmentForcesTest.jl:244-267 at the oracle test's bounds (2e-14
elementwise, 1e-11 in norm).  calcSegForce adds the seg-seg force, checked
against the GPU seg-seg path plus the oracle's self and PK forces.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

G_SELF = json.load(open(os.path.join(GOLDEN, "selfforce_goldens.json")))


def _golden_case(pkg, fixtures):
    c = G_SELF["cases"][0]
    p = G_SELF["params"]
    fnet = fixtures.make_network(c["loops"], G_SELF["slipSystems"], c["range"], c["shift"])
    net = pkg.DislocationNetwork(fnet.coord, fnet.bVec, fnet.segIdx)
    dln = pkg.DislocationParameters(coreRad=p["coreRad"], coreEnergy=p["coreEnergy"], minSegLen=100.0,
                                    maxSegLen=1000.0)
    mat = pkg.MaterialParameters(mu=p["mu"], nu=p["nu"])
    return c, net, dln, mat


def _random(pkg, synth, loops=60, seed=4):
    p, b = synth.square_loops(loops, seed, 50.0, 200.0, 3000.0, 0.5, 0.05)
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    dln = pkg.DislocationParameters(coreRad=1.0)
    mat = pkg.MaterialParameters(mu=1.0, nu=0.28)
    return net, dln, mat


def _sc(dln, mat):
    return np.array([dln.coreRad, dln.coreEnergy, mat.ν])


def _k5(dln, mat):
    return np.array([dln.coreRadSq, mat.μ4π, mat.μ8π, mat.μ4πν, mat.νμ4πν])


def test_golden(pkg, fixtures):
    c, net, dln, mat = _golden_case(pkg, fixtures)
    F1, F2 = pkg.calcSelfForce(dln, mat, net)
    for ours, gold in ((F1.T, np.array(c["f1"])), (F2.T, np.array(c["f2"]))):
        assert np.abs(ours - gold).max() <= 2e-14
        assert np.linalg.norm(ours - gold) <= 1e-11 * np.linalg.norm(gold)
    assert np.array_equal(F1, -F2)


def test_vs_oracle_idx_and_ext(pkg, synth, oracle):
    net, dln, mat = _random(pkg, synth)
    ref1, ref2 = oracle.self_force(_k5(dln, mat), _sc(dln, mat), net)
    F1, F2 = pkg.calcSelfForce(dln, mat, net)
    tol = 1e-14 * np.abs(ref2).max()
    assert np.abs(F2 - ref2).max() <= tol and np.abs(F1 - ref1).max() <= tol
    idx = np.array([5, 17, 5, 300, 1])
    G1, G2 = pkg.calcSelfForce(dln, mat, net, idx)
    assert np.array_equal(G2, F2[:, idx - 1])
    net.extSeg[[1, 16]] = 1  # positions 2 and 17: the idx form skips its entry 2 (segment 17)
    H1, H2 = pkg.calcSelfForce(dln, mat, net, idx)
    o1, o2 = oracle.self_force(_k5(dln, mat), _sc(dln, mat), net, idx)
    assert np.all(H2[:, 1] == 0) and np.abs(H2 - o2).max() <= tol
    assert np.array_equal(H2[:, [0, 2, 3, 4]], G2[:, [0, 2, 3, 4]])


def test_inplace(pkg, synth):
    net, dln, mat = _random(pkg, synth, loops=20, seed=6)
    F1, F2 = pkg.calcSelfForce(dln, mat, net)
    start = np.asfortranarray(np.arange(net.segForce.size, dtype=np.float64).reshape(net.segForce.shape, order="F"))
    net.segForce[...] = start
    idx = [3, 9, 3]
    pkg.calcSelfForce_inplace(dln, mat, net, idx)
    want = start.copy()
    for i in idx:
        want[:, 0, i - 1] -= F2[:, i - 1]
        want[:, 1, i - 1] += F2[:, i - 1]
    assert np.array_equal(net.segForce, want)


def test_seg_force_composition(pkg, synth, oracle):
    net, dln, mat = _random(pkg, synth, loops=40, seed=8)
    n = net.numSeg
    rng = np.random.default_rng(1)
    sh = np.asfortranarray(rng.normal(size=(6, n)) * 1e-3)
    F = pkg.calcSegForce(dln, mat, sh, net)
    SS = pkg.calcSegSegForce(dln, mat, net)
    ref1, ref2 = oracle.self_force(_k5(dln, mat), _sc(dln, mat), net)
    PK = oracle.pk_force(net, sh)
    want = SS.copy()
    want[:, 0, :] += ref1 + 0.5 * PK
    want[:, 1, :] += ref2 + 0.5 * PK
    assert np.abs(F - want).max() <= 1e-13 * np.abs(want).max()
    # No stress: the PK term drops out.
    F0 = pkg.calcSegForce(dln, mat, None, net)
    assert np.abs(F0[:, 1, :] - (SS[:, 1, :] + ref2)).max() <= 1e-13 * np.abs(want).max()
    # The idx form: the selected columns.
    idx = [7, 2, 7]
    Fi = pkg.calcSegForce(dln, mat, np.asfortranarray(sh[:, [6, 1, 6]]), net, idx)
    assert np.abs(Fi - F[:, :, [6, 1, 6]]).max() <= 1e-12 * np.abs(F).max()


def test_seg_force_inplace(pkg, synth, oracle):
    net, dln, mat = _random(pkg, synth, loops=30, seed=9)
    n = net.numSeg
    rng = np.random.default_rng(2)
    sh = np.asfortranarray(rng.normal(size=(6, n)) * 1e-3)
    net.segForce[...] = rng.normal(size=net.segForce.shape)
    pkg.calcSegForce_inplace(dln, mat, sh, net)
    F = pkg.calcSegForce(dln, mat, sh, net)  # the same sum, built in another order
    assert np.abs(net.segForce[:, :, :n] - F).max() <= 1e-12 * np.abs(F).max()
    # idx form: only the listed columns change; they are zeroed first.
    before = net.segForce.copy()
    idx = [4, 11]
    pkg.calcSegForce_inplace(dln, mat, np.asfortranarray(sh[:, [3, 10]]), net, idx)
    changed = np.nonzero(np.any(net.segForce != before, axis=(0, 1)))[0]
    assert set(changed) <= {3, 10}
    Fi = pkg.calcSegForce(dln, mat, np.asfortranarray(sh[:, [3, 10]]), net, idx)
    assert np.abs(net.segForce[:, :, [3, 10]] - Fi).max() <= 1e-12 * np.abs(Fi).max()
