"""BCC mobility on the GPU (through the C ABI).

Goldens: test/MobilityTest.jl:64-93, reached through the GPU pipeline of that
test (calcSegForce! with zero finite-element fields, then dlnMobility): node
forces to 1e-10 relative, velocities at the reference test's own rtol 1e-5 (the
climb drag of 1e10 against glide drags of 1-2 makes the 3×3 solve
ill-conditioned).  Against the oracle on the same segment forces the kernel
runs the same operations in the same order: node forces bit for bit,
velocities to 1e-12.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

G_MOB = json.load(open(os.path.join(GOLDEN, "mobility_goldens.json")))


def _params(pkg):
    p = G_MOB["params"]
    dln = pkg.DislocationParameters(coreRad=p["coreRad"], coreEnergy=p["coreEnergy"], dragCoeffs=p["drag"])
    mat = pkg.MaterialParameters(mu=p["mu"], nu=p["nu"], sigmaPN=p["sigmaPN"])
    return dln, mat


def _mp(dln, mat):
    d = dln.dragCoeffs
    return np.array([mat.σPN, d["edge"], d["screw"], d["climb"], d["line"]])


def test_golden_pipeline(pkg, fixtures):
    fnet = fixtures.make_network(G_MOB["loops"], G_MOB["slipSystems"], G_MOB["range"])
    net = pkg.DislocationNetwork(fnet.coord, fnet.bVec, fnet.segIdx, maxConnect=G_MOB["maxConnect"])
    dln, mat = _params(pkg)
    pkg.calcSegForce_inplace(dln, mat, None, net)
    F, V = pkg.dlnMobility(dln, mat, net)
    gf, gv = np.array(G_MOB["nodeForce"]), np.array(G_MOB["nodeVel"])
    assert np.abs(F.T - gf).max() <= 1e-10 * np.abs(gf).max()
    assert np.linalg.norm(V.T - gv) <= 1e-5 * np.linalg.norm(gv)
    pkg.dlnMobility_inplace(dln, mat, net)
    assert np.array_equal(net.nodeForce[:, :net.numNode], F) and np.array_equal(net.nodeVel[:, :net.numNode], V)


def _random(pkg, synth, loops, seed):
    p, b = synth.square_loops(loops, seed, 50.0, 200.0, 3000.0, 0.5, 0.0)
    coord, bvec, seg = synth.network_arrays(p, b)
    net = pkg.DislocationNetwork(coord, bvec, seg)
    rng = np.random.default_rng(seed)
    net.segForce[...] = rng.normal(size=net.segForce.shape)
    return net


# A node whose segments are collinear has no drag along the line when the line
# drag is 0 (a singular solve, in the reference as well): the straight sides of
# these loops need a line drag.  sigmaPN = 0.01 zeroes part of the segment forces
# (|f| / |t| spans about 0.002 to 0.05 here).
@pytest.mark.parametrize("drag,other_b", [(dict(edge=1.0, screw=2.0, climb=1e10, line=1e-4), False),
                                          (dict(edge=1.0, screw=1.5, climb=10.0, line=0.1), True)])
def test_vs_oracle(pkg, synth, oracle, drag, other_b):
    net = _random(pkg, synth, 50, 7)
    if other_b:
        net.bVec[:, 8:16] *= np.array([[1.0], [1.0], [-0.5]])  # a non-<111> Burgers vector on one loop
    dln = pkg.DislocationParameters(coreRad=1.0, dragCoeffs=drag)
    mat = pkg.MaterialParameters(mu=1.0, nu=0.28, sigmaPN=0.01)
    F, V = pkg.dlnMobility(dln, mat, net)
    rF, rV = oracle.mobility_bcc(_mp(dln, mat), net.coord, net.bVec, net.links, net.connectivity, net.segForce,
                                 net.numNode)
    assert np.array_equal(F, rF) and np.all(np.isfinite(V))
    assert np.abs(V - rV).max() <= 1e-12 * np.abs(rV).max()
    idx = [3, 40, 3, 1]
    Fi, Vi = pkg.dlnMobility(dln, mat, net, idx)
    assert np.array_equal(Fi, F[:, [2, 39, 2, 0]]) and np.array_equal(Vi, V[:, [2, 39, 2, 0]])
    pkg.dlnMobility_inplace(dln, mat, net, [5, 6])
    assert np.array_equal(net.nodeVel[:, [4, 5]], V[:, [4, 5]])
    assert np.all(net.nodeVel[:, 6:] == 0)


def test_errors(pkg, synth):
    net = _random(pkg, synth, 4, 3)
    dln = pkg.DislocationParameters(coreRad=1.0)
    mat = pkg.MaterialParameters(mu=1.0, nu=0.28)
    with pytest.raises(IndexError):  # DDD_ERANGE, Julia's BoundsError
        pkg.dlnMobility(dln, mat, net, [net.numNode + 1])
    net.connectivity[1, 0] = 10 ** 6  # a link that does not exist
    with pytest.raises(IndexError):
        pkg.dlnMobility(dln, mat, net)


def test_isolated_node(pkg, oracle):
    """A node without connections has no force and a singular drag: its
    velocity is NaN (0/0 in the 3x3 solve, as StaticArrays' Cramer solve in the
    reference gives); the other nodes are unaffected."""
    coord = np.array([[0.0, 100.0, 0.0, 500.0], [0.0, 0.0, 100.0, 500.0], [0.0, 0.0, 0.0, 500.0]])
    seg = np.array([[1, 1, 2], [2, 2, 3], [3, 3, 1]])
    b = np.ones((3, 3)) / np.sqrt(3.0)
    net = pkg.DislocationNetwork(coord, b, seg, numNode=4)
    net.segForce[...] = np.random.default_rng(2).normal(size=net.segForce.shape)
    dln = pkg.DislocationParameters(coreRad=1.0, dragCoeffs=dict(edge=1.0, screw=2.0, climb=1e10, line=1e-4))
    mat = pkg.MaterialParameters(mu=1.0, nu=0.28)
    F, V = pkg.dlnMobility(dln, mat, net)
    rF, rV = oracle.mobility_bcc(_mp(dln, mat), net.coord, net.bVec, net.links, net.connectivity, net.segForce,
                                 net.numNode)
    assert np.all(F[:, 3] == 0) and np.all(np.isnan(V[:, 3])) and np.all(np.isnan(rV[:, 3]))
    assert np.array_equal(F, rF) and np.array_equal(V[:, :3], rV[:, :3])
