"""detectCollision and minimumDistance on the GPU (through the C ABI).

Goldens: test/TopologyTest.jl:5-92 (21 detectCollision calls on two networks,
hinge and two-line results) and test/MiscTest.jl:82-150 (12 minimumDistance
cases), both exactly.  Against the oracle (a serial restatement of the
reference loops) every returned value is compared bit for bit, the sign of a
zero included: the GPU evaluates the same FP64 operations in the same order and
selects the pair by the reference's order (largest 1/distSq, then the first
pair), so nothing may differ.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

G_COL = json.load(open(os.path.join(GOLDEN, "collision_goldens.json")))
BURGERS = np.array([[1, 1, 1], [-1, 1, 1], [1, -1, 1], [1, 1, -1]], np.float64) / math.sqrt(3.0)


def _same(a, b):
    if isinstance(a, float) or isinstance(b, float):
        a, b = float(a), float(b)
        return (math.isnan(a) and math.isnan(b)) or (a == b and math.copysign(1, a) == math.copysign(1, b))
    return a == b


def _compare(pkg, oracle, net, cd2, skip=()):
    got, gp = pkg.get_context().detect_collision(cd2, net, skip)
    ref, rp = oracle.detect_collision(cd2, net.coord, net.nodeVel, net.label, net.links, net.bVec, net.connectivity,
                                      net.numNode, net.numSeg, skip)
    assert len(got) == len(ref) and all(_same(a, b) for a, b in zip(got, ref)), (got, ref)
    if got[0]:
        assert all(_same(gp[k], rp[k]) for k in ("distSq", "L1", "L2")), (gp, rp)
    return got


def polygons(pkg, n_loops, seed, box=200.0, rmin=5.0, rmax=40.0, copies=0.2, fixed=0.0):
    """Random planar polygons (3-8 nodes on a circle) in a small cube, Burgers
    vectors from the BCC <111> set; a fraction of loops are followed by a copy
    shifted by 0.5-3 (same b, reversed order, or b negated and reversed:
    the superdislocation filter's cases).  Random node velocities; a fraction
    of nodes fixed (label 2) or surface-mobile (label 3)."""
    rng = np.random.default_rng(seed)
    coords, segs, bv = [], [], []
    node0 = 0

    def add(pts, b):
        nonlocal node0
        m = len(pts)
        for q in range(m):
            coords.append(pts[q])
            segs.append((len(segs) + 1, node0 + q + 1, node0 + (q + 1) % m + 1))
            bv.append(b)
        node0 += m

    for _ in range(n_loops):
        m = int(rng.integers(3, 9))
        c = rng.uniform(0.0, box, 3)
        r = rng.uniform(rmin, rmax)
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        e1 = np.cross(n, rng.normal(size=3))
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(n, e1)
        ang = np.sort(rng.uniform(0.0, 2 * math.pi, m))
        pts = c + r * (np.cos(ang)[:, None] * e1 + np.sin(ang)[:, None] * e2)
        b = BURGERS[rng.integers(4)] * rng.choice([-1.0, 1.0])
        add(pts, b)
        if rng.random() < copies:
            shift = rng.normal(size=3)
            shift *= rng.uniform(0.5, 3.0) / np.linalg.norm(shift)
            kind = rng.integers(3)
            p2 = pts + shift
            if kind == 0:
                add(p2, b)
            elif kind == 1:
                add(p2[::-1], b)
            else:
                add(p2[::-1], -b)
    coord = np.array(coords).T
    seg = np.array(segs, np.int64)
    label = np.ones(coord.shape[1], np.int32)
    u = rng.random(coord.shape[1])
    label[u < fixed] = 2
    label[(u >= fixed) & (u < 1.5 * fixed)] = 3
    net = pkg.DislocationNetwork(coord, np.array(bv).T, seg, maxConnect=4, label=label,
                                 nodeVel=rng.normal(size=coord.shape))
    return net


def hinge_pairs(net):
    """Every pair of links that meet at a node (skipping them all leaves only two-line pairs)."""
    out = []
    for i in range(net.numNode):
        c = net.connectivity[:, i]
        ls = [int(c[2 * k + 1]) for k in range(int(c[0]))]
        out += [(a, b) for q, a in enumerate(ls) for b in ls[q + 1:]]
    return out


def _golden_net(pkg, g):
    links = np.array(g["links"], np.int64)
    n = links.shape[1]
    seg = np.c_[np.arange(1, n + 1), links.T]
    return pkg.DislocationNetwork(np.array(g["coord"]), np.array(g["bVec"]), seg, label=g["label"],
                                  nodeVel=np.array(g["nodeVel"]))


@pytest.mark.parametrize("net_i", range(len(G_COL["networks"])))
def test_golden(pkg, oracle, net_i):
    g = G_COL["networks"][net_i]
    net = _golden_net(pkg, g)
    dln = pkg.DislocationParameters(coreRad=90.78, minSegLen=314.47, maxSegLen=1572.33,
                                    collisionDist=G_COL["collisionDist"])
    for c in g["cases"]:
        skip = [tuple(p) for p in c["skip"]]
        res = pkg.detectCollision(dln, net, skip)
        assert list(res) == c["expected"], (skip, res)
        _compare(pkg, oracle, net, dln.collisionDistSq, skip)


def test_golden_minimum_distance(pkg):
    names = ("x0", "x1", "y0", "y1", "vx0", "vx1", "vy0", "vy1")
    cases = G_COL["minimumDistance"]
    for c in cases:
        got = pkg.minimumDistance(*(np.array(c["inputs"][k]) for k in names))
        assert list(got) == c["expected"], (c, got)
    # The batched form: all cases in one launch.
    batch = pkg.minimumDistance(*(np.array([c["inputs"][k] for c in cases]).T for k in names))
    assert np.array_equal(np.array(batch).T, np.array([c["expected"] for c in cases]))


def test_minimum_distance_vs_oracle(pkg, oracle):
    rng = np.random.default_rng(5)
    n = 4096
    args = [rng.normal(size=(3, n)) * 10 for _ in range(8)]
    args[3][:, :64] = args[2][:, :64]                      # collapsed second segment
    args[1][:, 64:128] = args[0][:, 64:128]                # collapsed first segment
    args[3][:, 128:192] = args[2][:, 128:192] + (args[1][:, 128:192] - args[0][:, 128:192])  # parallel
    got = pkg.minimumDistance(*args)
    ref = oracle.minimum_distance(*args)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r) and np.array_equal(np.signbit(g), np.signbit(r))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_hinge_and_two_line(pkg, oracle, seed):
    net = polygons(pkg, 300, seed, fixed=0.05)
    res = _compare(pkg, oracle, net, 12.0 ** 2)
    assert res[1] == "hinge"
    skip = hinge_pairs(net)
    res = _compare(pkg, oracle, net, 12.0 ** 2, skip)
    assert res[1] == "twoLine"
    # A smaller distance and the two-line pass only: a different pair.
    _compare(pkg, oracle, net, 2.0 ** 2, skip)
    # No candidate anywhere: L1, L2 from the last evaluated two-line pair.
    res = _compare(pkg, oracle, net, 1e-12, skip)
    assert res[:8] == (False, "null", 0, 0, 0, 0, 0, 0)


def test_large_vs_oracle(pkg, oracle):
    net = polygons(pkg, 1200, 9, box=1500.0, fixed=0.02)
    assert net.numSeg > 5000
    skip = hinge_pairs(net)
    assert _compare(pkg, oracle, net, 8.0 ** 2, skip)[1] == "twoLine"
    _compare(pkg, oracle, net, 8.0 ** 2)
    # Repeated calls give the same answer.
    a = pkg.get_context().detect_collision(64.0, net, skip)
    b = pkg.get_context().detect_collision(64.0, net, skip)
    assert a == b


def test_tie_goes_to_the_first_pair(pkg, oracle):
    """Two identical crossings (dyadic coordinates: exactly equal distSq): the
    first pair in the reference's order is reported, whichever lies where."""
    def cross(off):
        return [np.array([0.0, 0.0, 0.0]) + off, np.array([8.0, 0.0, 0.0]) + off,
                np.array([4.0, -4.0, 1.0]) + off, np.array([4.0, 4.0, 1.0]) + off]

    for offs in ([0.0, 1024.0], [1024.0, 0.0]):
        pts = cross(np.array([offs[0], 0, 0])) + cross(np.array([offs[1], 0, 0]))
        coord = np.array(pts).T
        seg = np.array([[1, 1, 2], [2, 3, 4], [3, 5, 6], [4, 7, 8]], np.int64)
        vel = np.zeros_like(coord)
        vel[2, [2, 3, 6, 7]] = -1.0  # the upper segments move down
        b = np.array([[1.0, 1.0, 1.0], [-1.0, 1.0, 1.0], [1.0, 1.0, 1.0], [-1.0, 1.0, 1.0]]).T / math.sqrt(3.0)
        net = pkg.DislocationNetwork(coord, b, seg, nodeVel=vel)
        res = _compare(pkg, oracle, net, 4.0)
        assert res[:8] == (True, "twoLine", 1, 2, 3, 4, 1, 2)


def test_errors(pkg):
    net = polygons(pkg, 10, 4)
    ctx = pkg.get_context()
    bad = pkg.DislocationNetwork(net.coord, net.bVec, net.segIdx, nodeVel=net.nodeVel.copy(), label=net.label)
    bad.nodeVel[1, 3] = np.nan
    with pytest.raises(ValueError):
        ctx.detect_collision(1.0, bad, ())
    bad = pkg.DislocationNetwork(net.coord, net.bVec, net.segIdx, nodeVel=net.nodeVel, label=net.label)
    bad.links[0, 2] = net.numNode + 5
    with pytest.raises(IndexError):
        ctx.detect_collision(1.0, bad, ())


def test_edge_cases(pkg, oracle):
    """No nodes, one segment, every node fixed: nothing to report, and the
    oracle agrees field by field."""
    ctx = pkg.get_context()
    empty = pkg.DislocationNetwork(np.zeros((3, 0)), np.zeros((3, 0)), np.zeros((0, 3), np.int64))
    assert ctx.detect_collision(1.0, empty)[0] == (False, "null", 0, 0, 0, 0, 0, 0, 0.0, 0.0)
    one = pkg.DislocationNetwork(np.array([[0.0, 1.0], [0.0, 0.0], [0.0, 0.0]]), np.ones((3, 1)) / math.sqrt(3.0),
                                 np.array([[1, 1, 2]]), nodeVel=np.array([[0.0, 1.0], [0.0, 0.0], [0.0, 0.0]]))
    assert _compare(pkg, oracle, one, 100.0)[:2] == (False, "null")
    fixed = polygons(pkg, 50, 5)
    fixed.label[:] = 2  # intFixDln: no hinge, no two-line pair is evaluated
    assert _compare(pkg, oracle, fixed, 1e6) == (False, "null", 0, 0, 0, 0, 0, 0, 0.0, 0.0)
