"""The CPU oracle against the reference's own golden vectors (CPU only).

Goldens: test/SegmentForcesTest.jl:281-443 (seg-seg, three networks) and
test/DislocationFEMTest.jl:5-155 (σ̃, edge and screw segment), extracted as
text by tests/golden/extract_goldens.py.  The goldens are printed with 15
decimals (absolute 5e-16 on values ~1e-3) and the networks are rebuilt here
with libm's sin/cos instead of Julia's, so the bound is:
  elementwise |Δ| <= 2e-14 and ||Δ|| / ||golden|| <= 1e-11
(the reference test itself uses isapprox, rtol = sqrt(eps) ≈ 1.5e-8).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

ABS_TOL = 2e-14
REL_TOL = 1e-11


def _segseg_cases():
    g = json.load(open(os.path.join(GOLDEN, "segseg_goldens.json")))
    return g, [c["name"] for c in g["cases"]]


G_SEG, SEG_NAMES = _segseg_cases()
G_SIG = json.load(open(os.path.join(GOLDEN, "sigma_goldens.json")))


def _seg_case(fixtures, name):
    c = next(c for c in G_SEG["cases"] if c["name"] == name)
    p = G_SEG["params"]
    net = fixtures.make_network(c["loops"], G_SEG["slipSystems"], c["range"], c["shift"])
    k5 = fixtures.consts5(p["coreRad"], p["mu"], p["nu"])
    return c, net, k5


def _close(ours, gold):
    d = ours - gold
    assert np.abs(d).max() <= ABS_TOL, np.abs(d).max()
    assert np.linalg.norm(d) <= REL_TOL * np.linalg.norm(gold), np.linalg.norm(d) / np.linalg.norm(gold)


@pytest.mark.parametrize("name", SEG_NAMES)
def test_segseg_serial_matches_golden(oracle, fixtures, name):
    c, net, k5 = _seg_case(fixtures, name)
    F = oracle.segseg_ser(k5, net)
    _close(F[:, 0, :].T, np.array(c["f1"]))
    _close(F[:, 1, :].T, np.array(c["f2"]))


@pytest.mark.parametrize("name", SEG_NAMES)
def test_segseg_threaded_matches_golden(oracle, fixtures, name):
    """calcSegSegForcePar restatement (contiguous i-chunks, atomic adds)."""
    c, net, k5 = _seg_case(fixtures, name)
    for nt in (1, 3, 4):
        F = oracle.segseg_par_atomic(k5, net, nt)
        _close(F[:, 0, :].T, np.array(c["f1"]))
        _close(F[:, 1, :].T, np.array(c["f2"]))
        Fp = oracle.segseg_par_private(k5, net, nt)  # the best-effort CPU baseline form
        _close(Fp[:, 0, :].T, np.array(c["f1"]))
        _close(Fp[:, 1, :].T, np.array(c["f2"]))


@pytest.mark.parametrize("name", SEG_NAMES)
def test_segseg_rows_equal_serial_bitwise(oracle, fixtures, name):
    """The sampled-row form adds each segment's contributions in Ser's order."""
    _, net, k5 = _seg_case(fixtures, name)
    F = oracle.segseg_ser(k5, net)
    rows = np.arange(net.numSeg)
    R = oracle.segseg_rows(k5, net, rows, 2)
    assert np.array_equal(F, R)


def test_segseg_idx_form_matches_all_pairs(oracle, fixtures):
    """SegmentForcesTest.jl:372-380: the idx form equals the all-pairs columns."""
    _, net, k5 = _seg_case(fixtures, "pentagons_shifted")
    F = oracle.segseg_ser(k5, net)
    rng = np.random.default_rng(3)
    idx = rng.integers(1, net.numSeg + 1, net.numSeg // 2)
    Fi = oracle.segseg_idx(k5, net, idx)
    # The idx form evaluates every pair with segment i first, the all-pairs
    # form with the lower index first: same forces up to rounding.
    d = Fi - F[:, :, idx - 1]
    assert np.linalg.norm(d) <= 1e-10 * np.linalg.norm(Fi)


def test_segseg_ext_segments_skipped(oracle, fixtures):
    _, net, k5 = _seg_case(fixtures, "hexagons_prism_shear")
    net.extSeg[[2, 7]] = 1
    F = oracle.segseg_ser(k5, net)
    assert np.all(F[:, :, [2, 7]] == 0)
    keep = [i for i in range(net.numSeg) if i not in (2, 7)]
    # Equivalent to dropping the two segments from the network.
    from oracle.fixtures import Network
    sub = Network(net.coord, net.bVec[:, keep], np.c_[np.arange(1, len(keep) + 1), net.segIdx[keep, 1:]],
                  np.zeros(len(keep), np.uint8), len(keep))
    np.testing.assert_allclose(F[:, :, keep], oracle.segseg_ser(k5, sub), rtol=1e-12, atol=1e-18)


@pytest.mark.parametrize("case", [c["name"] for c in G_SIG["cases"]])
def test_sigma_tilde_matches_golden(oracle, fixtures, case):
    c = next(c for c in G_SIG["cases"] if c["name"] == case)
    net, pts = fixtures.sigma_case_network(c)
    k5 = fixtures.consts5(c["coreRad"], c["mu"], c["nu"])
    sig = oracle.sigma_tilde(k5, pts, net)
    gold = np.array(c["golden"])
    ours = sig.T[:, [0, 1, 2, 3, 5, 4]]  # golden columns are (xx, yy, zz, xy, yz, xz)
    _close(ours, gold)


def test_sigma_threaded_bitwise_equal(oracle, fixtures):
    c = G_SIG["cases"][0]
    net, _ = fixtures.sigma_case_network(c)
    k5 = fixtures.consts5(c["coreRad"], c["mu"], c["nu"])
    rng = np.random.default_rng(0)
    pts = np.asfortranarray(rng.uniform(-400, 400, (3, 500)))
    assert np.array_equal(oracle.sigma_tilde(k5, pts, net, nthreads=1), oracle.sigma_tilde(k5, pts, net, nthreads=4))


def test_opcount_constants(oracle, fixtures):
    """Algorithmic work per unit, from the op-counting instantiation."""
    k5 = fixtures.consts5(1.0, 1.0, 0.28)
    rng = np.random.default_rng(1)
    a = [rng.normal(size=3) * 100 for _ in range(6)]
    c = oracle.opcount_pair(k5, *a)
    flops = c["add"] + c["mul"] + c["div"] + c["sqrt"] + c["log"] + c["atan"]
    assert c["log"] == 8 and c["atan"] == 4 and c["sqrt"] == 10
    assert 1000 < flops < 2000
    s = oracle.opcount_sigma(k5, a[0], a[1], a[2], a[3])
    assert s["sqrt"] == 2 and s["div"] == 3


G_SELF = json.load(open(os.path.join(GOLDEN, "selfforce_goldens.json")))


def _self_case(fixtures):
    c = G_SELF["cases"][0]
    p = G_SELF["params"]
    net = fixtures.make_network(c["loops"], G_SELF["slipSystems"], c["range"], c["shift"])
    k5 = fixtures.consts5(p["coreRad"], p["mu"], p["nu"])
    return c, net, k5, np.array([p["coreRad"], p["coreEnergy"], p["nu"]])


def test_self_force_matches_golden(oracle, fixtures):
    """calcSelfForce (DislocationForces.jl:320-353, 414-455) against
    test/SegmentForcesTest.jl:244-267: node 1 and node 2 forces of every segment."""
    c, net, k5, sc = _self_case(fixtures)
    F1, F2 = oracle.self_force(k5, sc, net)
    _close(F1.T, np.array(c["f1"]))
    _close(F2.T, np.array(c["f2"]))


def test_self_force_idx_and_ext(oracle, fixtures):
    """idx form = the selected columns of the full result (:270-278); the
    external flag is read at the entry's position in idx, as the reference does."""
    c, net, k5, sc = _self_case(fixtures)
    F1, F2 = oracle.self_force(k5, sc, net)
    idx = np.array([3, 9, 1, 3])
    G1, G2 = oracle.self_force(k5, sc, net, idx)
    assert np.array_equal(G1, F1[:, idx - 1]) and np.array_equal(G2, F2[:, idx - 1])
    net.extSeg[1] = 1
    H1, H2 = oracle.self_force(k5, sc, net, idx)
    assert np.all(H1[:, 1] == 0) and np.all(H2[:, 1] == 0)  # entry 2 (segment 9) skipped by extSeg[2]
    assert np.array_equal(H1[:, [0, 2, 3]], G1[:, [0, 2, 3]])


def test_pk_force_formula(oracle, fixtures):
    """(σ̂ b) × t for a random symmetric σ̂, against numpy."""
    c, net, k5, sc = _self_case(fixtures)
    rng = np.random.default_rng(3)
    sh = rng.normal(size=(6, net.numSeg))
    PK = oracle.pk_force(net, sh)
    for q in range(net.numSeg):
        S = np.array([[sh[0, q], sh[3, q], sh[4, q]], [sh[3, q], sh[1, q], sh[5, q]], [sh[4, q], sh[5, q], sh[2, q]]])
        l, a, b = net.segIdx[q] - 1
        t = net.coord[:, b] - net.coord[:, a]
        assert np.allclose(PK[:, q], np.cross(S @ net.bVec[:, l], t), rtol=1e-14, atol=1e-14)


G_MOB = json.load(open(os.path.join(GOLDEN, "mobility_goldens.json")))


def mobility_case(fixtures, oracle):
    """The MobilityTest.jl network and its segment forces as calcSegForce! builds
    them there (zero FE fields: no PK term): seg-seg plus self force."""
    g = G_MOB
    p = g["params"]
    net = fixtures.make_network(g["loops"], g["slipSystems"], g["range"])
    k5 = fixtures.consts5(p["coreRad"], p["mu"], p["nu"])
    seg_force = oracle.segseg_ser(k5, net)
    F1, F2 = oracle.self_force(k5, np.array([p["coreRad"], p["coreEnergy"], p["nu"]]), net)
    seg_force[:, 0, :] += F1
    seg_force[:, 1, :] += F2
    links = np.asfortranarray(net.segIdx[:, 1:3].T)
    conn = fixtures.make_connectivity(links, g["maxConnect"])
    d = p["drag"]
    mp = np.array([p["sigmaPN"], d["edge"], d["screw"], d["climb"], d["line"]])
    return net, seg_force, links, conn, mp


def test_mobility_bcc_matches_golden(oracle, fixtures):
    """dlnMobility (BCC), DislocationMobility.jl:16-178, against
    test/MobilityTest.jl:64-93.  Node forces to 1e-10 relative; velocities at
    the reference test's own rtol 1e-5: the climb drag (1e10) against the glide
    drags (1-2) makes the 3×3 solve ill-conditioned."""
    net, seg_force, links, conn, mp = mobility_case(fixtures, oracle)
    Fn, Vn = oracle.mobility_bcc(mp, net.coord, net.bVec, links, conn, seg_force, conn.shape[1])
    gf, gv = np.array(G_MOB["nodeForce"]), np.array(G_MOB["nodeVel"])
    assert np.abs(Fn.T - gf).max() <= 1e-10 * np.abs(gf).max()
    assert np.linalg.norm(Vn.T - gv) <= 1e-5 * np.linalg.norm(gv)
    idx = np.array([4, 1, 11, 4])
    Fi, Vi = oracle.mobility_bcc(mp, net.coord, net.bVec, links, conn, seg_force, conn.shape[1], idx)
    assert np.array_equal(Fi, Fn[:, idx - 1]) and np.array_equal(Vi, Vn[:, idx - 1])


def test_connectivity_layout(fixtures):
    """_makeConnect! (DislocationUtil.jl:213-237) on a closed 4-node loop."""
    links = np.array([[1, 2, 3, 4], [2, 3, 4, 1]])
    conn = fixtures.make_connectivity(links, 4)
    assert conn[:, 0].tolist() == [2, 1, 1, 4, 2, 0, 0, 0, 0]
    assert conn[:, 2].tolist() == [2, 2, 2, 3, 1, 0, 0, 0, 0]


G_COL = json.load(open(os.path.join(GOLDEN, "collision_goldens.json")))


def collision_net(fixtures, g):
    """A TopologyTest.jl network as its constructor and makeConnect! build it."""
    links = np.asfortranarray(np.array(g["links"], np.int64))
    return (np.asfortranarray(g["coord"], np.float64), np.asfortranarray(g["nodeVel"], np.float64),
            np.array(g["label"], np.int32), links, np.asfortranarray(g["bVec"], np.float64),
            fixtures.make_connectivity(links, 4))


@pytest.mark.parametrize("net_i", range(len(G_COL["networks"])))
def test_detect_collision_matches_golden(oracle, fixtures, net_i):
    """detectCollision (DislocationTopologyCollision.jl:1-221) against
    test/TopologyTest.jl:5-92: every skip list, all ten returned values exactly."""
    g = G_COL["networks"][net_i]
    coord, vel, label, links, bvec, conn = collision_net(fixtures, g)
    cd2 = G_COL["collisionDist"] * G_COL["collisionDist"]
    for c in g["cases"]:
        res, _ = oracle.detect_collision(cd2, coord, vel, label, links, bvec, conn, coord.shape[1], links.shape[1],
                                         [tuple(p) for p in c["skip"]])
        assert list(res) == c["expected"], (c["skip"], res)


def test_minimum_distance_matches_golden(oracle):
    """minimumDistance (Misc.jl:314-367) against test/MiscTest.jl:82-150."""
    for c in G_COL["minimumDistance"]:
        v = c["inputs"]
        out = oracle.minimum_distance(*(np.array(v[k]) for k in ("x0", "x1", "y0", "y1", "vx0", "vx1", "vy0", "vy1")))
        assert [float(o[0]) for o in out] == c["expected"], (v, out)


G_U = json.load(open(os.path.join(GOLDEN, "u_tilde_goldens.json")))


def u_tilde_case(fixtures):
    """The DislocationFEMTest.jl "Calculate uTilde" setup: mesh, network, the
    cantilever's displacement nodes and dofs, (omνInv8π, om2νomνInv8π)."""
    g, m = G_U, G_U["mesh"]
    mesh = fixtures.cuboid_mesh(m["dx"], m["dy"], m["dz"], m["mx"], m["my"], m["mz"])
    net = fixtures.make_network(g["loops"], g["slipSystems"], g["range"])
    nodes, dofs = fixtures.cantilever_u_gamma(m["mx"], m["my"], m["mz"])
    nu = g["nu"]
    om_nu_inv8pi = (1 / (1 - nu)) / (8 * np.pi)
    return mesh, net, nodes, dofs, np.array([om_nu_inv8pi, (1 - 2 * nu) * om_nu_inv8pi])


def test_u_tilde_matches_golden(oracle, fixtures):
    """calc_uTilde (DislocationFEM.jl:355-707) against
    test/DislocationFEMTest.jl:270-1000 (the test's rtol is 5e-5; the restatement
    agrees to 1e-12), and calc_uTilde!'s full vector through uDofsDln."""
    mesh, net, nodes, dofs, k2 = u_tilde_case(fixtures)
    pts = np.asfortranarray(mesh["coord"][:, nodes - 1])
    links = np.asfortranarray(net.segIdx[:, 1:3].T)
    label = np.ones(net.coord.shape[1], np.int32)
    u, ntri = oracle.u_tilde(k2, mesh, mesh["faceNorm"][:, 0:5:2], pts, net.coord, label, links, net.bVec,
                             net.coord.shape[1], net.numSeg)
    assert ntri == 16
    for c, key in enumerate(("ux", "uy", "uz")):
        gold = np.array(G_U[key])
        assert np.linalg.norm(u[c] - gold) <= 1e-12 * np.linalg.norm(gold)
    full = np.zeros(mesh["coord"].shape[1] * 3)
    flat = u.ravel(order="F")
    for k, d in enumerate(dofs):
        full[d - 1] += flat[k]
    gold = np.array(G_U["uTildeFull"])
    assert np.linalg.norm(full - gold) <= 1e-12 * np.linalg.norm(gold)
