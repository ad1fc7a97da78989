"""calc_uTilde / calc_uTilde! on the GPU (through the C ABI).

Goldens: test/DislocationFEMTest.jl:270-1000 (internal loops in a 3 x 5 x 7
cuboid; the reference test's rtol is 5e-5, the CPU restatement agrees to 3e-13).
Against the oracle, on networks that cross the mesh surface (external nodes,
surface nodes, projections out of faces, edges and corners), each point's sum
runs over the same triangles in the same order with the same FP64 operations;
only CUDA's acos / tan / atan / log differ from the C library's in the last
ulp.  Surface nodes close to the edges of the large external closure
triangles make the solid angle ill-conditioned, and there the reference's own
FP64 arithmetic is off from a long double evaluation of the same triangles by
up to ~3e-9 of the largest displacement.  So, as for the seg-seg force: the
GPU's error against long double must stay within 3x the reference
arithmetic's, and per point |u_gpu - u_oracle| <= 1e-12 max|u| + 4 x that
error.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

G_U = json.load(open(os.path.join(GOLDEN, "u_tilde_goldens.json")))


def _golden(pkg, fixtures):
    g, m = G_U, G_U["mesh"]
    mesh = pkg.fem.RegularCuboidMesh(m["dx"], m["dy"], m["dz"], m["mx"], m["my"], m["mz"])
    fnet = fixtures.make_network(g["loops"], g["slipSystems"], g["range"])
    net = pkg.DislocationNetwork(fnet.coord, fnet.bVec, fnet.segIdx)
    mat = pkg.MaterialParameters(mu=g["mu"], nu=g["nu"])
    return mesh, pkg.fem.cantilever_boundaries(mesh), mat, net


def test_golden(pkg, fixtures):
    mesh, bnd, mat, net = _golden(pkg, fixtures)
    u = pkg.calc_uTilde(mesh, bnd, mat, net)
    for c, key in enumerate(("ux", "uy", "uz")):
        gold = np.array(G_U[key])
        assert np.linalg.norm(u[c::3] - gold) <= 1e-11 * np.linalg.norm(gold)
    fd = pkg.fem.ForceDisplacement(mesh)
    fd.uTilde[:] = 7.0  # calc_uTilde! zeroes it first
    pkg.calc_uTilde_inplace(fd, mesh, bnd, mat, net)
    gold = np.array(G_U["uTildeFull"])
    assert np.linalg.norm(fd.uTilde - gold) <= 1e-11 * np.linalg.norm(gold)
    # The reference's own consistency check: uTilde == uTilde![uDofsDln].
    assert np.array_equal(fd.uTilde[bnd.uDofsDln - 1], u)


def crossing_network(pkg, seed, n_loops=60, size=1000.0):
    """Random polygons around a size^3 box, many crossing its surface: nodes
    outside are external (5); an inside node joined to an outside one is made a
    surface node (3) in half the cases, so some segments only record a surface
    connection and some external nodes take the surface node as their
    projection."""
    rng = np.random.default_rng(seed)
    coords, segs, bv = [], [], []
    for _ in range(n_loops):
        m = int(rng.integers(4, 9))
        c = rng.uniform(-0.2 * size, 1.2 * size, 3)
        r = rng.uniform(0.05, 0.3) * size
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        e1 = np.cross(n, rng.normal(size=3))
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(n, e1)
        ang = np.sort(rng.uniform(0, 2 * math.pi, m))
        base = len(coords)
        for q in range(m):
            coords.append(c + r * (math.cos(ang[q]) * e1 + math.sin(ang[q]) * e2))
        b = rng.normal(size=3)
        b /= np.linalg.norm(b)
        for q in range(m):
            segs.append((len(segs) + 1, base + q + 1, base + (q + 1) % m + 1))
            bv.append(b)
    coord = np.array(coords).T
    outside = np.any((coord < 0) | (coord > size), axis=0)
    label = np.where(outside, 5, 1).astype(np.int32)
    for _, a, b in segs:
        for x, y in ((a, b), (b, a)):
            if not outside[x - 1] and outside[y - 1] and rng.random() < 0.5:
                label[x - 1] = 3
    return pkg.DislocationNetwork(coord, np.array(bv).T, np.array(segs, np.int64), label=label)


def _oracle_u(oracle, mat, mesh, pts, net, long_double=False):
    md = {"faceNorm": mesh.faceNorm, "faceMidPt": mesh.faceMidPt, "C": mesh.closure, "lo": mesh.lo, "hi": mesh.hi}
    return oracle.u_tilde([mat.omνInv8π, mat.om2νomνInv8π], md, mesh.normals, pts, net.coord, net.label, net.links,
                          net.bVec, net.numNode, net.numSeg, long_double=long_double, nthreads=4)


@pytest.mark.parametrize("seed", [1, 2])
def test_crossing_network_vs_oracle(pkg, oracle, seed):
    # 5 x 5 x 5: no FE node at the closure point C (the mesh centre), where the
    # full triangle's log term divides by zero, in the reference as well.
    mesh = pkg.fem.RegularCuboidMesh(1000.0, 1000.0, 1000.0, 5, 5, 5)
    net = crossing_network(pkg, seed)
    assert (net.label == 5).sum() > 20 and (net.label == 3).sum() > 3
    mat = pkg.MaterialParameters(mu=1.0, nu=0.3)
    pts = np.asfortranarray(mesh.coord)
    ref, ntri = _oracle_u(oracle, mat, mesh, pts, net)
    assert ntri > net.numSeg  # external segments give five triangles
    u = pkg.get_context().u_tilde(mat.omνInv8π, mat.om2νomνInv8π, mesh, pts, net).reshape(3, -1, order="F")
    ld, _ = _oracle_u(oracle, mat, mesh, pts, net, long_double=True)
    noise = np.abs(ref - ld).max()
    scale = np.abs(ref).max()
    assert np.abs(u - ld).max() <= 3 * noise + 1e-13 * scale
    assert np.abs(u - ref).max() <= 1e-12 * scale + 4 * noise


@pytest.mark.parametrize("seed", [1, 2])
def test_fast_form(pkg, oracle, fixtures, seed):
    """The reformulated FP64 kernel (one atan2 solid angle; selected by any mode
    other than strict "fp64"): the goldens to 1e-11, and on the crossing
    networks the same accuracy bound against long double as the strict form."""
    ctx = pkg.get_context()
    ctx.mode = "fp64_fma"
    try:
        mesh, bnd, mat, net = _golden(pkg, fixtures)
        u = pkg.calc_uTilde(mesh, bnd, mat, net)
        for c, key in enumerate(("ux", "uy", "uz")):
            gold = np.array(G_U[key])
            assert np.linalg.norm(u[c::3] - gold) <= 1e-11 * np.linalg.norm(gold)
        mesh = pkg.fem.RegularCuboidMesh(1000.0, 1000.0, 1000.0, 5, 5, 5)
        net = crossing_network(pkg, seed)
        mat = pkg.MaterialParameters(mu=1.0, nu=0.3)
        pts = np.asfortranarray(mesh.coord)
        ref, _ = _oracle_u(oracle, mat, mesh, pts, net)
        ld, _ = _oracle_u(oracle, mat, mesh, pts, net, long_double=True)
        noise = np.abs(ref - ld).max()
        u = ctx.u_tilde(mat.omνInv8π, mat.om2νomνInv8π, mesh, pts, net).reshape(3, -1, order="F")
        assert np.abs(u - ld).max() <= 3 * noise + 1e-13 * np.abs(ref).max()
    finally:
        ctx.mode = "fp64"


def test_dofs_scatter(pkg, fixtures):
    mesh, bnd, mat, net = _golden(pkg, fixtures)
    pts = np.asfortranarray(mesh.coord[:, bnd.uGammaDln - 1])
    u = pkg.get_context().u_tilde(mat.omνInv8π, mat.om2νomνInv8π, mesh, pts, net)
    out = np.arange(3 * mesh.numNode, dtype=np.float64)
    pkg.get_context().u_tilde(mat.omνInv8π, mat.om2νomνInv8π, mesh, pts, net, bnd.uDofsDln, out)
    want = np.arange(3 * mesh.numNode, dtype=np.float64)
    for k, dof in enumerate(bnd.uDofsDln):
        want[dof - 1] += u[k]
    assert np.array_equal(out, want)


def test_errors(pkg, fixtures):
    mesh, bnd, mat, net = _golden(pkg, fixtures)
    ctx = pkg.get_context()
    pts = np.asfortranarray(mesh.coord[:, :4])
    with pytest.raises(IndexError):
        ctx.u_tilde(mat.omνInv8π, mat.om2νomνInv8π, mesh, pts, net, np.full(12, 10 ** 6), np.zeros(10))
    bad = pkg.DislocationNetwork(net.coord, net.bVec, net.segIdx)
    bad.links[1, 3] = 0
    with pytest.raises(IndexError):
        ctx.u_tilde(mat.omνInv8π, mat.om2νomνInv8π, mesh, pts, bad)
    pts = pts.copy()
    pts[0, 1] = np.inf
    with pytest.raises(ValueError):
        ctx.u_tilde(mat.omνInv8π, mat.om2νomνInv8π, mesh, pts, net)


def test_no_segments(pkg, fixtures):
    """A network without segments displaces nothing."""
    mesh, bnd, mat, _ = _golden(pkg, fixtures)
    empty = pkg.DislocationNetwork(np.zeros((3, 0)), np.zeros((3, 0)), np.zeros((0, 3), np.int64))
    assert not np.any(pkg.calc_uTilde(mesh, bnd, mat, empty))
