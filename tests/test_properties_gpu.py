"""Size-independent properties at the workloads' full sizes (GPU).

The oracle checks sampled rows at these sizes (test_segseg_gpu.py,
test_sigma_gpu.py); here every output is checked through properties that hold
exactly in floating point:

* the pair force is bilinear in the two Burgers vectors and every scaling
  below is by a power of two, which commutes with rounding: doubling every b
  multiplies every node force by exactly 4, negating every b leaves the forces
  bit for bit unchanged; the field stress σ̃ and the displacement ũ are linear
  in b (doubling b doubles them exactly);
* the surrogate form keeps the same structure (the network sees only the
  geometry; the Burgers vectors enter through an exact contraction), so it is
  exactly bilinear too, the audit and near-pair routing being scale-free;
* relabelling the segments permutes the forces (to the reference formula's
  own asymmetry in near-parallel pairs).

(Total force is not a property here: the near-parallel branch's projection
does not conserve it exactly.)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net(pkg, synth, config, seed, scale=1.0, loops=None):
    p, b, cfg = synth.make(config, seed=seed, num_loops=loops)
    coord, bvec, seg = synth.network_arrays(p, b)
    return pkg.DislocationNetwork(coord, bvec * scale, seg), cfg, p, b


def _params(pkg, synth):
    return pkg.DislocationParameters(coreRad=synth.CORE_RAD), pkg.MaterialParameters(mu=synth.MU, nu=synth.NU)


def test_force_bilinear_in_burgers_vectors_32k(pkg, synth):
    """32,768 segments (the GPU-scale parity workload), all pairs, FP64."""
    dln, mat = _params(pkg, synth)
    net, _, _, _ = _net(pkg, synth, "gpu32k", 3)
    F = pkg.calcSegSegForce(dln, mat, net)
    F2 = pkg.calcSegSegForce(dln, mat, _net(pkg, synth, "gpu32k", 3, 2.0)[0])
    assert np.array_equal(F2, 4.0 * F)
    Fn = pkg.calcSegSegForce(dln, mat, _net(pkg, synth, "gpu32k", 3, -1.0)[0])
    assert np.array_equal(Fn, F)


@pytest.mark.parametrize("mode", ["f32c", "df64"])
def test_precision_forms_bilinear(pkg, synth, mode):
    """The precision forms at 32,768 segments keep the exact bilinearity."""
    dln, mat = _params(pkg, synth)
    ctx = pkg.get_context()
    ctx.mode = mode
    try:
        F = pkg.calcSegSegForce(dln, mat, _net(pkg, synth, "gpu32k", 5)[0])
        F2 = pkg.calcSegSegForce(dln, mat, _net(pkg, synth, "gpu32k", 5, 2.0)[0])
    finally:
        ctx.mode = "fp64"
    assert np.array_equal(F2, 4.0 * F)


def test_permutation_32k(pkg, synth):
    """The segments of the 32,768-segment network relabelled at random: the
    same forces, permuted.  Not to rounding: a relabelling can swap which
    segment of a pair is the reference's first, and its near-parallel branch
    projects the second onto the first's line, so such pairs change at the
    1e-8 level (the CPU oracle shows the same: 2e-9 normwise, 1.6e-8 of the
    largest force at 2,400 segments).  A wrong index map would differ by
    O(1)."""
    dln, mat = _params(pkg, synth)
    net, _, _, _ = _net(pkg, synth, "gpu32k", 6)
    F = pkg.calcSegSegForce(dln, mat, net)
    perm = np.random.default_rng(1).permutation(net.numSeg)
    seg = net.segIdx.copy()[perm]
    seg[:, 0] = np.arange(1, net.numSeg + 1)
    netp = pkg.DislocationNetwork(net.coord, net.bVec[:, perm], seg)
    Fp = pkg.calcSegSegForce(dln, mat, netp)
    G = F[:, :, perm]
    assert np.linalg.norm(Fp - G) <= 1e-8 * np.linalg.norm(G)
    d = np.linalg.norm(Fp - G, axis=0)
    assert d.max() <= 1e-7 * np.linalg.norm(G, axis=0).max()


def test_sigma_linear_in_burgers_vectors(pkg, synth):
    """σ̃ of the 32,768-segment network at the 2^18 points of a 64^3 grid."""
    dln, mat = _params(pkg, synth)
    net, cfg, _, _ = _net(pkg, synth, "gpu32k", 4)
    pts = synth.grid_points(64, cfg["cube"])
    S = pkg.calc_σTilde(pts, dln, mat, net)
    S2 = pkg.calc_σTilde(pts, dln, mat, _net(pkg, synth, "gpu32k", 4, 2.0)[0])
    assert np.array_equal(S2, 2.0 * S)


def test_surrogate_bilinear_65k(pkg, synth):
    """The surrogate form at 65,536 segments with the committed checkpoint:
    doubling every b quadruples every force, the audit's estimate unchanged."""
    import bench

    dln, mat = _params(pkg, synth)
    sur = pkg.Surrogate(pkg.get_context()).load(bench.SURROGATE_CKPT)
    F, rep = sur.force_network(dln, mat, _net(pkg, synth, "gpu65k", 0)[0], exact_mode="f32c")
    F2, rep2 = sur.force_network(dln, mat, _net(pkg, synth, "gpu65k", 0, 2.0)[0], exact_mode="f32c")
    assert rep["fallback"] == 0 and rep2["fallback"] == 0
    assert rep2["audit_node_rel_rms"] == rep["audit_node_rel_rms"]
    assert np.array_equal(F2, 4.0 * F)


def test_u_tilde_linear_in_burgers_vectors(pkg, synth):
    """calc_uTilde of the 65,536-segment network at the 4,290 displacement
    nodes of a 64^3-element mesh over its cube."""
    net, cfg, _, _ = _net(pkg, synth, "gpu65k", 0)
    net2 = _net(pkg, synth, "gpu65k", 0, 2.0)[0]
    mesh = pkg.fem.RegularCuboidMesh(cfg["cube"], cfg["cube"], cfg["cube"], 64, 64, 64)
    bnd = pkg.fem.cantilever_boundaries(mesh)
    mat = pkg.MaterialParameters(mu=1.0, nu=0.28)
    u = pkg.calc_uTilde(mesh, bnd, mat, net)
    assert np.array_equal(pkg.calc_uTilde(mesh, bnd, mat, net2), 2.0 * u)


def test_banded_65k(pkg, synth):
    """The 65,536-segment workload (512 tiles, 131,328 tile pairs, 1.6 GB of
    partial sums) in the f32c form with the partial-sum buffer capped at 256
    MiB (7 bands of at most 21,845 tile pairs): the unbanded forces to
    rounding, bilinear as exactly as the unbanded form."""
    dln, mat = _params(pkg, synth)
    ctx = pkg.get_context()
    ctx.mode = "f32c"
    try:
        net = _net(pkg, synth, "gpu65k", 0)[0]
        F = pkg.calcSegSegForce(dln, mat, net)
        ctx.partial_limit = 256 << 20
        Fb = pkg.calcSegSegForce(dln, mat, net)
        F2 = pkg.calcSegSegForce(dln, mat, _net(pkg, synth, "gpu65k", 0, 2.0)[0])
    finally:
        ctx.partial_limit = 0
        ctx.mode = "fp64"
    assert np.linalg.norm(Fb - F) <= 1e-13 * np.linalg.norm(F)
    assert np.array_equal(F2, 4.0 * Fb)
