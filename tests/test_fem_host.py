"""Host-side structures of the product on a CPU, against the oracle's
independent restatements (oracle/fixtures.py): the mesh geometry calc_uTilde
reads (ddd.jl_gb300/fem.py) and a network's node connectivity."""
import numpy as np
import pytest


@pytest.mark.parametrize("dims", [(3.0, 5.0, 7.0, 3, 5, 7), (1000.0, 1000.0, 1000.0, 5, 5, 5),
                                  (20000.0, 8000.0, 12000.0, 8, 4, 6)])
def test_fem_mesh_matches_oracle_restatement(pkg, fixtures, dims):
    """The product's regular-cuboid geometry and cantilever boundary nodes
    (ddd.jl_gb300/fem.py, what calc_uTilde reads) against the oracle's
    independent restatement of buildMesh and Boundaries(::CantileverLoad)
    (oracle/fixtures.py), field by field and bit for bit."""
    mesh = pkg.fem.RegularCuboidMesh(*dims)
    ref = fixtures.cuboid_mesh(*dims)
    assert np.array_equal(mesh.coord, ref["coord"])
    assert np.array_equal(mesh.vertices, ref["vertices"])
    assert np.array_equal(mesh.faceNorm, ref["faceNorm"]) and np.array_equal(mesh.faceMidPt, ref["faceMidPt"])
    assert np.array_equal(mesh.closure, ref["C"])
    assert np.array_equal(mesh.lo, ref["lo"]) and np.array_equal(mesh.hi, ref["hi"])
    nodes, dofs = fixtures.cantilever_u_gamma(*dims[3:])
    bnd = pkg.fem.cantilever_boundaries(mesh)
    assert np.array_equal(bnd.uGammaDln, nodes) and np.array_equal(bnd.uDofsDln, dofs)


def test_network_connectivity_matches_oracle_restatement(pkg, synth, fixtures):
    """The product's default connectivity (what mobility and collision read),
    built from the links, against the oracle's restatement of _makeConnect!
    (DislocationUtil.jl:213-237), including nodes with three or four links."""
    p, b = synth.square_loops(30, 8, 20.0, 200.0, 2000.0, 0.5, 0.1)
    coord, bvec, seg = synth.network_arrays(p, b)
    # Join a few loops at shared nodes: node 1 gains links from 9 and 17.
    seg = seg.copy()
    seg[8, 1] = 1
    seg[16, 1] = 1
    net = pkg.DislocationNetwork(coord, bvec, seg, maxConnect=4)
    ref = fixtures.make_connectivity(net.links, 4)
    assert np.array_equal(net.connectivity[:, :ref.shape[1]], ref)
    assert net.connectivity[0, 0] == 4
