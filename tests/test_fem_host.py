"""The product's mesh geometry for calc_uTilde (ddd.jl_gb300/fem.py) on a
CPU, against the oracle's independent restatement of the reference's mesh
and boundary constructors (oracle/fixtures.py)."""
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
