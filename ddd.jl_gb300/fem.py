"""The finite-element data calc_uTilde reads, for a regular cuboid mesh.

Only the geometry of the reference's mesh and boundary constructors is kept
(no stiffness matrix, no solver): FE node coordinates, the 8 vertices, face
normals and midpoints, the surface node sets, and the cantilever's
displacement nodes and dofs.  Layouts and numbering follow
src/Type/FEMConstructor.jl (buildMesh for a regular cuboid :130-480, surface
node sets :274-300 and :495-545, Boundaries for CantileverLoad :761-850 and
:968-987), so arrays built here equal the reference's.
"""
import numpy as np


class RegularCuboidMesh:
    """[0, dx] x [0, dy] x [0, dz] cut into mx x my x mz hexahedra.

    coord: 3 x (mx+1)(my+1)(mz+1), node i + (j-1)(mx+1) + (k-1)(mx+1)(my+1)
    (1-based) at ((i-1) dx/mx, (j-1) dy/my, (k-1) dz/mz).  faceNorm and
    faceMidPt: 3 x 6, faces in the order xz@y0, yz@x1, xz@y1, yz@x0, xy@z0,
    xy@z1.  closure: mean of the vertices (the point C of calc_uTilde).
    normals: the projection directions calc_uTilde uses for a regular cuboid,
    faceNorm[:, 1:2:5].
    """

    def __init__(self, dx, dy, dz, mx, my, mz):
        self.dx, self.dy, self.dz = float(dx), float(dy), float(dz)
        self.mx, self.my, self.mz = int(mx), int(my), int(mz)
        w, h, d = self.dx / mx, self.dy / my, self.dz / mz
        mx1, my1, mz1 = mx + 1, my + 1, mz + 1
        i = np.arange(mx1, dtype=np.float64)
        j = np.arange(my1, dtype=np.float64)
        k = np.arange(mz1, dtype=np.float64)
        K, J, I = np.meshgrid(k, j, i, indexing="ij")
        self.coord = np.asfortranarray(np.stack([(I * w).ravel(), (J * h).ravel(), (K * d).ravel()]))
        self.numNode = self.coord.shape[1]
        dx_, dy_, dz_ = self.dx, self.dy, self.dz
        self.vertices = np.array([[0, 0, 0], [dx_, 0, 0], [dx_, dy_, 0], [0, dy_, 0], [0, 0, dz_], [dx_, 0, dz_],
                                  [dx_, dy_, dz_], [0, dy_, dz_]], np.float64).T
        faces = np.array([[1, 2, 6, 5], [2, 3, 7, 6], [3, 4, 8, 7], [4, 1, 5, 8], [4, 3, 2, 1], [5, 6, 7, 8]]) - 1
        mid = np.zeros((3, 6))
        for f in range(6):
            s = self.vertices[:, faces[f, 0]].copy()
            for q in range(1, 4):
                s = s + self.vertices[:, faces[f, q]]
            mid[:, f] = s / 4
        self.faceMidPt = np.asfortranarray(mid)
        self.faceNorm = np.asfortranarray(np.array([[0, -1, 0], [1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, 0, -1],
                                                    [0, 0, 1]], np.float64).T)
        c = self.vertices[:, 0].copy()
        for q in range(1, 8):
            c = c + self.vertices[:, q]
        self.closure = c / 8
        self.lo = self.vertices.min(axis=1)
        self.hi = self.vertices.max(axis=1)
        self.normals = np.asfortranarray(self.faceNorm[:, 0:5:2])
        self.surfNode = self._surface_nodes()

    def _surface_nodes(self):
        mx, my, mz = self.mx, self.my, self.mz
        mx1, my1, mz1 = mx + 1, my + 1, mz + 1
        top = mx1 * my1 * mz
        s = {
            "x0y0z0": [1], "x1y0z0": [mx1], "x1y1z0": [mx1 * my1], "x0y1z0": [mx1 * my + 1],
            "x0y0z1": [1 + top], "x1y0z1": [mx1 + top], "x1y1z1": [mx1 * my1 * mz1],
            "x0y1z1": [mx1 * my + 1 + top],
            "x_y0z0": [i + 1 for i in range(1, mx)], "x_y1z0": [i + 1 + mx1 * my for i in range(1, mx)],
            "x_y0z1": [i + 1 + top for i in range(1, mx)], "x_y1z1": [i + 1 + top + mx1 * my for i in range(1, mx)],
            "y_x0z0": [i * mx1 + 1 for i in range(1, my)], "y_x1z0": [i * mx1 + mx1 for i in range(1, my)],
            "y_x0z1": [i * mx1 + 1 + top for i in range(1, my)], "y_x1z1": [i * mx1 + mx1 + top for i in range(1, my)],
            "z_x0y0": [i * mx1 * my1 + 1 for i in range(1, mz)],
            "z_x1y0": [i * mx1 * my1 + mx1 for i in range(1, mz)],
            "z_x0y1": [i * mx1 * my1 + 1 + mx1 * my for i in range(1, mz)],
            "z_x1y1": [i * mx1 * my1 + mx1 + mx1 * my for i in range(1, mz)],
            "xy_z0": [j * mx1 + 1 + i for j in range(1, my) for i in range(1, mx)],
            "xy_z1": [j * mx1 + 1 + i + top for j in range(1, my) for i in range(1, mx)],
            "xz_y0": [j * mx1 * my1 + 1 + i for j in range(1, mz) for i in range(1, mx)],
            "xz_y1": [j * mx1 * my1 + 1 + i + mx1 * my for j in range(1, mz) for i in range(1, mx)],
            "yz_x0": [j * mx1 * my1 + 1 + i * mx1 for j in range(1, mz) for i in range(1, my)],
            "yz_x1": [j * mx1 * my1 + mx1 + i * mx1 for j in range(1, mz) for i in range(1, my)],
        }
        return {k: np.array(v, np.int64) for k, v in s.items()}


class Boundaries:
    """The Boundaries fields calc_uTilde reads: uGammaDln (FE nodes with applied
    displacements, 1-based) and uDofsDln = [3u-2; 3u-1; 3u]."""

    def __init__(self, uGammaDln):
        self.uGammaDln = np.asarray(uGammaDln, np.int64)
        u = self.uGammaDln
        self.uDofsDln = np.concatenate([3 * u - 2, 3 * u - 1, 3 * u])


def cantilever_boundaries(mesh):
    """Boundaries(::CantileverLoad, mesh): uGamma = the x0 face with its edges
    and corners (surface sets in the reference's order), then mGamma = the
    x1/z1 edge and its corners."""
    u = ["x0y0z0", "x0y1z0", "x0y0z1", "x0y1z1", "y_x0z0", "y_x0z1", "z_x0y0", "z_x0y1", "yz_x0"]
    m = ["x1y0z1", "x1y1z1", "y_x1z1"]
    return Boundaries(np.concatenate([mesh.surfNode[k] for k in u + m]))


class ForceDisplacement:
    """The uTilde field of ForceDisplacement: 3 x numNode of the mesh, flat."""

    def __init__(self, mesh):
        self.uTilde = np.zeros(3 * mesh.numNode)
