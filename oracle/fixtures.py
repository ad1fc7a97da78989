"""Test fixtures: the reference's loop and network generators, restated in Python.

Test infrastructure only.  Rebuilds the exact networks the reference's golden
tests are computed on, so the oracle (and through it the GPU path) can be
checked against those goldens.

Restated from (paths within the DDD.jl project):
  src/Misc/Misc.jl:143-207                    internalAngle / externalAngle / rot3D
  src/Type/DislocationConstructor.jl:196-298  DislocationLoop (loopPure: prism / shear)
  src/Type/DislocationConstructor.jl:477-551  DislocationNetwork(sources; memBuffer)
  src/Type/DislocationConstructor.jl:645-688  makeNetwork!
  src/Type/DislocationUtil.jl:96-152          loopDistribution(Zeros), limits!, translatePoints!
  src/Type/DislocationUtil.jl:161-164         makeSegment(segEdge)
  src/Type/DislocationUtil.jl:253-295         getSegmentIdx
  src/Type/MaterialConstructor.jl:42-82       MaterialParameters derived constants
"""
import math

import numpy as np

EXT_DLN = 5  # nodeTypeDln.extDln (src/Type/DislocationType.jl:24-32)


def material_constants(mu, nu):
    """(μ4π, μ8π, μ4πν, νμ4πν) as MaterialParameters computes them (MaterialConstructor.jl:66-82)."""
    om_nu_inv = 1.0 / (1.0 - nu)
    mu4pi = mu / (4.0 * math.pi)
    mu8pi = mu4pi / 2.0
    mu4pinu = mu4pi * om_nu_inv
    nu_mu4pinu = nu * mu4pinu
    return mu4pi, mu8pi, mu4pinu, nu_mu4pinu


def consts5(core_rad, mu, nu):
    """Oracle constant vector (aSq, μ4π, μ8π, μ4πν, νμ4πν); aSq = coreRad^2 (DislocationConstructor.jl:83)."""
    mu4pi, mu8pi, mu4pinu, nu_mu4pinu = material_constants(mu, nu)
    return np.array([core_rad * core_rad, mu4pi, mu8pi, mu4pinu, nu_mu4pinu], dtype=np.float64)


def _norm3(v):
    return math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])


def external_angle(n):
    internal = (n - 2) * math.pi / n
    return math.pi - internal


def rot3D(xyz, uvw, abc, theta):
    """Rotate xyz about the axis uvw through abc by theta (Misc.jl:185-207)."""
    inv = 1.0 / _norm3(uvw)
    u = [inv * uvw[0], inv * uvw[1], inv * uvw[2]]
    c = math.cos(theta)
    omc = 1.0 - c
    s = math.sin(theta)
    xdu = xyz[0] * u[0] + xyz[1] * u[1] + xyz[2] * u[2]
    return [
        (abc[0] * (u[1] * u[1] + u[2] * u[2]) - u[0] * (abc[1] * u[1] + abc[2] * u[2] - xdu)) * omc
        + xyz[0] * c
        + s * (-abc[2] * u[1] + abc[1] * u[2] - u[2] * xyz[1] + u[1] * xyz[2]),
        (abc[1] * (u[0] * u[0] + u[2] * u[2]) - u[1] * (abc[0] * u[0] + abc[2] * u[2] - xdu)) * omc
        + xyz[1] * c
        + s * (abc[2] * u[0] - abc[0] * u[2] + u[2] * xyz[0] - u[0] * xyz[2]),
        (abc[2] * (u[0] * u[0] + u[1] * u[1]) - u[2] * (abc[0] * u[0] + abc[1] * u[1] - xdu)) * omc
        + xyz[2] * c
        + s * (-abc[1] * u[0] + abc[0] * u[1] - u[1] * xyz[0] + u[0] * xyz[1]),
    ]


def make_loop(loop_type, num_sides, node_side, seg_len, slip_plane, b_vec):
    """Coordinates (nodeTotal×3) of one centred loop (DislocationConstructor.jl:196-298)."""
    node_total = num_sides * node_side
    if np.isscalar(seg_len):
        seg_len = [float(seg_len)] * node_total
    n_len = len(seg_len)
    n = [float(v) for v in slip_plane]
    b = [float(v) for v in b_vec]
    nn, nb = _norm3(n), _norm3(b)
    n = [v / nn for v in n]
    b = [v / nb for v in b]
    rot_axis = n if loop_type == "shear" else b
    # makeSegment(segEdge(), n, b) = (n × b) / |n × b|
    e = [n[1] * b[2] - n[2] * b[1], n[2] * b[0] - n[0] * b[2], n[0] * b[1] - n[1] * b[0]]
    ne = _norm3(e)
    e = [v / ne for v in e]
    segs = [[e[0] * L, e[1] * L, e[2] * L] for L in seg_len]
    theta = external_angle(num_sides)
    coord = [[0.0, 0.0, 0.0] for _ in range(node_total)]
    for i in range(1, num_sides + 1):
        idx = (i - 1) * node_side
        mod_idx = (i - 1) % n_len
        rseg = rot3D(segs[mod_idx], rot_axis, [0.0, 0.0, 0.0], theta * (i - 1))
        for j in range(1, node_side + 1):
            if i == j == 1:
                coord[0] = [0.0, 0.0, 0.0]
                continue
            if idx + j <= node_total:
                prev = coord[idx + j - 2]
                cur = coord[idx + j - 1]
                coord[idx + j - 1] = [cur[k] + (prev[k] + rseg[k]) for k in range(3)]
    mean = [0.0, 0.0, 0.0]
    for p in coord:
        for k in range(3):
            mean[k] += p[k]
    mean = [m / node_total for m in mean]
    coord = [[p[k] - mean[k] for k in range(3)] for p in coord]
    return coord, b


class Network:
    """Arrays in the reference's DislocationNetwork layout, column-major, 1-based indices.

    coord (3×nodeBuf), bVec (3×linkBuf), segIdx (linkBuf×3: link, node1, node2),
    extSeg (linkBuf bools), numSeg.  numpy stores them Fortran-ordered so
    `.ravel(order="F")` is the exact Julia memory image.
    """

    def __init__(self, coord, bvec, seg_idx, ext_seg, num_seg, label=None):
        self.coord = np.asfortranarray(coord, dtype=np.float64)
        self.bVec = np.asfortranarray(bvec, dtype=np.float64)
        self.segIdx = np.asfortranarray(seg_idx, dtype=np.int64)
        self.extSeg = np.ascontiguousarray(ext_seg, dtype=np.uint8)
        self.numSeg = int(num_seg)
        self.label = label
        self.segForce = np.zeros((3, 2, self.bVec.shape[1]), dtype=np.float64, order="F")


def make_network(loops, slip_systems, ranges, shift=None):
    """DislocationNetwork(loops; memBuffer=1) with dist = Zeros() and buffer = 0.

    Zeros() puts every loop's centre at the lower corner of `range`
    (DislocationUtil.jl:130-152).
    """
    coords, bvecs, links, labels = [], [], [], []
    base = 0
    for L in loops:
        sp = slip_systems["slipPlane"][L["slipSystemIdx"] - 1]
        bv = slip_systems["bVec"][L["slipSystemIdx"] - 1]
        c, b = make_loop(L["type"], L["numSides"], L["nodeSide"], L["segLen"], sp, bv)
        nl = len(c)
        for _ in range(L["numLoops"]):
            for q in range(nl):
                p = c[q]
                coords.append([p[k] + (ranges[k][0] + (ranges[k][1] - ranges[k][0]) * 0.0) for k in range(3)])
                bvecs.append(list(b))
                labels.append(L["label"][q])
                links.append((base + q + 1, base + (q + 1) % nl + 1))
            base += nl
    n = len(coords)
    coord = np.array(coords, dtype=np.float64).T
    if shift is not None:
        coord[:, shift["fromNode"] - 1:] += np.array(shift["by"], dtype=np.float64)[:, None]
    bvec = np.array(bvecs, dtype=np.float64).T
    seg_idx = np.zeros((n, 3), dtype=np.int64)
    ext = np.zeros(n, dtype=np.uint8)
    for i, (n1, n2) in enumerate(links):
        seg_idx[i] = (i + 1, n1, n2)
        ext[i] = 1 if (labels[n1 - 1] == EXT_DLN or labels[n2 - 1] == EXT_DLN) else 0
    return Network(coord, bvec, seg_idx, ext, n, label=np.array(labels))


def sigma_case_network(case):
    """The single-segment network of DislocationFEMTest.jl:5-155 and its 3×3 grid of points."""
    coord = np.array(case["coord"], dtype=np.float64).T
    nseg = len(case["links"])
    bvec = np.tile(np.array(case["b"], dtype=np.float64)[:, None], (1, nseg))
    seg_idx = np.array([[i + 1, l[0], l[1]] for i, l in enumerate(case["links"])], dtype=np.int64)
    net = Network(coord, bvec, seg_idx, np.zeros(nseg, np.uint8), nseg)
    r = [-300.0, 0.0, 300.0]
    pts = np.array([[x, y, 0.0] for x in r for y in r], dtype=np.float64).T  # x outer, y inner
    return net, np.asfortranarray(pts)


def make_connectivity(links, max_connect=4):
    """connectivity ((1 + 2 max_connect) × numNode, 1-based) as _makeConnect!
    builds it (DislocationUtil.jl:213-237): row 1 counts a node's links, rows
    2c and 2c+1 hold its c-th link and the node's column (1 or 2) in that link,
    links taken in order.  links: 2 × numLinks, 1-based node numbers."""
    links = np.asarray(links, dtype=np.int64)
    num_node = int(links.max())
    conn = np.zeros((1 + 2 * max_connect, num_node), dtype=np.int64, order="F")
    for i in range(links.shape[1]):
        n1, n2 = links[0, i] - 1, links[1, i] - 1
        conn[0, n1] += 1
        conn[0, n2] += 1
        t1, t2 = 2 * conn[0, n1], 2 * conn[0, n2]
        conn[t1 - 1:t1 + 1, n1] = (i + 1, 1)
        conn[t2 - 1:t2 + 1, n2] = (i + 1, 2)
    return conn


def cuboid_mesh(dx, dy, dz, mx, my, mz):
    """The geometry of buildMesh for a regular cuboid (FEMConstructor.jl:130-480):
    FE node coordinates (3 × (mx+1)(my+1)(mz+1), node i + (j-1)(mx+1) +
    (k-1)(mx+1)(my+1) at ((i-1)w, (j-1)h, (k-1)d)), the 8 vertices, face normals
    and face midpoints (3 × 6, faces xz@y0, yz@x1, xz@y1, yz@x0, xy@z0, xy@z1),
    and the closure point mean(vertices) summed in order."""
    w, h, d = dx / mx, dy / my, dz / mz
    mx1, my1, mz1 = mx + 1, my + 1, mz + 1
    coord = np.zeros((3, mx1 * my1 * mz1), order="F")
    for k in range(mz1):
        for j in range(my1):
            for i in range(mx1):
                g = i + j * mx1 + k * mx1 * my1
                coord[:, g] = (i * w, j * h, k * d)
    vtx = np.array([[0, 0, 0], [dx, 0, 0], [dx, dy, 0], [0, dy, 0], [0, 0, dz], [dx, 0, dz], [dx, dy, dz],
                    [0, dy, dz]], np.float64).T
    faces = np.array([[1, 2, 6, 5], [2, 3, 7, 6], [3, 4, 8, 7], [4, 1, 5, 8], [4, 3, 2, 1], [5, 6, 7, 8]]).T - 1
    mid = np.zeros((3, 6))
    for f in range(6):
        s = vtx[:, faces[0, f]].copy()
        for q in range(1, 4):
            s = s + vtx[:, faces[q, f]]
        mid[:, f] = s / 4
    norm = np.array([[0, -1, 0], [1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, 0, -1], [0, 0, 1]], np.float64).T
    c = vtx[:, 0].copy()
    for q in range(1, 8):
        c = c + vtx[:, q]
    return {"coord": coord, "vertices": vtx, "faceNorm": np.asfortranarray(norm), "faceMidPt": np.asfortranarray(mid),
            "C": c / 8, "lo": vtx.min(axis=1), "hi": vtx.max(axis=1)}


def cantilever_u_gamma(mx, my, mz):
    """Boundaries(::CantileverLoad) (FEMConstructor.jl:761-850, 968-987):
    uGammaDln = [uGamma nodes; mGamma nodes] from the mesh's surface node sets
    (FEMConstructor.jl:274-300, 495-545) and uDofsDln = [3u-2; 3u-1; 3u]."""
    mx1, my1, mz1 = mx + 1, my + 1, mz + 1
    mxm1, mym1, mzm1 = mx - 1, my - 1, mz - 1
    s = {
        "x0y0z0": [1], "x0y1z0": [mx1 * my + 1], "x0y0z1": [1 + mx1 * my1 * mz],
        "x0y1z1": [mx1 * my + 1 + mx1 * my1 * mz], "x1y0z1": [mx1 + mx1 * my1 * mz], "x1y1z1": [mx1 * my1 * mz1],
        "y_x0z0": [i * mx1 + 1 for i in range(1, mym1 + 1)],
        "y_x0z1": [i * mx1 + 1 + mx1 * my1 * mz for i in range(1, mym1 + 1)],
        "y_x1z1": [i * mx1 + mx1 + mx1 * my1 * mz for i in range(1, mym1 + 1)],
        "z_x0y0": [i * mx1 * my1 + 1 for i in range(1, mzm1 + 1)],
        "z_x0y1": [i * mx1 * my1 + 1 + mx1 * my for i in range(1, mzm1 + 1)],
        "yz_x0": [j * mx1 * my1 + 1 + i * mx1 for j in range(1, mzm1 + 1) for i in range(1, mym1 + 1)],
    }
    u = ["x0y0z0", "x0y1z0", "x0y0z1", "x0y1z1", "y_x0z0", "y_x0z1", "z_x0y0", "z_x0y1", "yz_x0"]
    m = ["x1y0z1", "x1y1z1", "y_x1z1"]
    nodes = np.array([n for k in u + m for n in s[k]], np.int64)
    dofs = np.concatenate([3 * nodes - 2, 3 * nodes - 1, 3 * nodes])
    return nodes, dofs
