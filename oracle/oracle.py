"""ctypes wrapper of the CPU oracle (liboracle.so built from ddd_oracle.cpp).

Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline load it, always as the checker, never as the thing measured or shipped.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int64)
_up = ctypes.POINTER(ctypes.c_uint8)
_llp = ctypes.POINTER(ctypes.c_longlong)


def build(force=False):
    """Compile liboracle.so with g++ (no -march flags: the same build runs on x86 and Arm)."""
    src = os.path.join(HERE, "ddd_oracle.cpp")
    hdr = os.path.join(HERE, "ddd_oracle.hpp")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB_PATH
    import subprocess
    tmp = LIB_PATH + ".tmp"
    cmd = ["g++", "-std=c++20", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_segseg_pair.argtypes = [_dp] * 8
        L.oracle_segseg_pair_f32.argtypes = [_dp] * 8
        L.oracle_segseg_pair_quad.argtypes = [_dp] * 7 + [ctypes.c_int, _dp]
        L.oracle_segseg_ser.argtypes = [_dp, _dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _dp]
        L.oracle_segseg_par_atomic.argtypes = [_dp, _dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _dp,
                                               ctypes.c_int]
        L.oracle_segseg_par_private.argtypes = [_dp, _dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _dp,
                                                ctypes.c_int]
        L.oracle_self_force.argtypes = [_dp, _dp, _dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _ip,
                                        ctypes.c_int64, _dp, _dp]
        L.oracle_pk_force.argtypes = [_dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _ip, ctypes.c_int64, _dp,
                                      _dp]
        L.oracle_mobility_bcc.argtypes = [_dp, _dp, _dp, _ip, _ip, ctypes.c_int64, _dp, ctypes.c_int64, _ip,
                                          ctypes.c_int64, _dp, _dp]
        L.oracle_minimum_distance.argtypes = [_dp, ctypes.c_int64, _dp]
        L.oracle_u_tilde.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int64, _dp, ctypes.c_int64, _dp, ctypes.c_double,
                                     _dp, ctypes.c_int64, _dp, ctypes.POINTER(ctypes.c_int32), _ip, _dp,
                                     ctypes.c_int64, ctypes.c_int64, _dp, ctypes.c_int]
        L.oracle_u_tilde.restype = ctypes.c_int64
        L.oracle_u_tilde_ld.argtypes = L.oracle_u_tilde.argtypes
        L.oracle_u_tilde_tris.argtypes = [_dp, _dp, _dp, ctypes.c_int64, _dp, ctypes.c_int64, _dp, ctypes.c_double,
                                          _dp, ctypes.POINTER(ctypes.c_int32), _ip, _dp, ctypes.c_int64,
                                          ctypes.c_int64, _dp, ctypes.c_int64]
        L.oracle_u_tilde_tris.restype = ctypes.c_int64
        L.oracle_u_tilde_ld.restype = ctypes.c_int64
        L.oracle_detect_collision.argtypes = [ctypes.c_double, _dp, _dp, ctypes.POINTER(ctypes.c_int32), _ip, _dp, _ip,
                                              ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _ip, ctypes.c_int64,
                                              _ip, _dp]
        L.oracle_segseg_rows.argtypes = [_dp, _dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _ip,
                                         ctypes.c_int64, _dp, ctypes.c_int]
        L.oracle_segseg_idx.argtypes = [_dp, _dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _ip,
                                        ctypes.c_int64, _dp, ctypes.c_int]
        L.oracle_sigma_tilde.argtypes = [_dp, _dp, ctypes.c_int64, _dp, _dp, _ip, ctypes.c_int64, ctypes.c_int64,
                                         _ip, ctypes.c_int64, _dp, ctypes.c_int]
        L.oracle_sigma_tilde_ld.argtypes = [_dp, _dp, ctypes.c_int64, _dp, _dp, _ip, ctypes.c_int64, ctypes.c_int64,
                                            _dp, ctypes.c_int]
        L.oracle_segseg_ser_ld.argtypes = [_dp, _dp, _dp, _ip, ctypes.c_int64, _up, ctypes.c_int64, _ip,
                                           ctypes.c_int64, _dp, ctypes.c_int]
        L.oracle_opcount_pair.argtypes = [_dp] * 7 + [_llp, _dp]
        L.oracle_opcount_sigma.argtypes = [_dp] * 5 + [_llp, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return np.require(a, np.float64, ["F", "A"])


def _net_arrays(net):
    coord = np.require(net.coord, np.float64, ["F"])
    bvec = np.require(net.bVec, np.float64, ["F"])
    seg = np.require(net.segIdx, np.int64, ["F"])
    ext = np.require(net.extSeg, np.uint8, ["C"])
    return coord, bvec, seg, ext, seg.shape[0]


def pair(k5, b1, n11, n12, b2, n21, n22, f32=False):
    """Fnode1..4 (4×3) of one pair."""
    args = [np.ascontiguousarray(v, np.float64) for v in (k5, b1, n11, n12, b2, n21, n22)]
    F = np.zeros(12)
    fn = lib().oracle_segseg_pair_f32 if f32 else lib().oracle_segseg_pair
    fn(*[_d(a) for a in args], _d(F))
    return F.reshape(4, 3)


def pair_quad(k5, b1, n11, n12, b2, n21, n22, nq):
    """Fnode1..4 (4×3) of one pair by nq-point Gauss quadrature of the σ̃ field
    (the checker of a planned far-field form; not a reference function)."""
    args = [np.ascontiguousarray(v, np.float64) for v in (k5, b1, n11, n12, b2, n21, n22)]
    F = np.zeros(12)
    lib().oracle_segseg_pair_quad(*[_d(a) for a in args], int(nq), _d(F))
    return F.reshape(4, 3)


def segseg_ser(k5, net):
    """calcSegSegForceSer! into a fresh 3×2×numSeg array (Fortran order)."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    F = np.zeros((3, 2, net.numSeg), np.float64, order="F")
    lib().oracle_segseg_ser(_d(np.ascontiguousarray(k5, np.float64)), _d(coord), _d(bvec), _i(seg), ld,
                            ext.ctypes.data_as(_up), net.numSeg, _d(F))
    return F


def segseg_ser_ld(k5, net, rows=None, nthreads=1):
    """All-pairs forces with every operation in long double (rounded to double at
    the end), for all segments or the given 0-based rows.  Its distance from the
    Float64 result is the rounding error of the reference's own arithmetic."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    if rows is not None:
        rows = np.ascontiguousarray(rows, np.int64)
    n = net.numSeg if rows is None else len(rows)
    F = np.zeros((3, 2, n), np.float64, order="F")
    lib().oracle_segseg_ser_ld(_d(np.ascontiguousarray(k5, np.float64)), _d(coord), _d(bvec), _i(seg), ld,
                               ext.ctypes.data_as(_up), net.numSeg, None if rows is None else _i(rows),
                               0 if rows is None else len(rows), _d(F), int(nthreads))
    return F


def segseg_par_atomic(k5, net, nthreads):
    coord, bvec, seg, ext, ld = _net_arrays(net)
    F = np.zeros((3, 2, net.numSeg), np.float64, order="F")
    lib().oracle_segseg_par_atomic(_d(np.ascontiguousarray(k5, np.float64)), _d(coord), _d(bvec), _i(seg), ld,
                                   ext.ctypes.data_as(_up), net.numSeg, _d(F), int(nthreads))
    return F


def segseg_par_private(k5, net, nthreads):
    """All-pairs forces with per-thread private accumulators (best-effort CPU form)."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    F = np.zeros((3, 2, net.numSeg), np.float64, order="F")
    lib().oracle_segseg_par_private(_d(np.ascontiguousarray(k5, np.float64)), _d(coord), _d(bvec), _i(seg), ld,
                                    ext.ctypes.data_as(_up), net.numSeg, _d(F), int(nthreads))
    return F


def self_force(k5, sc, net, idx=None):
    """calcSelfForce: (F1, F2), each 3 × n (n = numSeg or len(idx)); sc =
    (coreRad, coreEnergy, ν)."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    n = net.numSeg if idx is None else len(idx)
    F1 = np.zeros((3, n), np.float64, order="F")
    F2 = np.zeros((3, n), np.float64, order="F")
    ip = None if idx is None else _i(np.ascontiguousarray(idx, np.int64))
    lib().oracle_self_force(_d(np.ascontiguousarray(k5, np.float64)), _d(np.ascontiguousarray(sc, np.float64)),
                            _d(coord), _d(bvec), _i(seg), ld, ext.ctypes.data_as(_up), net.numSeg, ip,
                            0 if idx is None else len(idx), _d(F1), _d(F2))
    return F1, F2


def pk_force(net, sigma_hat, idx=None):
    """(σ̂ b) × (n2 - n1) per segment (3 × n) from sigma_hat (6 × n: xx, yy, zz, xy, xz, yz)."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    n = net.numSeg if idx is None else len(idx)
    PK = np.zeros((3, n), np.float64, order="F")
    sh = np.asfortranarray(sigma_hat, np.float64)
    ip = None if idx is None else _i(np.ascontiguousarray(idx, np.int64))
    lib().oracle_pk_force(_d(coord), _d(bvec), _i(seg), ld, ext.ctypes.data_as(_up), net.numSeg, ip,
                          0 if idx is None else len(idx), _d(sh), _d(PK))
    return PK


def mobility_bcc(mp, coord, bvec, links, conn, seg_force, num_node, idx=None):
    """dlnMobility (BCC): (nodeForce, nodeVel), 3 × n each.  mp = (σPN, edge,
    screw, climb, line drag); links 2 × nLinks and conn ((1+2 maxConnect) ×
    nodes) 1-based; seg_force 3 × 2 × nLinks."""
    coord = np.require(coord, np.float64, ["F"])
    bvec = np.require(bvec, np.float64, ["F"])
    links = np.require(links, np.int64, ["F"])
    conn = np.require(conn, np.int64, ["F"])
    sf = np.require(seg_force, np.float64, ["F"])
    n = num_node if idx is None else len(idx)
    Fo = np.zeros((3, n), np.float64, order="F")
    Vo = np.zeros((3, n), np.float64, order="F")
    ip = None if idx is None else _i(np.ascontiguousarray(idx, np.int64))
    lib().oracle_mobility_bcc(_d(np.ascontiguousarray(mp, np.float64)), _d(coord), _d(bvec), _i(links), _i(conn),
                              conn.shape[0], _d(sf), num_node, ip, 0 if idx is None else len(idx), _d(Fo), _d(Vo))
    return Fo, Vo


def minimum_distance(x0, x1, y0, y1, vx0, vx1, vy0, vy1):
    """minimumDistance for n pairs: each argument 3 × n (or a 3-vector for one
    pair); returns (distSq, dDistSqDt, L1, L2), arrays of n."""
    arrs = [np.asarray(a, np.float64).reshape(3, -1, order="F") for a in (x0, x1, y0, y1, vx0, vx1, vy0, vy1)]
    n = arrs[0].shape[1]
    pts = np.asfortranarray(np.stack(arrs, axis=1))  # 3 x 8 x n
    out = np.zeros((4, n), np.float64, order="F")
    lib().oracle_minimum_distance(_d(pts), n, _d(out))
    return out[0], out[1], out[2], out[3]


def u_tilde(k2, mesh, normals, points, coord, label, links, bvec, num_node, num_seg, tol=None, nthreads=1,
            long_double=False):
    """calc_uTilde's displacements (3 × M) at points (3 × M); mesh: the dict of
    fixtures.cuboid_mesh (faceNorm, faceMidPt, C, lo, hi); normals 3 × K.
    long_double: the same triangles summed in long double (the reference
    arithmetic's error is the difference).  Returns (u, number of triangles)."""
    pts = np.require(points, np.float64, ["F"])
    M = pts.shape[1]
    u = np.zeros((3, M), np.float64, order="F")
    fn = np.require(mesh["faceNorm"], np.float64, ["F"])
    fm = np.require(mesh["faceMidPt"], np.float64, ["F"])
    nr = np.require(normals, np.float64, ["F"])
    box = np.ascontiguousarray(np.r_[mesh["lo"], mesh["hi"]], np.float64)
    if tol is None:
        tol = 1e-10 * float(np.max(mesh["hi"] - mesh["lo"]))
    lab = np.ascontiguousarray(label, np.int32)
    fn_ = lib().oracle_u_tilde_ld if long_double else lib().oracle_u_tilde
    nt = fn_(_d(np.ascontiguousarray(k2, np.float64)), _d(np.ascontiguousarray(mesh["C"], np.float64)),
             _d(fn), _d(fm), fn.shape[1], _d(nr), nr.shape[1], _d(box), float(tol), _d(pts), M,
             _d(np.require(coord, np.float64, ["F"])), lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
             _i(np.require(links, np.int64, ["F"])), _d(np.require(bvec, np.float64, ["F"])), int(num_node),
             int(num_seg), _d(u), int(nthreads))
    return u, int(nt)


def u_tilde_tris(mesh, normals, coord, label, links, bvec, num_node, num_seg, tol=None):
    """calc_uTilde's triangles in the reference's order: (T × 13: A, B, C, b, full)."""
    fn = np.require(mesh["faceNorm"], np.float64, ["F"])
    fm = np.require(mesh["faceMidPt"], np.float64, ["F"])
    nr = np.require(normals, np.float64, ["F"])
    box = np.ascontiguousarray(np.r_[mesh["lo"], mesh["hi"]], np.float64)
    if tol is None:
        tol = 1e-10 * float(np.max(mesh["hi"] - mesh["lo"]))
    lab = np.ascontiguousarray(label, np.int32)
    args = [_d(np.ascontiguousarray(mesh["C"], np.float64)), _d(fn), _d(fm), fn.shape[1], _d(nr), nr.shape[1],
            _d(box), float(tol), _d(np.require(coord, np.float64, ["F"])),
            lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _i(np.require(links, np.int64, ["F"])),
            _d(np.require(bvec, np.float64, ["F"])), int(num_node), int(num_seg)]
    n = lib().oracle_u_tilde_tris(*args, None, 0)
    out = np.zeros((n, 13))
    lib().oracle_u_tilde_tris(*args, _d(out), n)
    return out


_COLLISION_TYPES = ("null", "hinge", "twoLine")


def detect_collision(collision_dist_sq, coord, node_vel, label, links, bvec, conn, num_node, num_seg, skip_segs=()):
    """detectCollision: (collision, type, n1s1, n2s1, n1s2, n2s2, s1, s2, L1, L2)
    as the reference returns it (type "null" / "hinge" / "twoLine"), and a dict
    with the reported pair's own distSq, L1, L2."""
    coord = np.require(coord, np.float64, ["F"])
    node_vel = np.require(node_vel, np.float64, ["F"])
    label = np.ascontiguousarray(label, np.int32)
    links = np.require(links, np.int64, ["F"])
    bvec = np.require(bvec, np.float64, ["F"])
    conn = np.require(conn, np.int64, ["F"])
    skip = np.ascontiguousarray(np.asarray(list(skip_segs), np.int64).reshape(-1, 2))
    iout = np.zeros(8, np.int64)
    dout = np.zeros(5, np.float64)
    lib().oracle_detect_collision(float(collision_dist_sq), _d(coord), _d(node_vel),
                                  label.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _i(links), _d(bvec), _i(conn),
                                  conn.shape[0], int(num_node), int(num_seg), _i(skip), len(skip), _i(iout), _d(dout))
    res = (bool(iout[0]), _COLLISION_TYPES[iout[1]], *(int(v) for v in iout[2:]), float(dout[0]), float(dout[1]))
    return res, {"distSq": float(dout[2]), "L1": float(dout[3]), "L2": float(dout[4])}


def segseg_rows(k5, net, rows, nthreads=1):
    """All-pairs result restricted to the given 0-based segment rows (3×2×len(rows))."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    rows = np.ascontiguousarray(rows, np.int64)
    F = np.zeros((3, 2, len(rows)), np.float64, order="F")
    lib().oracle_segseg_rows(_d(np.ascontiguousarray(k5, np.float64)), _d(coord), _d(bvec), _i(seg), ld,
                             ext.ctypes.data_as(_up), net.numSeg, _i(rows), len(rows), _d(F), int(nthreads))
    return F


def segseg_idx(k5, net, idx, nthreads=1):
    """Index-list form (idx 1-based) into a fresh 3×2×len(idx) array."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    idx = np.ascontiguousarray(idx, np.int64)
    F = np.zeros((3, 2, len(idx)), np.float64, order="F")
    lib().oracle_segseg_idx(_d(np.ascontiguousarray(k5, np.float64)), _d(coord), _d(bvec), _i(seg), ld,
                            ext.ctypes.data_as(_up), net.numSeg, _i(idx), len(idx), _d(F), int(nthreads))
    return F


def sigma_tilde(k5, x0, net, idx=None, nthreads=1):
    """σ̃ (6×M, Fortran order) at the points x0 (3×M)."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    x0 = np.require(x0, np.float64, ["F"])
    M = x0.shape[1]
    sig = np.zeros((6, M), np.float64, order="F")
    if idx is None:
        ip, n = None, 0
    else:
        idx = np.ascontiguousarray(idx, np.int64)
        ip, n = _i(idx), len(idx)
    lib().oracle_sigma_tilde(_d(np.ascontiguousarray(k5, np.float64)), _d(x0), M, _d(coord), _d(bvec), _i(seg), ld,
                             net.numSeg, ip, n, _d(sig), int(nthreads))
    return sig


def sigma_tilde_ld(k5, x0, net, nthreads=1):
    """σ̃ (6×M) with every operation in long double, rounded to double at the
    end; its distance from sigma_tilde is the Float64 algorithm's own error."""
    coord, bvec, seg, ext, ld = _net_arrays(net)
    x0 = np.require(x0, np.float64, ["F"])
    M = x0.shape[1]
    sig = np.zeros((6, M), np.float64, order="F")
    lib().oracle_sigma_tilde_ld(_d(np.ascontiguousarray(k5, np.float64)), _d(x0), M, _d(coord), _d(bvec), _i(seg), ld,
                                net.numSeg, _d(sig), int(nthreads))
    return sig


OPCOUNT_FIELDS = ("add", "mul", "div", "sqrt", "log", "atan", "cmp")


def opcount_pair(k5, b1, n11, n12, b2, n21, n22):
    args = [np.ascontiguousarray(v, np.float64) for v in (k5, b1, n11, n12, b2, n21, n22)]
    c = np.zeros(7, np.int64)
    F = np.zeros(12)
    lib().oracle_opcount_pair(*[_d(a) for a in args], c.ctypes.data_as(_llp), _d(F))
    return dict(zip(OPCOUNT_FIELDS, (int(v) for v in c)))


def opcount_sigma(k5, b, n1, n2, x):
    args = [np.ascontiguousarray(v, np.float64) for v in (k5, b, n1, n2, x)]
    c = np.zeros(7, np.int64)
    s = np.zeros(6)
    lib().oracle_opcount_sigma(*[_d(a) for a in args], c.ctypes.data_as(_llp), _d(s))
    return dict(zip(OPCOUNT_FIELDS, (int(v) for v in c)))
