"""ddd_gb300 — host-side mirror of DDD.jl's seg-seg force / σ̃ interface over
the C-ABI library libddd_gb300.so (include/ddd_gb300.h).

The reference is Julia; its drop-in is a `ccall` shim (julia/DDDGB300.jl).
This module is the same binding written with ctypes so the path can be driven
and tested from Python: the functions keep the reference's names, argument
order, array layouts and semantics:

  calcSegSegForce(dlnParams, matParams, network, idx=None)        DislocationForces.jl:470-561
  calcSegSegForce_inplace(dlnParams, matParams, network, idx=None) calcSegSegForce!  :576-669
  calc_σTilde(x0, dlnParams, matParams, network, idx=None)        DislocationFEM.jl:24-41
  calc_σTilde_inplace(σ, x0, dlnParams, matParams, network, idx=None) calc_σTilde! :67-84
  calcSelfForce(dlnParams, matParams, network, idx=None)          DislocationForces.jl:320-353 (and _inplace)
  calcSegForce(dlnParams, matParams, sigmaHat, network, idx=None) DislocationForces.jl:23-46 (and _inplace;
      sigmaHat = the FE stress at the segment midpoints, in place of mesh and forceDisplacement)
  dlnMobility(dlnParams, matParams, network, idx=None)            DislocationMobility.jl:16-178, BCC (and _inplace)

All computation runs on the GPU.  There is no CPU fallback: if the library is
not built or no GPU is usable, calls raise.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libddd_gb300.so")

DDD_OK, DDD_EINVAL, DDD_ERANGE, DDD_ENONFINITE, DDD_EDEVICE, DDD_ENOMEM, DDD_ETOOBIG = 0, -1, -2, -3, -4, -5, -6
DDD_ETIMEOUT = -7
# Largest network ddd_segseg_force_device_noalloc accepts (include/ddd_gb300.h).
NOALLOC_MAX_SEGMENTS = 4096

# Every symbol include/ddd_gb300.h declares.
EXPORTED_SYMBOLS = (
    "ddd_create", "ddd_destroy", "ddd_last_error", "ddd_last_kernel_ms", "ddd_version",
    "ddd_detect_collision", "ddd_minimum_distance", "ddd_u_tilde",
    "ddd_segseg_force", "ddd_segseg_force_inplace", "ddd_sigma_tilde",
    "ddd_segseg_force_device", "ddd_sigma_tilde_device", "ddd_set_mode", "ddd_get_mode", "ddd_probe_fma_peak",
    "ddd_selftest_bounded_wait",
    "ddd_set_partial_limit", "ddd_get_partial_limit",
    "ddd_segseg_force_device_noalloc",
    "ddd_batch_create", "ddd_batch_run", "ddd_batch_info", "ddd_batch_last_error", "ddd_batch_destroy",
    "ddd_tc_gemm_bf16",
    "ddd_surrogate_create", "ddd_surrogate_destroy", "ddd_surrogate_num_params", "ddd_surrogate_params",
    "ddd_surrogate_make_data", "ddd_surrogate_train", "ddd_surrogate_forward", "ddd_surrogate_grads",
    "ddd_surrogate_force", "ddd_surrogate_force_host", "ddd_surrogate_last_error", "ddd_surrogate_save",
    "ddd_surrogate_load",
    "ddd_self_force", "ddd_self_force_inplace", "ddd_seg_force", "ddd_seg_force_inplace",
    "ddd_mobility_bcc", "ddd_mobility_bcc_inplace",
)

# Arithmetic modes (ddd_set_mode).
MODE_FP64, MODE_FP64_FMA, MODE_DF64, MODE_F32C, MODE_FP64_FAST = 0, 1, 2, 3, 4
MODES = {"fp64": MODE_FP64, "fp64_fma": MODE_FP64_FMA, "df64": MODE_DF64, "f32c": MODE_F32C,
         "fp64_fast": MODE_FP64_FAST}


class DDDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class ddd_consts(ctypes.Structure):
    _fields_ = [("aSq", ctypes.c_double), ("mu4pi", ctypes.c_double), ("mu8pi", ctypes.c_double),
                ("mu4pinu", ctypes.c_double), ("nuMu4pinu", ctypes.c_double)]


class ddd_batch_info_t(ctypes.Structure):
    _fields_ = [("tile", ctypes.c_int), ("order", ctypes.c_int), ("work_items", ctypes.c_int64),
                ("total_segments", ctypes.c_int64), ("graph_launches", ctypes.c_int64),
                ("tune_ms", ctypes.c_double * 4)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "tune_ms"}
        d["tune_ms"] = list(self.tune_ms)
        return d


class ddd_report(ctypes.Structure):
    _fields_ = [("pairs_general", ctypes.c_int64), ("pairs_parallel", ctypes.c_int64),
                ("core_sides", ctypes.c_int64), ("kernel_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ddd_self_params(ctypes.Structure):
    _fields_ = [("coreRad", ctypes.c_double), ("coreEnergy", ctypes.c_double), ("nu", ctypes.c_double)]


class ddd_mob_params(ctypes.Structure):
    _fields_ = [("sigmaPN", ctypes.c_double), ("edgeDrag", ctypes.c_double), ("screwDrag", ctypes.c_double),
                ("climbDrag", ctypes.c_double), ("lineDrag", ctypes.c_double)]


class ddd_collision(ctypes.Structure):
    _fields_ = [("collision", ctypes.c_int32), ("type", ctypes.c_int32), ("n1s1", ctypes.c_int64),
                ("n2s1", ctypes.c_int64), ("n1s2", ctypes.c_int64), ("n2s2", ctypes.c_int64), ("s1", ctypes.c_int64),
                ("s2", ctypes.c_int64), ("L1", ctypes.c_double), ("L2", ctypes.c_double),
                ("pairDistSq", ctypes.c_double), ("pairL1", ctypes.c_double), ("pairL2", ctypes.c_double)]


class ddd_u_mesh(ctypes.Structure):
    _fields_ = [("C", ctypes.c_double * 3), ("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3),
                ("tol", ctypes.c_double), ("faceNorm", ctypes.POINTER(ctypes.c_double)),
                ("faceMidPt", ctypes.POINTER(ctypes.c_double)), ("numFaces", ctypes.c_int64),
                ("normals", ctypes.POINTER(ctypes.c_double)), ("numNormals", ctypes.c_int64)]


class ddd_sur_opts(ctypes.Structure):
    _fields_ = [("kappa", ctypes.c_double), ("audit_fraction", ctypes.c_double), ("audit_tol", ctypes.c_double),
                ("exact_mode", ctypes.c_int), ("far_mode", ctypes.c_int), ("kappa_two", ctypes.c_double)]


# Far-pair passes of ddd_surrogate_force (ddd_sur_opts.far_mode).
FAR_MODES = {"network": 0, "quad2": 2, "quad3": 3}
# Default trust factor of the quadrature far field: the 3-point rule (far_mode
# 3) stays at its FP32 noise level (~2e-7 per pair) down to R = 8 max(L_i, L_j),
# so the near pass can stop at 10 lengths; the 2-point rule (far_mode 2) needs
# 20 (4e-6 per pair there, 3e-5 at 10).  The network's factor is its training
# range (the checkpoint's kappa).
QUAD_KAPPA = 10.0
QUAD2_KAPPA = 20.0
# The 3-point far pass switches a warp's step of 32 pairs to the 2-point rule
# when each of its far pairs lies beyond this many lengths: the 2-point rule's
# truncation (~5e-6 per pair at 20 lengths, falling as (L/R)^4) is then small
# enough that the node-force errors measure as with 3 points everywhere.
QUAD_KAPPA_TWO = 30.0


class ddd_sur_report(ctypes.Structure):
    _fields_ = [("pairs_total", ctypes.c_int64), ("pairs_near_general", ctypes.c_int64),
                ("pairs_near_parallel", ctypes.c_int64), ("tiles_total", ctypes.c_int64),
                ("tiles_near", ctypes.c_int64), ("tiles_audit", ctypes.c_int64),
                ("audit_rel_rms", ctypes.c_double), ("audit_rel_max", ctypes.c_double),
                ("audit_node_rel_rms", ctypes.c_double), ("fallback", ctypes.c_int),
                ("ms_prep", ctypes.c_double), ("ms_network", ctypes.c_double), ("ms_audit", ctypes.c_double),
                ("ms_near", ctypes.c_double), ("ms_reduce", ctypes.c_double), ("ms_total", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int64)
_up = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64


def build(verbose=False):
    """Compile libddd_gb300.so for sm_103a (nvcc; works without a GPU)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_ddd_gb300_build", os.path.join(HERE, "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build(verbose=verbose)


def library():
    """The loaded C-ABI library (ctypes.CDLL).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libddd_gb300.so is not built (run __graft_entry__.build() or build()); "
                               "there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        cp = ctypes.POINTER(ddd_consts)
        rp = ctypes.POINTER(ddd_report)
        L.ddd_create.argtypes = [ctypes.c_int]
        L.ddd_create.restype = _vp
        L.ddd_destroy.argtypes = [_vp]
        L.ddd_destroy.restype = None
        L.ddd_last_error.argtypes = [_vp]
        L.ddd_last_error.restype = ctypes.c_char_p
        L.ddd_last_kernel_ms.restype = ctypes.c_double
        L.ddd_last_kernel_ms.argtypes = [ctypes.c_void_p]
        L.ddd_version.argtypes = []
        L.ddd_segseg_force.argtypes = [_vp, cp, _dp, _i64, _dp, _i64, _ip, _i64, _up, _i64, _ip, _i64, _dp, rp]
        L.ddd_segseg_force_inplace.argtypes = [_vp, cp, _dp, _i64, _dp, _i64, _ip, _i64, _up, _i64, _ip, _i64, _dp,
                                               _i64, rp]
        L.ddd_sigma_tilde.argtypes = [_vp, cp, _dp, _i64, _dp, _i64, _dp, _i64, _ip, _i64, _i64, _ip, _i64, _dp, rp]
        L.ddd_segseg_force_device.argtypes = [_vp, cp, _vp, _i64, _vp, _i64, _vp, _vp, rp]
        L.ddd_sigma_tilde_device.argtypes = [_vp, cp, _vp, _i64, _vp, _i64, _i64, _vp, _vp, rp]
        L.ddd_segseg_force_device_noalloc.argtypes = [cp, _vp, _i64, _vp, _i64, _vp, _vp]
        L.ddd_batch_create.argtypes = [_vp, _i64, _ip, ctypes.c_int, ctypes.c_int]
        L.ddd_batch_create.restype = _vp
        L.ddd_batch_run.argtypes = [_vp, cp, _vp, _vp, _vp, _vp]
        L.ddd_batch_info.argtypes = [_vp, ctypes.POINTER(ddd_batch_info_t)]
        L.ddd_batch_last_error.argtypes = [_vp]
        L.ddd_batch_last_error.restype = ctypes.c_char_p
        L.ddd_batch_destroy.argtypes = [_vp]
        L.ddd_batch_destroy.restype = None
        L.ddd_tc_gemm_bf16.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp]
        L.ddd_surrogate_create.argtypes = [_vp, ctypes.c_uint64]
        L.ddd_surrogate_create.restype = _vp
        L.ddd_surrogate_destroy.argtypes = [_vp]
        L.ddd_surrogate_destroy.restype = None
        L.ddd_surrogate_num_params.argtypes = []
        L.ddd_surrogate_params.argtypes = [_vp, ctypes.POINTER(ctypes.c_float), ctypes.c_int]
        L.ddd_surrogate_make_data.argtypes = [_vp, cp, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp]
        L.ddd_surrogate_train.argtypes = [_vp, _vp, _vp, _vp, _i64, _i64, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_float, _dp]
        L.ddd_surrogate_forward.argtypes = [_vp, _vp, _vp, _i64, _vp]
        L.ddd_surrogate_grads.argtypes = [_vp, _vp, _vp, _vp, _i64, _dp, ctypes.POINTER(ctypes.c_float)]
        L.ddd_surrogate_force.argtypes = [_vp, cp, _vp, _i64, _vp, _i64, _vp, _vp, ctypes.POINTER(ddd_sur_opts),
                                          ctypes.POINTER(ddd_sur_report)]
        L.ddd_surrogate_force_host.argtypes = [_vp, cp, _dp, _i64, _dp, _i64, _ip, _i64, _up, _i64, _dp,
                                               ctypes.POINTER(ddd_sur_opts), ctypes.POINTER(ddd_sur_report)]
        L.ddd_surrogate_save.argtypes = [_vp, ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.ddd_surrogate_load.argtypes = [_vp, ctypes.c_char_p, _dp, _dp, _dp]
        L.ddd_surrogate_last_error.argtypes = [_vp]
        L.ddd_surrogate_last_error.restype = ctypes.c_char_p
        spp = ctypes.POINTER(ddd_self_params)
        net_args = [_dp, _i64, _dp, _i64, _ip, _i64, _up, _i64]
        L.ddd_self_force.argtypes = [_vp, cp, spp] + net_args + [_ip, _i64, _dp, _dp]
        L.ddd_self_force_inplace.argtypes = [_vp, cp, spp] + net_args + [_ip, _i64, _dp, _i64]
        L.ddd_seg_force.argtypes = [_vp, cp, spp] + net_args + [_dp, _ip, _i64, _dp, rp]
        L.ddd_seg_force_inplace.argtypes = [_vp, cp, spp] + net_args + [_dp, _ip, _i64, _dp, _i64, rp]
        mob_args = [_vp, ctypes.POINTER(ddd_mob_params), _dp, _i64, _dp, _i64, _ip, _i64, _ip, _i64, _i64, _dp,
                    _i64, _i64, _ip, _i64, _dp, _dp]
        L.ddd_mobility_bcc.argtypes = mob_args
        L.ddd_mobility_bcc_inplace.argtypes = mob_args + [_i64]
        L.ddd_detect_collision.argtypes = [_vp, ctypes.c_double, _dp, _i64, _dp, _i64, ctypes.POINTER(ctypes.c_int32),
                                           _i64, _ip, _i64, _dp, _i64, _ip, _i64, _i64, _i64, _i64, _ip, _i64,
                                           ctypes.POINTER(ddd_collision)]
        L.ddd_minimum_distance.argtypes = [_vp, _dp, _i64, _dp]
        L.ddd_u_tilde.argtypes = [_vp, ctypes.c_double, ctypes.c_double, ctypes.POINTER(ddd_u_mesh), _dp, _i64, _dp,
                                  _i64, ctypes.POINTER(ctypes.c_int32), _i64, _ip, _i64, _dp, _i64, _i64, _i64, _ip,
                                  _dp, _i64]
        L.ddd_set_mode.argtypes = [_vp, ctypes.c_int]
        L.ddd_get_mode.argtypes = [_vp]
        L.ddd_set_partial_limit.argtypes = [_vp, ctypes.c_int64]
        L.ddd_get_partial_limit.argtypes = [_vp]
        L.ddd_get_partial_limit.restype = ctypes.c_int64
        L.ddd_probe_fma_peak.argtypes = [_vp, ctypes.c_int, _dp]
        L.ddd_selftest_bounded_wait.argtypes = [_vp, ctypes.c_longlong, ctypes.c_int]
        _lib = L
    return _lib


# ---------------------------------------------------------------------------
# Parameter and network types (fields as in src/Type/*.jl).

class MaterialParameters:
    """MaterialParameters (src/Type/MaterialConstructor.jl:42-101): derived constants from μ and ν."""

    def __init__(self, *, crystalStruct="BCC", mu=1.0, muMag=1.0, nu=0.2, sigmaPN=0.0):
        self.crystalStruct = crystalStruct
        self.μ = self.mu = float(mu)
        self.μMag = float(muMag)
        self.ν = self.nu = float(nu)
        self.omνInv = 1.0 / (1.0 - self.nu)
        self.opνInv = 1.0 / (1.0 + self.nu)
        self.νomνInv = self.nu * self.omνInv
        self.νopνInv = self.nu * self.opνInv
        self.μ4π = self.mu / (4.0 * math.pi)
        self.μ8π = self.μ4π / 2.0
        self.μ4πν = self.μ4π * self.omνInv
        self.νμ4πν = self.nu * self.μ4πν
        self.omνInv8π = self.omνInv / (8.0 * math.pi)
        self.om2νomνInv8π = (1.0 - 2.0 * self.nu) * self.omνInv8π
        self.σPN = float(sigmaPN)


class DislocationParameters:
    """The DislocationParameters fields this path reads (src/Type/DislocationConstructor.jl:55-105).

    Like the reference's constructor (:75-78) it asserts coreRad < minSegLen <
    maxSegLen unless all three are 0, and minArea < maxArea unless both are 0
    (AssertionError, as Julia's @assert raises)."""

    def __init__(self, *, coreRad=1.0, coreRadMag=1.0, coreEnergy=None, minSegLen=None, maxSegLen=None,
                 minArea=None, maxArea=None, collisionDist=None, parCPU=False, parGPU=True, dragCoeffs=None,
                 **other):
        self.dragCoeffs = dict(edge=1.0, screw=2.0, climb=1e9, line=0.0)
        if dragCoeffs:
            self.dragCoeffs.update({k: float(v) for k, v in dict(dragCoeffs).items()})
        self.coreRad = float(coreRad)
        self.coreRadSq = self.coreRad * self.coreRad
        # Julia's log(0.0) is -Inf where Python's math.log raises.
        self.coreEnergy = ((1 / (4 * math.pi) * math.log(self.coreRad / 0.1) if self.coreRad > 0 else -math.inf)
                           if coreEnergy is None else float(coreEnergy))
        self.coreRadMag = float(coreRadMag)
        self.minSegLen = 2 * self.coreRad if minSegLen is None else float(minSegLen)
        self.maxSegLen = 20 * self.coreRad if maxSegLen is None else float(maxSegLen)
        self.minArea = self.minSegLen ** 2 / math.sqrt(2) if minArea is None else float(minArea)
        self.maxArea = 100 * self.minArea if maxArea is None else float(maxArea)
        if not (self.coreRad == self.minSegLen == self.maxSegLen == 0):
            assert self.coreRad < self.minSegLen < self.maxSegLen, \
                "coreRad < minSegLen < maxSegLen does not hold (%g, %g, %g)" % (self.coreRad, self.minSegLen,
                                                                                 self.maxSegLen)
        if not (self.minArea == self.maxArea == 0):
            assert self.minArea < self.maxArea, "minArea < maxArea does not hold (%g, %g)" % (self.minArea,
                                                                                            self.maxArea)
        self.collisionDist = self.minSegLen / 2 if collisionDist is None else float(collisionDist)
        self.collisionDistSq = self.collisionDist * self.collisionDist
        self.parCPU = bool(parCPU)
        self.parGPU = bool(parGPU)
        for k, v in other.items():
            setattr(self, k, v)


class DislocationNetwork:
    """The DislocationNetwork arrays this path reads and writes (src/Type/DislocationType.jl:324-340).

    coord (3×nodeBuf), bVec (3×linkBuf), segIdx (linkBuf×3; link, node1, node2;
    1-based), extSeg (linkBuf), segForce (3×2×linkBuf), numSeg; for the
    mobility also links (2×linkBuf), connectivity ((1+2 maxConnect)×nodeBuf),
    numNode, nodeForce and nodeVel (3×nodeBuf); for collision detection also
    label (nodeBuf int32, the nodeTypeDln values; default 1 = intMobDln);
    slipPlane and linksConnect are carried for the JSON files.
    links defaults to segIdx's node columns and connectivity to the one
    _makeConnect! builds from it.
    Stored Fortran-ordered, which is the Julia memory image.
    """

    def __init__(self, coord, bVec, segIdx, numSeg=None, extSeg=None, segForce=None, links=None,
                 connectivity=None, numNode=None, nodeForce=None, nodeVel=None, maxConnect=4, label=None,
                 slipPlane=None, linksConnect=None):
        self.coord = np.asfortranarray(coord, dtype=np.float64)
        self.bVec = np.asfortranarray(bVec, dtype=np.float64)
        self.segIdx = np.asfortranarray(segIdx, dtype=np.int64)
        ld = self.segIdx.shape[0]
        self.numSeg = int(ld if numSeg is None else numSeg)
        self.extSeg = (np.zeros(ld, np.uint8) if extSeg is None else np.ascontiguousarray(extSeg, dtype=np.uint8))
        self.segForce = (np.zeros((3, 2, self.bVec.shape[1]), np.float64, order="F") if segForce is None
                         else np.asfortranarray(segForce, dtype=np.float64))
        self.maxConnect = int(maxConnect)
        self.links = (np.asfortranarray(self.segIdx[:self.numSeg, 1:3].T) if links is None
                      else np.asfortranarray(links, dtype=np.int64))
        nodes = self.coord.shape[1]
        self.connectivity = (make_connectivity(self.links, nodes, self.maxConnect) if connectivity is None
                             else np.asfortranarray(connectivity, dtype=np.int64))
        self.numNode = int(nodes if numNode is None else numNode)
        self.nodeForce = (np.zeros((3, nodes), np.float64, order="F") if nodeForce is None
                          else np.asfortranarray(nodeForce, dtype=np.float64))
        self.nodeVel = (np.zeros((3, nodes), np.float64, order="F") if nodeVel is None
                        else np.asfortranarray(nodeVel, dtype=np.float64))
        self.label = (np.ones(nodes, np.int32) if label is None
                      else np.ascontiguousarray(np.asarray(label).astype(np.int32)))
        nl = self.bVec.shape[1]
        self.slipPlane = (np.zeros((3, nl), np.float64, order="F") if slipPlane is None
                          else np.asfortranarray(slipPlane, dtype=np.float64))
        self.linksConnect = (np.zeros((2, nl), np.int64, order="F") if linksConnect is None
                             else np.asfortranarray(linksConnect, dtype=np.int64))


def make_connectivity(links, num_node, max_connect=4):
    """connectivity ((1 + 2 max_connect) × num_node, 1-based) in the layout of
    _makeConnect! (DislocationUtil.jl:213-237): row 1 counts a node's links,
    rows 2c, 2c+1 hold its c-th link and the node's column in it; links are
    taken in order up to the first undefined (zero) one."""
    links = np.asarray(links, dtype=np.int64)
    conn = np.zeros((1 + 2 * max_connect, num_node), dtype=np.int64, order="F")
    for i in range(links.shape[1]):
        n1, n2 = int(links[0, i]), int(links[1, i])
        if n1 == 0:
            break
        for node, col in ((n1, 1), (n2, 2)):
            conn[0, node - 1] += 1
            c = conn[0, node - 1]
            if 2 * c + 1 > conn.shape[0]:
                raise ValueError("node %d has more than maxConnect = %d links" % (node, max_connect))
            conn[2 * c - 1, node - 1] = i + 1
            conn[2 * c, node - 1] = col
    return conn


def self_params_of(dlnParams, matParams):
    sp = ddd_self_params()
    sp.coreRad = dlnParams.coreRad
    sp.coreEnergy = dlnParams.coreEnergy
    sp.nu = matParams.ν
    return sp


def consts_of(dlnParams, matParams):
    k = ddd_consts()
    k.aSq = dlnParams.coreRadSq
    k.mu4pi = matParams.μ4π
    k.mu8pi = matParams.μ8π
    k.mu4pinu = matParams.μ4πν
    k.nuMu4pinu = matParams.νμ4πν
    return k


# ---------------------------------------------------------------------------
# Context.

class Context:
    """Owns one ddd_ctx (device buffers, stream) on one CUDA device."""

    def __init__(self, device=0):
        L = library()
        self._L = L
        self._h = L.ddd_create(int(device))
        if not self._h:
            raise DDDError(DDD_EDEVICE, "ddd_create(%d) failed: %s" % (device, L.ddd_last_error(None).decode()))
        self.device = device
        self.last_report = None

    def close(self):
        if self._h:
            self._L.ddd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != DDD_OK:
            msg = self._L.ddd_last_error(self._h).decode()
            if rc == DDD_ERANGE:
                raise IndexError(msg)
            if rc in (DDD_EINVAL, DDD_ENONFINITE):
                raise ValueError(msg)
            raise DDDError(rc, msg)

    @staticmethod
    def _net(network):
        coord = np.require(network.coord, np.float64, ["F"])
        bvec = np.require(network.bVec, np.float64, ["F"])
        seg = np.require(network.segIdx, np.int64, ["F"])
        ext = np.require(network.extSeg, np.uint8, ["C"])
        if coord.ndim != 2 or coord.shape[0] != 3 or bvec.ndim != 2 or bvec.shape[0] != 3:
            raise ValueError("coord and bVec must be 3×n")
        if seg.ndim != 2 or seg.shape[1] != 3:
            raise ValueError("segIdx must be n×3")
        if ext.shape[0] < network.numSeg:
            raise ValueError("extSeg shorter than numSeg")
        return coord, bvec, seg, ext

    @staticmethod
    def _idx(idx):
        if idx is None:
            return None
        return np.ascontiguousarray(np.atleast_1d(np.asarray(idx)), dtype=np.int64)

    def segseg_force(self, k, network, idx=None, out=None):
        coord, bvec, seg, ext = self._net(network)
        idx = self._idx(idx)
        n = network.numSeg if idx is None else len(idx)
        if out is None:
            out = np.zeros((3, 2, n), np.float64, order="F")
        rep = ddd_report()
        rc = self._L.ddd_segseg_force(
            self._h, ctypes.byref(k), coord.ctypes.data_as(_dp), coord.shape[1], bvec.ctypes.data_as(_dp),
            bvec.shape[1], seg.ctypes.data_as(_ip), seg.shape[0], ext.ctypes.data_as(_up), network.numSeg,
            None if idx is None else idx.ctypes.data_as(_ip), 0 if idx is None else len(idx),
            out.ctypes.data_as(_dp), ctypes.byref(rep))
        self._check(rc)
        self.last_report = rep.as_dict()
        return out

    def _netp(self, network):
        coord, bvec, seg, ext = self._net(network)
        return [coord.ctypes.data_as(_dp), coord.shape[1], bvec.ctypes.data_as(_dp), bvec.shape[1],
                seg.ctypes.data_as(_ip), seg.shape[0], ext.ctypes.data_as(_up), network.numSeg]

    @staticmethod
    def _segforce(network):
        sf = network.segForce
        if not (sf.flags.f_contiguous and sf.dtype == np.float64 and sf.shape[:2] == (3, 2)):
            raise ValueError("segForce must be a Fortran-ordered float64 3×2×n array")
        return sf

    @staticmethod
    def _sigma_hat(sigma_hat, n):
        if sigma_hat is None:
            return None
        sh = np.require(sigma_hat, np.float64, ["F"])
        if sh.shape != (6, n):
            raise ValueError("sigmaHat must be 6×n (xx, yy, zz, xy, xz, yz per entry)")
        return sh

    def self_force(self, k, sp, network, idx=None):
        """calcSelfForce: (F1, F2), each 3×n."""
        idx = self._idx(idx)
        n = network.numSeg if idx is None else len(idx)
        F1 = np.zeros((3, n), np.float64, order="F")
        F2 = np.zeros((3, n), np.float64, order="F")
        self._check(self._L.ddd_self_force(self._h, ctypes.byref(k), ctypes.byref(sp), *self._netp(network),
                                           None if idx is None else idx.ctypes.data_as(_ip),
                                           0 if idx is None else len(idx), F1.ctypes.data_as(_dp),
                                           F2.ctypes.data_as(_dp)))
        return F1, F2

    def self_force_inplace(self, k, sp, network, idx=None):
        idx = self._idx(idx)
        sf = self._segforce(network)
        self._check(self._L.ddd_self_force_inplace(self._h, ctypes.byref(k), ctypes.byref(sp), *self._netp(network),
                                                   None if idx is None else idx.ctypes.data_as(_ip),
                                                   0 if idx is None else len(idx), sf.ctypes.data_as(_dp),
                                                   sf.shape[2]))

    def seg_force(self, k, sp, network, sigma_hat=None, idx=None):
        """calcSegForce: seg-seg + self + PK/2 per node (3×2×n)."""
        idx = self._idx(idx)
        n = network.numSeg if idx is None else len(idx)
        sh = self._sigma_hat(sigma_hat, n)
        out = np.zeros((3, 2, n), np.float64, order="F")
        rep = ddd_report()
        self._check(self._L.ddd_seg_force(self._h, ctypes.byref(k), ctypes.byref(sp), *self._netp(network),
                                          None if sh is None else sh.ctypes.data_as(_dp),
                                          None if idx is None else idx.ctypes.data_as(_ip),
                                          0 if idx is None else len(idx), out.ctypes.data_as(_dp), ctypes.byref(rep)))
        self.last_report = rep.as_dict()
        return out

    def seg_force_inplace(self, k, sp, network, sigma_hat=None, idx=None):
        idx = self._idx(idx)
        n = network.numSeg if idx is None else len(idx)
        sh = self._sigma_hat(sigma_hat, n)
        sf = self._segforce(network)
        rep = ddd_report()
        self._check(self._L.ddd_seg_force_inplace(self._h, ctypes.byref(k), ctypes.byref(sp), *self._netp(network),
                                                  None if sh is None else sh.ctypes.data_as(_dp),
                                                  None if idx is None else idx.ctypes.data_as(_ip),
                                                  0 if idx is None else len(idx), sf.ctypes.data_as(_dp),
                                                  sf.shape[2], ctypes.byref(rep)))
        self.last_report = rep.as_dict()

    def _mob_args(self, mp, network, idx):
        coord = np.require(network.coord, np.float64, ["F"])
        bvec = np.require(network.bVec, np.float64, ["F"])
        links = np.require(network.links, np.int64, ["F"])
        conn = np.require(network.connectivity, np.int64, ["F"])
        sf = np.require(network.segForce, np.float64, ["F"])
        keep = (coord, bvec, links, conn, sf)
        args = [self._h, ctypes.byref(mp), coord.ctypes.data_as(_dp), coord.shape[1], bvec.ctypes.data_as(_dp),
                bvec.shape[1], links.ctypes.data_as(_ip), links.shape[1], conn.ctypes.data_as(_ip), conn.shape[0],
                conn.shape[1], sf.ctypes.data_as(_dp), sf.shape[2], network.numNode,
                None if idx is None else idx.ctypes.data_as(_ip), 0 if idx is None else len(idx)]
        return args, keep

    def detect_collision(self, collision_dist_sq, network, skip_segs=()):
        """detectCollision: the reference's 10-tuple and a dict with the reported
        pair's own distSq, L1 and L2."""
        net = network
        sk = np.ascontiguousarray(np.asarray(list(skip_segs), np.int64).reshape(-1, 2))
        for name in ("coord", "nodeVel", "bVec", "links", "connectivity"):
            a = getattr(net, name)
            if not a.flags.f_contiguous:
                raise ValueError(name + " must be Fortran-ordered")
        lab = np.ascontiguousarray(net.label, np.int32)
        r = ddd_collision()
        self._check(self._L.ddd_detect_collision(
            self._h, float(collision_dist_sq), net.coord.ctypes.data_as(_dp), net.coord.shape[1],
            net.nodeVel.ctypes.data_as(_dp), net.nodeVel.shape[1], lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            lab.shape[0], net.links.ctypes.data_as(_ip), net.links.shape[1], net.bVec.ctypes.data_as(_dp),
            net.bVec.shape[1], net.connectivity.ctypes.data_as(_ip), net.connectivity.shape[0],
            net.connectivity.shape[1], net.numNode, net.links.shape[1] if net.numSeg is None else net.numSeg,
            sk.ctypes.data_as(_ip), sk.shape[0], ctypes.byref(r)))
        res = (bool(r.collision), ("null", "hinge", "twoLine")[r.type], r.n1s1, r.n2s1, r.n1s2, r.n2s2, r.s1, r.s2,
               r.L1, r.L2)
        return res, {"distSq": r.pairDistSq, "L1": r.pairL1, "L2": r.pairL2}

    def u_tilde(self, omNuInv8pi, om2NuOmNuInv8pi, mesh, points, network, uDofs=None, out=None, tol=0.0):
        """calc_uTilde's kernel: adds u of point p, component c to
        out[uDofs[3p + c] - 1] (or out[3p + c]); returns out."""
        pts = np.require(points, np.float64, ["F"])
        M = pts.shape[1]
        if out is None:
            out = np.zeros(3 * M)
        if out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float64 vector")
        dofs = None if uDofs is None else np.ascontiguousarray(uDofs, np.int64)
        if dofs is not None and dofs.shape[0] != 3 * M:
            raise ValueError("uDofs must have 3 entries per point")
        fn = np.require(mesh.faceNorm, np.float64, ["F"])
        fm = np.require(mesh.faceMidPt, np.float64, ["F"])
        nr = np.require(mesh.normals, np.float64, ["F"])
        m = ddd_u_mesh()
        for k in range(3):
            m.C[k], m.lo[k], m.hi[k] = mesh.closure[k], mesh.lo[k], mesh.hi[k]
        m.tol = float(tol)
        m.faceNorm, m.faceMidPt, m.numFaces = fn.ctypes.data_as(_dp), fm.ctypes.data_as(_dp), fn.shape[1]
        m.normals, m.numNormals = nr.ctypes.data_as(_dp), nr.shape[1]
        net = network
        lab = np.ascontiguousarray(net.label, np.int32)
        self._check(self._L.ddd_u_tilde(
            self._h, float(omNuInv8pi), float(om2NuOmNuInv8pi), ctypes.byref(m), pts.ctypes.data_as(_dp), M,
            net.coord.ctypes.data_as(_dp), net.coord.shape[1], lab.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            lab.shape[0], net.links.ctypes.data_as(_ip), net.links.shape[1], net.bVec.ctypes.data_as(_dp),
            net.bVec.shape[1], net.numNode, net.numSeg, None if dofs is None else dofs.ctypes.data_as(_ip),
            out.ctypes.data_as(_dp), out.shape[0]))
        return out

    def minimum_distance(self, pts):
        """minimumDistance for pts (3 × 8 × n): 4 × n (distSq, dDistSqDt, L1, L2)."""
        pts = np.require(pts, np.float64, ["F"])
        n = pts.shape[2]
        out = np.zeros((4, n), np.float64, order="F")
        self._check(self._L.ddd_minimum_distance(self._h, pts.ctypes.data_as(_dp), n, out.ctypes.data_as(_dp)))
        return out

    @property
    def last_kernel_ms(self):
        """Device time of the kernel of the last self-force / segment-force / mobility call."""
        return self._L.ddd_last_kernel_ms(self._h)

    def mobility_bcc(self, mp, network, idx=None):
        """dlnMobility (BCC): (nodeForce, nodeVel), 3×n each."""
        idx = self._idx(idx)
        n = network.numNode if idx is None else len(idx)
        F = np.zeros((3, n), np.float64, order="F")
        V = np.zeros((3, n), np.float64, order="F")
        args, keep = self._mob_args(mp, network, idx)
        self._check(self._L.ddd_mobility_bcc(*args, F.ctypes.data_as(_dp), V.ctypes.data_as(_dp)))
        return F, V

    def mobility_bcc_inplace(self, mp, network, idx=None):
        idx = self._idx(idx)
        nf, nv = network.nodeForce, network.nodeVel
        for a in (nf, nv):
            if not (a.flags.f_contiguous and a.dtype == np.float64 and a.shape[0] == 3):
                raise ValueError("nodeForce / nodeVel must be Fortran-ordered float64 3×n arrays")
        args, keep = self._mob_args(mp, network, idx)
        self._check(self._L.ddd_mobility_bcc_inplace(*args, nf.ctypes.data_as(_dp), nv.ctypes.data_as(_dp),
                                                     min(nf.shape[1], nv.shape[1])))

    def segseg_force_inplace(self, k, network, idx=None):
        coord, bvec, seg, ext = self._net(network)
        idx = self._idx(idx)
        sf = network.segForce
        if not (sf.flags.f_contiguous and sf.dtype == np.float64 and sf.shape[:2] == (3, 2)):
            raise ValueError("segForce must be a Fortran-ordered float64 3×2×n array")
        rep = ddd_report()
        rc = self._L.ddd_segseg_force_inplace(
            self._h, ctypes.byref(k), coord.ctypes.data_as(_dp), coord.shape[1], bvec.ctypes.data_as(_dp),
            bvec.shape[1], seg.ctypes.data_as(_ip), seg.shape[0], ext.ctypes.data_as(_up), network.numSeg,
            None if idx is None else idx.ctypes.data_as(_ip), 0 if idx is None else len(idx),
            sf.ctypes.data_as(_dp), sf.shape[2], ctypes.byref(rep))
        self._check(rc)
        self.last_report = rep.as_dict()

    def sigma_tilde(self, k, x0, network, idx=None, out=None):
        coord, bvec, seg, _ = self._net(network)
        x0 = np.require(x0, np.float64, ["F"])
        if x0.ndim == 1:
            x0 = x0.reshape(3, -1, order="F")
        if x0.shape[0] != 3:
            raise ValueError("x0 must be 3×M")
        M = x0.shape[1]
        idx = self._idx(idx)
        if out is None:
            out = np.zeros((6, M), np.float64, order="F")
        rep = ddd_report()
        rc = self._L.ddd_sigma_tilde(
            self._h, ctypes.byref(k), x0.ctypes.data_as(_dp), M, coord.ctypes.data_as(_dp), coord.shape[1],
            bvec.ctypes.data_as(_dp), bvec.shape[1], seg.ctypes.data_as(_ip), seg.shape[0], network.numSeg,
            None if idx is None else idx.ctypes.data_as(_ip), 0 if idx is None else len(idx),
            out.ctypes.data_as(_dp), ctypes.byref(rep))
        self._check(rc)
        self.last_report = rep.as_dict()
        return out

    def segseg_force_device(self, k, segs_ptr, ld, numSeg, force_ptr, ext_ptr=None, stream=None, report=False):
        """Device-resident all-pairs call; pointers are raw device addresses (ints)."""
        rep = ddd_report() if report else None
        rc = self._L.ddd_segseg_force_device(self._h, ctypes.byref(k), segs_ptr, ld, ext_ptr, numSeg, force_ptr,
                                             stream, ctypes.byref(rep) if report else None)
        self._check(rc)
        return rep.as_dict() if report else None

    def sigma_tilde_device(self, k, x0_ptr, M, segs_ptr, ld, numSeg, sigma_ptr, stream=None, report=False):
        rep = ddd_report() if report else None
        rc = self._L.ddd_sigma_tilde_device(self._h, ctypes.byref(k), x0_ptr, M, segs_ptr, ld, numSeg, sigma_ptr,
                                            stream, ctypes.byref(rep) if report else None)
        self._check(rc)
        return rep.as_dict() if report else None

    @property
    def mode(self):
        return self._L.ddd_get_mode(self._h)

    @mode.setter
    def mode(self, m):
        self._check(self._L.ddd_set_mode(self._h, MODES.get(m, m) if isinstance(m, str) else int(m)))

    @property
    def partial_limit(self):
        """Bytes of device memory for the all-pairs partial sums; past it the
        tile pairs run in bands of tile columns (set 0 for the default)."""
        return self._L.ddd_get_partial_limit(self._h)

    @partial_limit.setter
    def partial_limit(self, nbytes):
        self._check(self._L.ddd_set_partial_limit(self._h, int(nbytes)))

    def tc_gemm_bf16(self, M, N, K, a_ptr, b_ptr, d_ptr, stream=None):
        """D[M×N] fp32 = A[M×K] · B[N×K]^T on tcgen05 (device pointers)."""
        self._check(self._L.ddd_tc_gemm_bf16(self._h, M, N, K, a_ptr, b_ptr, d_ptr, stream))

    def probe_fma_peak(self, precision=64):
        v = ctypes.c_double(0)
        self._check(self._L.ddd_probe_fma_peak(self._h, int(precision), ctypes.byref(v)))
        return v.value

    @property
    def last_error(self):
        """ddd_last_error: the message of this context's last failed call."""
        return self._L.ddd_last_error(self._h).decode()

    def selftest_bounded_wait(self, max_clocks, arrive):
        """ddd_selftest_bounded_wait: the return code (DDD_OK or DDD_ETIMEOUT), not raised."""
        return self._L.ddd_selftest_bounded_wait(self._h, int(max_clocks), 1 if arrive else 0)


class Batch:
    """A batch plan (ddd_batch_*): many networks, one persistent launch in a CUDA graph."""

    def __init__(self, ctx, num_seg, mode="fp64", tune=False):
        self._L = ctx._L
        self.ctx = ctx
        sizes = np.ascontiguousarray(num_seg, dtype=np.int64)
        m = MODES.get(mode, mode) if isinstance(mode, str) else int(mode)
        self._h = self._L.ddd_batch_create(ctx._h, len(sizes), sizes.ctypes.data_as(_ip), m, 1 if tune else 0)
        if not self._h:
            raise DDDError(DDD_EINVAL, "ddd_batch_create failed (sizes or mode)")
        self.num_seg = sizes
        self.total = int(sizes.sum())

    def run(self, k, segs_ptr, force_ptr, ext_ptr=None, stream=None):
        rc = self._L.ddd_batch_run(self._h, ctypes.byref(k), segs_ptr, ext_ptr, force_ptr, stream)
        if rc != DDD_OK:
            raise DDDError(rc, self._L.ddd_batch_last_error(self._h).decode())

    def info(self):
        i = ddd_batch_info_t()
        self._L.ddd_batch_info(self._h, ctypes.byref(i))
        return i.as_dict()

    def close(self):
        if self._h:
            self._L.ddd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# Flat parameter layout of the surrogate (csrc/surrogate.cuh): name -> (offset, size).
_PARAM_OFF = {}
_o = 0
for _name, _size in (("W1", 128 * 8), ("b1", 128), ("W2", 128 * 128), ("b2", 128), ("W3", 128 * 128), ("b3", 128),
                     ("W4", 112 * 128), ("b4", 112)):
    _PARAM_OFF[_name] = (_o, _size)
    _o += _size
del _o, _name, _size

def packed_segments(network):
    """Packed 9 × numSeg segment array (n1 xyz, n2 xyz, b xyz per segment) of a
    DislocationNetwork, in segIdx row order (the layout of the device entry points)."""
    n = network.numSeg
    si = network.segIdx[:n]
    n1 = network.coord[:, si[:, 1] - 1]
    n2 = network.coord[:, si[:, 2] - 1]
    b = network.bVec[:, si[:, 0] - 1]
    return np.ascontiguousarray(np.concatenate([n1, n2, b], axis=0))


def _nu_of(k):
    """Poisson ratio from the derived constants (mu4pinu = mu4pi / (1 - nu))."""
    return 1.0 - k.mu4pi / k.mu4pinu


def sample_far_pairs(segs, count, kappa, rng, focus=0.0):
    """`count` random pairs (i != j) of the packed segments with midpoint
    separation R >= kappa * max(L_i, L_j): int32 array 2 × count.  focus > 0
    keeps a uniformly drawn far pair with probability (kappa max(L_i, L_j) / R)^focus,
    moving samples toward the trust region's edge, where a pair's force (and so
    its share of the node-force error) is largest."""
    n = segs.shape[1]
    m = 0.5 * (segs[0:3] + segs[3:6])
    L = np.linalg.norm(segs[3:6] - segs[0:3], axis=0)
    out, have = [], 0
    while have < count:
        ij = rng.integers(0, n, (2, max(1024, 2 * (count - have))))
        d2 = ((m[:, ij[1]] - m[:, ij[0]]) ** 2).sum(0)
        r02 = (kappa * np.maximum(L[ij[0]], L[ij[1]])) ** 2
        ok = (ij[0] != ij[1]) & (d2 >= r02)
        if focus > 0:
            ok &= rng.random(ok.shape) < (r02 / np.maximum(d2, r02)) ** (0.5 * focus)
        out.append(ij[:, ok])
        have += int(ok.sum())
    return np.ascontiguousarray(np.concatenate(out, axis=1)[:, :count].astype(np.int32))


class Surrogate:
    """The learned far-field surrogate (ddd_surrogate_*): training and evaluation on the GPU.

    kappa is the trust-region factor the network was trained for (far pairs:
    R >= kappa max(L_i, L_j)); nu the Poisson ratio of its training data (the
    scaled pair forces depend on nu, not on mu).  Both travel with save/load.
    """

    def __init__(self, ctx, seed=0):
        self._L = ctx._L
        self.ctx = ctx
        self._h = self._L.ddd_surrogate_create(ctx._h, int(seed))
        if not self._h:
            raise DDDError(DDD_EDEVICE, "ddd_surrogate_create failed")
        self.num_params = self._L.ddd_surrogate_num_params()
        self.kappa = 20.0
        self.nu = None
        self.aSq = None

    def _rc(self, rc, what):
        if rc != DDD_OK:
            detail = self._L.ddd_surrogate_last_error(self._h)
            raise DDDError(rc, what + (": " + detail.decode() if detail else ""))

    # -- training (the product path: sampling, output normalisation, folding) --
    def fit(self, k, networks, pairs_per_network=1 << 20, epochs=30, batch=4096, lr=2e-3, kappa=20.0,
            kappa_train=None, seed=0, weight_decay=0.0, focus=0.0):
        """Train on far pairs of `networks` (packed 9 × n float64 arrays) with
        the exact FP64 forces as targets.  Pairs are sampled among the pairs with
        R >= kappa_train max(L_i, L_j) (default 0.9 kappa, a margin around the
        trust region's edge), uniformly or, with focus > 0, weighted toward that
        edge (sample_far_pairs).  Each of the 12 scaled outputs is
        normalised by its standard deviation for training; the scales are folded
        into the last layer afterwards, so evaluation needs no extra step.
        Returns {"loss": per-epoch history, "samples": P, "sigma": scales}."""
        import torch
        kt = 0.9 * kappa if kappa_train is None else kappa_train
        rng = np.random.default_rng(seed)
        Xs, Bs, Ts = [], [], []
        for segs in networks:
            segs = np.ascontiguousarray(segs, dtype=np.float64)
            pairs = sample_far_pairs(segs, pairs_per_network, kt, rng, focus)
            P = pairs.shape[1]
            X = torch.zeros((P, 16), dtype=torch.float16, device="cuda")  # hi and lo feature parts
            Bp = torch.zeros((P, 16), dtype=torch.float32, device="cuda")
            T = torch.zeros((P, 16), dtype=torch.float32, device="cuda")
            dsegs, dpairs = torch.from_numpy(segs).cuda(), torch.from_numpy(pairs).cuda()
            self.make_data(k, dsegs.data_ptr(), segs.shape[1], dpairs.data_ptr(), P, X.data_ptr(), Bp.data_ptr(),
                           T.data_ptr())
            Xs.append(X)
            Bs.append(Bp)
            Ts.append(T)
            del dsegs, dpairs
        X, Bp, T = torch.cat(Xs), torch.cat(Bs), torch.cat(Ts)
        del Xs, Bs, Ts
        g = torch.Generator().manual_seed(int(seed))
        perm = torch.randperm(X.shape[0], generator=g).cuda()
        P = (X.shape[0] // batch) * batch
        X, Bp, T = X[perm[:P]].contiguous(), Bp[perm[:P]].contiguous(), T[perm[:P]].contiguous()
        sig = T[:, :12].double().std(0).clamp_min(1e-12).float()
        sig16 = torch.ones(16, device="cuda")
        sig16[:12] = sig
        Tn = (T / sig16).contiguous()
        hist = self.train(X.data_ptr(), Bp.data_ptr(), Tn.data_ptr(), P, batch, epochs, lr=lr,
                          weight_decay=weight_decay)
        # Fold the output scales into the last layer: coefficient row 12 ac + o scales by sigma_o.
        flat = self.params()
        s12 = sig.cpu().numpy().astype(np.float64)
        rows = np.ones(112)
        rows[:108] = np.tile(s12, 9)
        o, n = _PARAM_OFF["W4"]
        flat[o:o + n] = (flat[o:o + n].reshape(112, 128) * rows[:, None]).ravel()
        o, n = _PARAM_OFF["b4"]
        flat[o:o + n] *= rows
        self.set_params(flat)
        self.kappa, self.nu, self.aSq = float(kappa), _nu_of(k), float(k.aSq)
        return {"loss": hist, "samples": P, "sigma": s12}

    # -- forces ---------------------------------------------------------------
    def force(self, k, segs, ext=None, kappa=None, audit_fraction=0.01, audit_tol=1e-3, exact_mode="fp64", out=None,
              stream=None, far="network", kappa_two=None):
        """ddd_surrogate_force on packed 9 × n segments (a CUDA float64 tensor or
        a numpy array); exact_mode: arithmetic of the exact near / audit passes
        ("fp64", "fp64_fast", "df64" or "f32c"); far: "network", or "quad2" / "quad3" for
        the far pairs by FP32 Gauss-Legendre quadrature (no network used);
        kappa_two: "quad3"'s switch to 2 points beyond that many lengths
        (default QUAD_KAPPA_TWO, 0 = off).
        Returns (forces as a CUDA tensor n × 6 = the 3 × 2 × n column-major
        array, report dict)."""
        import torch
        o = self._opts(k, kappa, audit_fraction, audit_tol, exact_mode, far, kappa_two)
        if not isinstance(segs, torch.Tensor):
            segs = torch.from_numpy(np.ascontiguousarray(segs, dtype=np.float64)).cuda()
        assert segs.dtype == torch.float64 and segs.is_cuda and segs.dim() == 2 and segs.shape[0] == 9
        segs = segs.contiguous()
        n = segs.shape[1]
        if ext is not None and not isinstance(ext, torch.Tensor):
            ext = torch.from_numpy(np.ascontiguousarray(ext, dtype=np.uint8)).cuda()
        if out is None:
            out = torch.empty((n, 6), dtype=torch.float64, device=segs.device)
        rep = ddd_sur_report()
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        self._rc(self._L.ddd_surrogate_force(self._h, ctypes.byref(k), segs.data_ptr(), n,
                                             ext.data_ptr() if ext is not None else None, n, out.data_ptr(), st,
                                             ctypes.byref(o), ctypes.byref(rep)), "surrogate force")
        return out, rep.as_dict()

    def _opts(self, k, kappa, audit_fraction, audit_tol, exact_mode, far="network", kappa_two=None):
        fm = FAR_MODES.get(far, far) if isinstance(far, str) else int(far)
        if fm == 0 and self.nu is not None and abs(_nu_of(k) - self.nu) > 1e-9:
            raise DDDError(DDD_EINVAL, "surrogate trained for nu = %.6g, called with nu = %.6g"
                           % (self.nu, _nu_of(k)))
        if kappa is None:
            kappa = QUAD_KAPPA if fm == 3 else (QUAD2_KAPPA if fm == 2 else self.kappa)
        if kappa_two is None:
            kappa_two = QUAD_KAPPA_TWO if fm == 3 else 0.0
        return ddd_sur_opts(float(kappa), float(audit_fraction), float(audit_tol),
                            MODES.get(exact_mode, exact_mode) if isinstance(exact_mode, str) else int(exact_mode),
                            fm, float(kappa_two))

    def force_network(self, dlnParams, matParams, network, kappa=None, audit_fraction=0.01, audit_tol=1e-3,
                      exact_mode="fp64", far="network", kappa_two=None):
        """The surrogate's calcSegSegForce on a DislocationNetwork's own host arrays
        (ddd_surrogate_force_host): a fresh 3×2×numSeg array and the report."""
        k = consts_of(dlnParams, matParams)
        o = self._opts(k, kappa, audit_fraction, audit_tol, exact_mode, far, kappa_two)
        n = network.numSeg
        F = np.zeros((3, 2, n), np.float64, order="F")
        rep = ddd_sur_report()
        self._rc(self._L.ddd_surrogate_force_host(
            self._h, ctypes.byref(k), network.coord.ctypes.data_as(_dp), network.coord.shape[1],
            network.bVec.ctypes.data_as(_dp), network.bVec.shape[1], network.segIdx.ctypes.data_as(_ip),
            network.segIdx.shape[0], network.extSeg.ctypes.data_as(_up), n, F.ctypes.data_as(_dp),
            ctypes.byref(o), ctypes.byref(rep)), "surrogate force")
        return F, rep.as_dict()

    # -- checkpoints (format: ddd_surrogate_save in include/ddd_gb300.h) -------
    def save(self, path):
        self._rc(self._L.ddd_surrogate_save(self._h, os.fsencode(path), self.kappa,
                                            math.nan if self.nu is None else self.nu,
                                            math.nan if self.aSq is None else self.aSq), "save")

    def load(self, path):
        kappa, nu, aSq = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._rc(self._L.ddd_surrogate_load(self._h, os.fsencode(path), ctypes.byref(kappa), ctypes.byref(nu),
                                            ctypes.byref(aSq)), "load")
        self.kappa = kappa.value
        self.nu = None if math.isnan(nu.value) else nu.value
        self.aSq = None if math.isnan(aSq.value) else aSq.value
        return self

    def params(self):
        out = np.zeros(self.num_params, np.float32)
        self._rc(self._L.ddd_surrogate_params(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 0),
                 "params")
        return out

    def set_params(self, flat):
        flat = np.ascontiguousarray(flat, np.float32)
        assert flat.size == self.num_params
        self._rc(self._L.ddd_surrogate_params(self._h, flat.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 1),
                 "set_params")

    def make_data(self, k, segs_ptr, n, pairs_ptr, P, X_ptr, Bp_ptr, T_ptr, F_ptr=None):
        """Features X (P x 16 BF16), Burgers-vector products Bp and scaled exact
        targets T (P x 16 FP32 each) of P pairs (device pointers)."""
        self.ctx._check(self._L.ddd_surrogate_make_data(self.ctx._h, ctypes.byref(k), segs_ptr, n, pairs_ptr, P,
                                                        X_ptr, Bp_ptr, T_ptr, F_ptr))

    def train(self, X_ptr, Bp_ptr, T_ptr, P, batch, epochs, lr=1e-3, weight_decay=0.0):
        hist = np.zeros(epochs)
        self._rc(self._L.ddd_surrogate_train(self._h, X_ptr, Bp_ptr, T_ptr, P, batch, epochs, lr, weight_decay,
                                             hist.ctypes.data_as(_dp)), "train")
        return hist

    def forward(self, X_ptr, Bp_ptr, P, O_ptr):
        self._rc(self._L.ddd_surrogate_forward(self._h, X_ptr, Bp_ptr, P, O_ptr), "forward")

    def grads(self, X_ptr, Bp_ptr, T_ptr, B):
        loss = ctypes.c_double(0)
        g = np.zeros(self.num_params, np.float32)
        self._rc(self._L.ddd_surrogate_grads(self._h, X_ptr, Bp_ptr, T_ptr, B, ctypes.byref(loss),
                                             g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "grads")
        return loss.value, g

    def close(self):
        if self._h:
            self._L.ddd_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_contexts = {}


def get_context(device=0):
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


# ---------------------------------------------------------------------------
# The reference's interface.

def calcSegSegForce(dlnParams, matParams, network, idx=None):
    """calcSegSegForce (DislocationForces.jl:470-561): a fresh 3×2×numSeg array
    (or 3×2×length(idx) for an index list)."""
    return get_context().segseg_force(consts_of(dlnParams, matParams), network, idx)


def calcSegSegForce_inplace(dlnParams, matParams, network, idx=None):
    """calcSegSegForce! (DislocationForces.jl:576-669): adds into network.segForce."""
    get_context().segseg_force_inplace(consts_of(dlnParams, matParams), network, idx)
    return None


def calcSelfForce(dlnParams, matParams, network, idx=None):
    """calcSelfForce (DislocationForces.jl:320-353): (selfForceNode1, selfForceNode2), each 3×n."""
    return get_context().self_force(consts_of(dlnParams, matParams), self_params_of(dlnParams, matParams), network,
                                    idx)


def calcSelfForce_inplace(dlnParams, matParams, network, idx=None):
    """calcSelfForce! (DislocationForces.jl:354-387): node 1 -= s, node 2 += s in network.segForce."""
    get_context().self_force_inplace(consts_of(dlnParams, matParams), self_params_of(dlnParams, matParams), network,
                                     idx)
    return None


def calcSegForce(dlnParams, matParams, sigmaHat, network, idx=None):
    """calcSegForce (DislocationForces.jl:23-46) with the finite-element part given
    as data: sigmaHat (6×n: xx, yy, zz, xy, xz, yz) is calc_σHat(mesh,
    forceDisplacement, x0) at each segment's midpoint (None: no PK term).  Returns
    3×2×n: seg-seg + self + PK/2 per node."""
    return get_context().seg_force(consts_of(dlnParams, matParams), self_params_of(dlnParams, matParams), network,
                                   sigmaHat, idx)


def calcSegForce_inplace(dlnParams, matParams, sigmaHat, network, idx=None):
    """calcSegForce! (DislocationForces.jl:48-72): zeroes the entries' columns of
    network.segForce, then adds PK/2, the self force and the seg-seg force."""
    get_context().seg_force_inplace(consts_of(dlnParams, matParams), self_params_of(dlnParams, matParams), network,
                                    sigmaHat, idx)
    return None


def mob_params_of(dlnParams, matParams):
    d = dlnParams.dragCoeffs
    mp = ddd_mob_params()
    mp.sigmaPN = matParams.σPN
    mp.edgeDrag, mp.screwDrag, mp.climbDrag, mp.lineDrag = d["edge"], d["screw"], d["climb"], d["line"]
    return mp


def dlnMobility(dlnParams, matParams, network, idx=None):
    """dlnMobility for a BCC material (DislocationMobility.jl:16-178): (nodeForce, nodeVel), 3×n each."""
    return get_context().mobility_bcc(mob_params_of(dlnParams, matParams), network, idx)


def dlnMobility_inplace(dlnParams, matParams, network, idx=None):
    """dlnMobility! (DislocationMobility.jl:186-341): writes network.nodeForce and nodeVel."""
    get_context().mobility_bcc_inplace(mob_params_of(dlnParams, matParams), network, idx)
    return network


def detectCollision(dlnParams, network, skipSegs=()):
    """detectCollision (DislocationTopologyCollision.jl:1-221): (collision,
    collisionType, n1s1, n2s1, n1s2, n2s2, s1, s2, L1, L2), collisionType one of
    "null", "hinge", "twoLine" (the reference's symbols).  L1, L2 are the
    reference's: those of the last pair it evaluated."""
    return get_context().detect_collision(dlnParams.collisionDistSq, network, skipSegs)[0]


def minimumDistance(x0, x1, y0, y1, vx0, vx1, vy0, vy1):
    """minimumDistance (Misc.jl:314-367) for one pair of segments (3-vectors) or
    n pairs (3 × n arrays): (distSq, dDistSqDt, L1, L2)."""
    arrs = [np.asarray(a, np.float64).reshape(3, -1, order="F") for a in (x0, x1, y0, y1, vx0, vx1, vy0, vy1)]
    out = get_context().minimum_distance(np.stack(arrs, axis=1))
    single = all(np.ndim(a) == 1 for a in (x0, x1, y0, y1, vx0, vx1, vy0, vy1))
    return tuple(float(v[0]) for v in out) if single else tuple(out)


def calc_uTilde(mesh, boundaries, matParams, network):
    """calc_uTilde (DislocationFEM.jl:375-391): the displacements at the FE nodes
    boundaries.uGammaDln, point-major (ux, uy, uz of each node in turn).  mesh:
    fem.RegularCuboidMesh; boundaries: fem.Boundaries."""
    pts = np.asfortranarray(mesh.coord[:, boundaries.uGammaDln - 1])
    return get_context().u_tilde(matParams.omνInv8π, matParams.om2νomνInv8π, mesh, pts, network)


def calc_uTilde_inplace(forceDisplacement, mesh, boundaries, matParams, network):
    """calc_uTilde! (DislocationFEM.jl:362-373): zeroes forceDisplacement.uTilde
    and adds point p's component c at uDofsDln[3p + c], the reference's indexing."""
    forceDisplacement.uTilde[:] = 0.0
    pts = np.asfortranarray(mesh.coord[:, boundaries.uGammaDln - 1])
    get_context().u_tilde(matParams.omνInv8π, matParams.om2νomνInv8π, mesh, pts, network, boundaries.uDofsDln,
                          forceDisplacement.uTilde)
    return forceDisplacement


class ProductIterator:
    """Iterators.product(xs, ys, zs), the grid form of calc_σTilde's points
    (DislocationFEM.jl:33-37, :126-140): every (x, y, z) of xs × ys × zs, the
    first factor varying fastest as Julia enumerates it."""

    def __init__(self, xs, ys, zs):
        self.factors = [np.asarray(f, dtype=np.float64).ravel() for f in (xs, ys, zs)]

    def __len__(self):
        return int(np.prod([len(f) for f in self.factors]))

    @property
    def ndim(self):
        return 3

    def points(self):
        """The points as a 3 × M array, in the iterator's order."""
        grids = np.meshgrid(*self.factors, indexing="ij")
        return np.asfortranarray(np.stack([g.ravel(order="F") for g in grids]))


def calc_σTilde(x0, dlnParams, matParams, network, idx=None):
    """calc_σTilde (DislocationFEM.jl:24-41): 6×M stresses, or a 6-vector for
    one point; x0 a 3×M array or a ProductIterator (a grid of points)."""
    x0 = x0.points() if isinstance(x0, ProductIterator) else np.asarray(x0, dtype=np.float64)
    sig = get_context().sigma_tilde(consts_of(dlnParams, matParams), x0.reshape(3, -1, order="F"), network, idx)
    return sig[:, 0].copy() if sig.shape[1] == 1 else sig


def calc_σTilde_inplace(σ, x0, dlnParams, matParams, network, idx=None):
    """calc_σTilde! (DislocationFEM.jl:67-84): asserts the shapes, then overwrites σ.
    A ProductIterator fails the assertion, as in the reference (ndims 3)."""
    if not isinstance(x0, ProductIterator):
        x0 = np.asarray(x0, dtype=np.float64)
    if not (σ.ndim == x0.ndim and σ.shape[0] == 6):
        raise AssertionError("ndims(σ) == ndims(x0) && size(σ, 1) == 6")
    if σ.ndim == 2 and σ.shape[1] != x0.shape[1]:
        raise AssertionError("size(σ, 2) == size(x0, 2)")
    sig = get_context().sigma_tilde(consts_of(dlnParams, matParams), x0.reshape(3, -1, order="F"), network, idx)
    σ[...] = sig.reshape(σ.shape, order="F")
    return σ


calc_sigmaTilde = calc_σTilde
calc_sigmaTilde_inplace = calc_σTilde_inplace


from . import fem  # noqa: E402  (RegularCuboidMesh, Boundaries, cantilever_boundaries, ForceDisplacement)
from . import json_io  # noqa: E402
from .json_io import loadJSON, loadNetwork, saveJSON  # noqa: E402,F401
