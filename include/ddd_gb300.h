/* ddd_gb300 — C ABI of the GB300 implementation of DDD.jl's O(N^2) elastic
 * interaction hot path: the non-singular segment–segment force and the
 * field-point stress of a dislocation network.
 *
 * Every array argument uses the memory image of the corresponding Julia field
 * of DDD.jl's DislocationNetwork (src/Type/DislocationType.jl:324-340):
 * column-major, 1-based indices, Float64 / Int64 / Bool(1 byte):
 *
 *   coord    double[3 * coordCols]      network.coord      (3 × nodeBuf)
 *   bVec     double[3 * bVecCols]       network.bVec       (3 × linkBuf)
 *   segIdx   int64 [ldSegIdx * 3]       network.segIdx     (linkBuf × 3: link, node1, node2)
 *   extSeg   uint8 [numSeg]             network.extSeg     (may be NULL = no external segments)
 *   force    double[3 * 2 * n]          segForce layout    F[k + 3*(node + 2*s)]
 *   x0       double[3 * numPoints]      field points       (3 × M)
 *   sigma    double[6 * numPoints]      (xx, yy, zz, xy, xz, yz) per point
 *   idx      int64 [nIdx]               1-based segment numbers, NULL = all segments
 *
 * The caller owns all host arrays; the library copies in, computes on the GPU
 * and copies out before returning.  No pointer is kept after a call returns.
 * Device scratch belongs to the context and is reused across calls (grow-only).
 * Calls on one context are serialised by an internal mutex; separate contexts
 * are independent.  There is no CPU fallback: with no usable GPU, ddd_create
 * returns NULL and every call reports DDD_EDEVICE.
 *
 * Return codes: DDD_OK (0) or a negative DDD_E* code; ddd_last_error() gives
 * the message.  Nothing aborts, traps or exits the process.
 */
#ifndef DDD_GB300_H
#define DDD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DDD_OK 0
#define DDD_EINVAL (-1)     /* null pointer, negative or inconsistent size */
#define DDD_ERANGE (-2)     /* an index (segIdx entry or idx entry) out of range */
#define DDD_ENONFINITE (-3) /* a non-finite coordinate / Burgers vector / constant, or a zero-length segment */
#define DDD_EDEVICE (-4)    /* CUDA error (message in ddd_last_error) */
#define DDD_ENOMEM (-5)     /* device allocation failed */
#define DDD_ETOOBIG (-6)    /* input larger than the entry point accepts (noalloc segment limit, 2^31 nodes) */
#define DDD_ETIMEOUT (-7)   /* a bounded wait inside a kernel gave up (the kernel returned early) */

typedef struct ddd_ctx ddd_ctx;

/* Arithmetic modes of a context (ddd_set_mode).  The reference has one method,
 * Float64 with every multiply and add rounded separately; DDD_MODE_FP64 is
 * that method and the default.  DDD_MODE_FP64_FMA evaluates the same formulas
 * with fused multiply-adds (faster; its rounding differs at the level of the
 * algorithm's own Float64 noise). */
#define DDD_MODE_FP64 0
#define DDD_MODE_FP64_FMA 1
/* DDD_MODE_DF64, the precision form of the seg-seg force: the general-branch
 * pair arithmetic as double-float (pairs of FP32, ~48-bit significands) on the
 * FP32 pipes; the near-parallel branch, the branch decision and the per-node
 * accumulation stay FP64.  Its error is of the order of 2^6 times the FP64
 * form's own rounding error (FP32-pair vs FP64 unit roundoff).  The field
 * stress (ddd_sigma_tilde*) runs in the mixed form in this mode and in
 * DDD_MODE_F32C: geometry, endpoint terms and their differences in df64,
 * coefficient assembly in FP32, per-point sums in df64 (~1e-7 relative). */
#define DDD_MODE_DF64 2
/* DDD_MODE_F32C, the FP32 form with compensated terms: the integration-domain
 * geometry, the four corner antiderivatives (their logs, arctangents, roots and
 * quotients) and their first moments in double-float, where the formula
 * cancels; the V-vector assembly and node sums in plain FP32; near-parallel
 * branch, branch decision and per-node accumulation in FP64 as in
 * DDD_MODE_DF64.  Measured node-force error ~5e-8 relative RMS. */
#define DDD_MODE_F32C 3
/* DDD_MODE_FP64_FAST, FP64 throughout with fewer FP64 instructions per pair:
 * the general branch with one division per corner instead of four,
 * logarithms and arctangents computed in integer fixed point on the integer
 * pipes (within 0.51 ulp; they take no FP64 pipe time), and fused multiply-adds
 * wherever the reference's terms do not cancel; the quantities whose rounding
 * sets the reference's own error (c, 1 - c^2, the pair geometry, the local
 * coordinates, Ra and Ra + y + x c) are rounded as the reference rounds them,
 * and the near-parallel branch is the strict code.  Its node forces stay
 * within the reference arithmetic's own rounding noise (the same parity bound
 * as DDD_MODE_FP64).  The field stress runs its own fast form in this mode:
 * the six components regrouped on four vectors and seven scalars, 1/Ra by a
 * reciprocal square root, fused multiply-adds (about half the FP64
 * instructions; within the strict form's per-point bound). */
#define DDD_MODE_FP64_FAST 4

/* Constants of the path.  The reference computes them in
 * MaterialParameters (src/Type/MaterialConstructor.jl:66-82) and
 * DislocationParameters (src/Type/DislocationConstructor.jl:83). */
typedef struct ddd_consts {
  double aSq;       /* dlnParams.coreRadSq = coreRad^2 */
  double mu4pi;     /* matParams.μ4π  = μ / (4π) */
  double mu8pi;     /* matParams.μ8π  = μ4π / 2 */
  double mu4pinu;   /* matParams.μ4πν = μ4π / (1 - ν) */
  double nuMu4pinu; /* matParams.νμ4πν = ν μ4πν (σ̃ only) */
} ddd_consts;

/* Optional per-call report (pass NULL to skip). */
typedef struct ddd_report {
  int64_t pairs_general;   /* pairs evaluated on the general branch */
  int64_t pairs_parallel;  /* pairs routed to the near-parallel branch (1 - c^2 <= sqrt(eps)) */
  int64_t core_sides;      /* near-parallel sides that needed the two core-correction evaluations */
  double kernel_ms;        /* device time of the compute kernels */
  double total_ms;         /* device time of the call including host<->device copies */
  int64_t h2d_bytes;       /* bytes copied host -> device */
  int64_t d2h_bytes;       /* bytes copied device -> host */
} ddd_report;

/* Context on CUDA device `device`; NULL on failure (ddd_last_error(NULL)). */
ddd_ctx* ddd_create(int device);
void ddd_destroy(ddd_ctx* ctx);
/* Message of the last failed call on ctx (or of the last failed ddd_create when ctx is NULL). */
const char* ddd_last_error(const ddd_ctx* ctx);
/* Device time (ms, CUDA events around the launches) of the kernels of the last
 * successful ddd_self_force* / ddd_seg_force* / ddd_mobility_bcc* /
 * ddd_detect_collision / ddd_u_tilde call on ctx.
 * No reference counterpart: measurement only. */
double ddd_last_kernel_ms(const ddd_ctx* ctx);
/* ABI version, 100 * major + minor. */
int ddd_version(void);

/* calcSegSegForce(dlnParams, matParams, network, idx = nothing)
 *   src/Processing/DislocationForces.jl:470-561 (dispatch :497-561, Ser :778-829,
 *   Par :719-777, idx form :528-557 + calcSegSegForceIdx! :831-877).
 * idx == NULL: all unordered pairs i < j, both skipped when extSeg; force is
 *   3 × 2 × numSeg and is overwritten.
 * idx != NULL: for each k, i = idx[k] (1-based, duplicates allowed), the sum over
 *   all j != i (non-external) of the forces on segment i's two nodes; force is
 *   3 × 2 × nIdx and is overwritten; column k stays 0 when segment i is external. */
int ddd_segseg_force(ddd_ctx* ctx, const ddd_consts* k, const double* coord, int64_t coordCols, const double* bVec,
                     int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx, const uint8_t* extSeg,
                     int64_t numSeg, const int64_t* idx, int64_t nIdx, double* force, ddd_report* rep);

/* calcSegSegForce!(dlnParams, matParams, network, idx = nothing)
 *   src/Processing/DislocationForces.jl:576-669.
 * Adds into segForce (3 × 2 × segForceCols, segForceCols >= numSeg):
 * idx == NULL: columns 1:numSeg += all-pairs forces;
 * idx != NULL: for each k, column idx[k] += that segment's forces (a repeated
 *   index adds repeatedly, as the reference's loop does). */
int ddd_segseg_force_inplace(ddd_ctx* ctx, const ddd_consts* k, const double* coord, int64_t coordCols,
                             const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                             const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx,
                             double* segForce, int64_t segForceCols, ddd_report* rep);

/* Self force and total segment force (the next row of the hot path's callers).
 * Parameters beyond ddd_consts: dlnParams.coreRad, dlnParams.coreEnergy and
 * matParams.ν (omνInv = 1/(1-ν), νomνInv = ν·omνInv as MaterialConstructor.jl:20-22
 * derives them); ddd_consts supplies coreRadSq (aSq) and μ4π. */
typedef struct ddd_self_params {
  double coreRad;
  double coreEnergy;
  double nu;
} ddd_self_params;

/* calcSelfForce(dlnParams, matParams, network, idx = nothing)
 *   src/Processing/DislocationForces.jl:320-353, kernel _calcSelfForce :414-455.
 * For each entry k of idx (1-based rows of segIdx) or of 1:numSeg: F1[:, k] =
 * the force on node 1, F2[:, k] = on node 2 (3 × n each, F1 = -F2).  As in the
 * reference, entry k is skipped (zeros) when extSeg[k] is set: the flag at the
 * position in idx, not at the segment (positions past numSeg count as internal). */
int ddd_self_force(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                   int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                   const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx, double* F1, double* F2);

/* calcSelfForce!(…) — :354-387: segForce[:, 1, idx[k]] -= s, segForce[:, 2, idx[k]] += s. */
int ddd_self_force_inplace(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                           int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx,
                           int64_t ldSegIdx, const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx,
                           double* segForce, int64_t segForceCols);

/* calcSegForce(dlnParams, matParams, mesh, forceDisplacement, network, idx)
 *   :23-46 — seg-seg + self + 0.5 PK per node, 3 × 2 × n fresh.  The PK force
 *   (σ̂ b) × t (:292-300) is computed here from sigmaHat (6 × n: xx, yy, zz, xy,
 *   xz, yz), the finite-element stress at each entry's segment midpoint that
 *   the caller evaluates with calc_σHat(mesh, forceDisplacement, x0) — the FE
 *   mesh is not part of this library; NULL = no PK term.
 * ddd_seg_force_inplace: calcSegForce! :48-72 — the columns of the entries
 *   are zeroed, then PK/2 (both nodes), the self force and the seg-seg force
 *   are added in the reference's order. */
int ddd_seg_force(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                  int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                  const uint8_t* extSeg, int64_t numSeg, const double* sigmaHat, const int64_t* idx, int64_t nIdx,
                  double* force, ddd_report* rep);
int ddd_seg_force_inplace(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                          int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx,
                          int64_t ldSegIdx, const uint8_t* extSeg, int64_t numSeg, const double* sigmaHat,
                          const int64_t* idx, int64_t nIdx, double* segForce, int64_t segForceCols, ddd_report* rep);

/* dlnMobility / dlnMobility! for a BCC material (mobBCC)
 *   src/Processing/DislocationMobility.jl:16-178 and :186-341.
 * For each node of idx (1-based) or of 1:numNode: the node force (sum of the
 * forces its connected segments put on it, zeroed below the Peierls-Nabarro
 * stress) and the velocity solving drag · v = force, the drag tensor built
 * from every connection (edge, screw, climb and line drags; BCC screw
 * families by the ratios of |b| components).  Arrays in the network's layout:
 * links 2 × linkCols and connectivity ldConn × connCols (ldConn = 1 +
 * 2 maxConnect; the _makeConnect! layout, DislocationUtil.jl:213-237), both
 * 1-based; segForce 3 × 2 × segForceCols.  ddd_mobility_bcc writes nodeForce
 * and nodeVel as 3 × n arrays; the _inplace form writes the nodes' columns of
 * the network's nodeForce / nodeVel (3 × nodeCols).  A node whose drag is
 * singular (no connections) gets NaN velocities, as the reference's solve. */
typedef struct ddd_mob_params {
  double sigmaPN;  /* matParams.σPN */
  double edgeDrag, screwDrag, climbDrag, lineDrag; /* dlnParams.dragCoeffs */
} ddd_mob_params;
int ddd_mobility_bcc(ddd_ctx* ctx, const ddd_mob_params* mp, const double* coord, int64_t coordCols,
                     const double* bVec, int64_t bVecCols, const int64_t* links, int64_t linkCols,
                     const int64_t* connectivity, int64_t ldConn, int64_t connCols, const double* segForce,
                     int64_t segForceCols, int64_t numNode, const int64_t* idx, int64_t nIdx, double* nodeForce,
                     double* nodeVel);
int ddd_mobility_bcc_inplace(ddd_ctx* ctx, const ddd_mob_params* mp, const double* coord, int64_t coordCols,
                             const double* bVec, int64_t bVecCols, const int64_t* links, int64_t linkCols,
                             const int64_t* connectivity, int64_t ldConn, int64_t connCols, const double* segForce,
                             int64_t segForceCols, int64_t numNode, const int64_t* idx, int64_t nIdx,
                             double* nodeForce, double* nodeVel, int64_t nodeCols);

/* detectCollision(dlnParams, network, skipSegs) —
 * src/Processing/DislocationTopologyCollision.jl:1-221 (minimumDistance:
 * src/Misc/Misc.jl:314-367).  Hinges (pairs of links at one mobile node) are
 * checked first, then every pair of unconnected segments whose four nodes are
 * mobile (label intMobDln = 1 or srfMobDln = 3); the reported pair is the one
 * with the largest 1/distSq among pairs closer than collisionDist and
 * approaching (dDistSqDt < -eps), the first in the reference's loop order on a
 * tie.  label: numNode int32 (the nodeTypeDln enum); nodeVel 3 × nodeVelCols;
 * links 2 × linkCols, connectivity ldConn × connCols (1-based); skipSegs: nSkip
 * (s1, s2) link pairs (Vector{Tuple{Int,Int}}), either order.  L1, L2 are what
 * the reference returns: the values of ITS LAST minimumDistance call (of the
 * last pair its loops evaluated), which need not be the reported pair;
 * pairDistSq, pairL1 and pairL2 belong to the reported pair (an extension).
 * Non-finite coordinates or velocities: DDD_ENONFINITE. */
typedef struct ddd_collision {
  int32_t collision; /* 1 when a collision was found */
  int32_t type;      /* 0 :null, 1 :hinge, 2 :twoLine */
  int64_t n1s1, n2s1, n1s2, n2s2, s1, s2; /* 1-based node and link numbers; 0 when none */
  double L1, L2;
  double pairDistSq, pairL1, pairL2;
} ddd_collision;
int ddd_detect_collision(ddd_ctx* ctx, double collisionDistSq, const double* coord, int64_t coordCols,
                         const double* nodeVel, int64_t nodeVelCols, const int32_t* label, int64_t labelLen,
                         const int64_t* links, int64_t linkCols, const double* bVec, int64_t bVecCols,
                         const int64_t* connectivity, int64_t ldConn, int64_t connCols, int64_t numNode,
                         int64_t numSeg, const int64_t* skipSegs, int64_t nSkip, ddd_collision* out);
/* minimumDistance(x0, x1, y0, y1, vx0, vx1, vy0, vy1) for n pairs at once:
 * pts 3 × 8 × n (the eight points of each pair), out 4 × n (distSq,
 * dDistSqDt, L1, L2). */
int ddd_minimum_distance(ddd_ctx* ctx, const double* pts, int64_t n, double* out);

/* calc_uTilde(mesh, boundaries, matParams, network) and calc_uTilde!(...) —
 * src/Processing/DislocationFEM.jl:355-581 (Barnett triangles :600-707): the
 * displacement the network causes at the FE nodes with applied displacements.
 * Each internal segment is closed on C (a full triangle, with the f and g
 * terms); a segment with an external node (label extDln = 5) is closed through
 * the points its nodes were projected out from (found on the mesh faces along
 * `normals`, or by walking the face planes), five solid-angle triangles; a
 * segment joining a surface node (labels 3, 4) to an external node only records
 * that connection for the segments after it.  The mesh enters as data:
 * mesh.vertices' mean (C), its bounding box (the "inside the volume" test,
 * widened by tol; tol <= 0 means 1e-10 of the largest extent), faceNorm and
 * faceMidPt (3 × numFaces) and the projection directions (3 × numNormals;
 * faceNorm[:, 1:2:5] for a regular cuboid, as the reference uses).  points:
 * mesh.coord[:, boundaries.uGammaDln] (3 × numPoints).  For point p and
 * component c: uTilde[uDofs[3p + c] - 1] += u_c(p), or uTilde[3p + c] when
 * uDofs is NULL (calc_uTilde's 1:3numPoints); calc_uTilde! passes
 * boundaries.uDofsDln after zeroing uTilde, exactly the reference's indexing.
 * Each point's sum runs over the triangles in the reference's order. */
typedef struct ddd_u_mesh {
  double C[3];
  double lo[3], hi[3];
  double tol;
  const double* faceNorm;
  const double* faceMidPt;
  int64_t numFaces;
  const double* normals;
  int64_t numNormals;
} ddd_u_mesh;
int ddd_u_tilde(ddd_ctx* ctx, double omNuInv8pi, double om2NuOmNuInv8pi, const ddd_u_mesh* mesh,
                const double* points, int64_t numPoints, const double* coord, int64_t coordCols, const int32_t* label,
                int64_t labelLen, const int64_t* links, int64_t linkCols, const double* bVec, int64_t bVecCols,
                int64_t numNode, int64_t numSeg, const int64_t* uDofs, double* uTilde, int64_t uLen);

/* calc_σTilde(x0, dlnParams, matParams, network, idx = nothing) and
 * calc_σTilde!(σ, x0, ...) — src/Processing/DislocationFEM.jl:24-84, kernel
 * _calc_σTilde! :86-303.  Both write sigma (6 × numPoints) fresh.  Segments are
 * rows 1:numSeg of segIdx, or the rows listed in idx (1-based, <= ldSegIdx);
 * extSeg is ignored, as in the reference. */
int ddd_sigma_tilde(ddd_ctx* ctx, const ddd_consts* k, const double* x0, int64_t numPoints, const double* coord,
                    int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx,
                    int64_t ldSegIdx, int64_t numSeg, const int64_t* idx, int64_t nIdx, double* sigma,
                    ddd_report* rep);

/* Device-resident forms, for callers whose network already lives in GPU memory.
 * segs is a packed structure-of-arrays of 9 rows × ldSegs (device pointer):
 * rows n1x n1y n1z n2x n2y n2z bx by bz, segment s in column s (0-based).
 * ext (device, may be NULL) marks external segments.  force / sigma are device
 * pointers in the layouts above.  The work is enqueued on `stream`
 * (a cudaStream_t, NULL = the context's stream) and the call returns without
 * waiting unless rep != NULL.  Same semantics as ddd_segseg_force (idx == NULL)
 * and ddd_sigma_tilde (idx == NULL). */
int ddd_segseg_force_device(ddd_ctx* ctx, const ddd_consts* k, const double* segs, int64_t ldSegs,
                            const uint8_t* ext, int64_t numSeg, double* force, void* stream, ddd_report* rep);
int ddd_sigma_tilde_device(ddd_ctx* ctx, const ddd_consts* k, const double* x0, int64_t numPoints,
                           const double* segs, int64_t ldSegs, int64_t numSeg, double* sigma, void* stream,
                           ddd_report* rep);

/* Allocation-free form of ddd_segseg_force_device (no counterpart in the
 * reference, which has no device memory): for callers that cannot let this
 * library allocate device memory — an application whose GPU memory is owned by
 * its own pool allocator, or a time-stepping loop that cannot afford the
 * device-wide synchronisation of cudaMalloc/cudaFree.  Inputs and output are
 * the caller's device buffers (layouts as ddd_segseg_force_device; ext may be
 * NULL); the work runs on the current CUDA device, on `stream` (a
 * cudaStream_t; NULL = the legacy default stream), in DDD_MODE_FP64 arithmetic,
 * and the call returns without waiting.  It calls no cudaMalloc, cudaFree or
 * other allocating routine: its scratch is a fixed device array of about
 * 6.9 MB.  The CUDA driver reserves that array, and loads the force kernels,
 * when it loads the library's modules on a device: under CUDA's default lazy
 * module loading that is inside the first call on each device (with
 * CUDA_MODULE_LOADING=EAGER, at context creation), and the memory stays
 * reserved until the process exits.  So make one call on each device during
 * set-up, before a pool allocator reserves the GPU: a call with numSeg = 0
 * does only this set-up (module loads, address lookup) and launches nothing.
 * Make that first call before any stream capture that contains later calls.
 * Limits: numSeg <= DDD_NOALLOC_MAX_SEGMENTS, else DDD_ETOOBIG.
 * Every call shares that array (it keeps the last call's contents; each call
 * writes every element it reads first), so calls that overlap on the GPU race:
 * serialise them.
 * Returns DDD_OK, DDD_EINVAL, DDD_ENONFINITE (a non-finite constant in k),
 * DDD_ETOOBIG or DDD_EDEVICE (no message). */
#define DDD_NOALLOC_MAX_SEGMENTS 4096
int ddd_segseg_force_device_noalloc(const ddd_consts* k, const double* segs, int64_t ldSegs, const uint8_t* ext,
                                    int64_t numSeg, double* force, void* stream);

/* Batched form (no reference counterpart: the reference evaluates one network
 * per call).  Many independent networks of uneven sizes in one persistent
 * launch replayed from a captured CUDA graph.  A batch plan is made for a list
 * of network sizes and a mode (DDD_MODE_FP64, DDD_MODE_FP64_FAST, DDD_MODE_DF64 or
 * DDD_MODE_F32C);
 * with tune != 0 its first run times the candidate tile sizes (64, 128) and
 * work orders on the actual inputs and keeps the fastest (remembered per size
 * list and mode for the rest of the process).  Inputs: all networks
 * concatenated as one packed 9 × sum(numSeg) device array (rows n1 n2 b,
 * network n in consecutive columns), ext (device, may be NULL); output the
 * forces in the same order (3 × 2 × sum(numSeg), device).  The first run with a
 * given (consts, segs, ext, force, stream) captures the work into a CUDA graph;
 * later runs with the same arguments replay it.  Runs are asynchronous on
 * `stream` (NULL = the plan's own stream).  A plan must not be run
 * concurrently with itself. */
typedef struct ddd_batch ddd_batch;
typedef struct ddd_batch_info_t {
  int tile;                /* chosen tile size (segments per side) */
  int order;               /* chosen work order: 0 network order, 1 largest networks first */
  int64_t work_items;      /* tile pairs in the chosen layout */
  int64_t total_segments;  /* sum of numSeg */
  int64_t graph_launches;  /* runs replayed from the captured graph */
  double tune_ms[4];       /* timings of (128, largest first), (128, network order), (64, …), (64, …); -1 if untuned */
} ddd_batch_info_t;
ddd_batch* ddd_batch_create(ddd_ctx* ctx, int64_t nNet, const int64_t* numSeg, int mode, int tune);
int ddd_batch_run(ddd_batch* b, const ddd_consts* k, const double* segs, const uint8_t* ext, double* force,
                  void* stream);
int ddd_batch_info(const ddd_batch* b, ddd_batch_info_t* out);
const char* ddd_batch_last_error(const ddd_batch* b);
void ddd_batch_destroy(ddd_batch* b);

/* Select / query the arithmetic mode of ctx (DDD_MODE_*).  No reference
 * counterpart: the reference's dispatch flags are parCPU / parGPU only. */
int ddd_set_mode(ddd_ctx* ctx, int mode);
int ddd_get_mode(const ddd_ctx* ctx);

/* Device memory for the all-pairs seg-seg partial sums of ctx, in bytes (0:
 * the default, 16 GiB).  The all-pairs forms keep 12 x 128 doubles per pair
 * of 128-segment tiles, nt(nt+1)/2 of them for nt tiles (6.4 GB at 131,072
 * segments, 184 GB at 700,000).  When they exceed the limit the pairs run in
 * bands of tile columns through a buffer of the limit's size (never below one
 * column, nt slots), each band's sums added to the output in band order: the
 * same deterministic result on every call, equal to the unbanded one to
 * rounding.  The idx forms keep 6 x 128 doubles per pair of a 128-row tile
 * of idx and a column tile; past the limit their rows run in chunks of whole
 * row tiles (at least one), with results unchanged bit for bit.  No reference
 * counterpart (the reference allocates per call).
 * ddd_get_partial_limit returns the limit in force. */
int ddd_set_partial_limit(ddd_ctx* ctx, int64_t bytes);
int64_t ddd_get_partial_limit(const ddd_ctx* ctx);

/* Tensor-core building block of the learned surrogate (no reference
 * counterpart): D[M x N] (FP32) = A[M x K] * B[N x K]^T with BF16 A and B,
 * row-major with K contiguous, on tcgen05 (accumulators in TMEM).  M a multiple
 * of 128, N a multiple of 16 in [16, 256], K a multiple of 16; device pointers,
 * 16-byte aligned.  Synchronous; DDD_ETIMEOUT if a bounded wait gave up. */
int ddd_tc_gemm_bf16(ddd_ctx* ctx, int M, int N, int K, const void* A, const void* B, float* D, void* stream);

/* Learned far-field surrogate (no reference counterpart: an extension of the
 * seg-seg force).  A pair's four node forces, in the pair's own frame and scaled by
 * mu4pi L_i L_j / R^2, are bilinear in the two Burgers vectors; a small MLP
 * (16 -> 128 -> 128 -> 128 -> 112, GELU, FP16 operands, FP32 accumulation) maps
 * the pair geometry to the 108 coefficients of that bilinear form, and an exact
 * contraction with (b_i.e_a)(b_j.e_c) gives the forces (features, frame and
 * contraction: csrc/surrogate.cuh).  It is trained on the GPU by this library's
 * kernels (tcgen05 GEMMs: FP16 forward, BF16 backward; Adam) on pairs whose
 * exact forces the FP64 kernel computes.  Per-sample rows (device, row-major):
 *   X  FP16 [P x 16]: the 8 geometric features' hi parts f16(f), then their
 *      lo parts f16(f - hi);
 *   Bp FP32 [P x 16]: the 9 Burgers-vector products (7 zero columns);
 *   T  FP32 [P x 16]: the 12 scaled exact node forces (4 zero columns).
 *   make_data: X, Bp, T of the pairs (i, j) in `pairs` (device int32, 2 x P:
 *     all i, then all j; 0-based columns of the packed 9 x n device array segs);
 *     F (device, P x 12, may be NULL) receives the exact forces.
 *   train: Adam over P samples in batches of B (P % B == 0, B % 128 == 0),
 *     cosine learning-rate decay; per-epoch mean loss into lossHistory.
 *   forward: O [P x 16] = the contracted outputs for P % 128 == 0 rows.
 *   grads: one forward and backward pass (no update): loss and the flat
 *     gradient (host), for checks against a CPU evaluation.
 *   params: copy the flat FP32 parameters to (set = 0) or from (set = 1) the host.
 * These calls are synchronous: each first waits for all work already queued on
 * the device (so inputs the caller is still producing on its own stream are
 * complete) and returns when its results are ready. */
typedef struct ddd_surrogate ddd_surrogate;
ddd_surrogate* ddd_surrogate_create(ddd_ctx* ctx, uint64_t seed);
void ddd_surrogate_destroy(ddd_surrogate* s);
int ddd_surrogate_num_params(void);
int ddd_surrogate_params(ddd_surrogate* s, float* host, int set);
int ddd_surrogate_make_data(ddd_ctx* ctx, const ddd_consts* k, const double* segs, int64_t n, const int32_t* pairs,
                            int64_t P, void* X, float* Bp, float* T, double* F);
int ddd_surrogate_train(ddd_surrogate* s, const void* X, const float* Bp, const float* T, int64_t P, int64_t B,
                        int epochs, float lr, float weightDecay, double* lossHistory);
int ddd_surrogate_forward(ddd_surrogate* s, const void* X, const float* Bp, int64_t P, float* O);
int ddd_surrogate_grads(ddd_surrogate* s, const void* X, const float* Bp, const float* T, int64_t B, double* loss,
                        float* grads);
/* Checkpoints (little-endian): "DDDGBSUR", u32 version 1, u32 parameter count,
 * f64 kappa, f64 nu, f64 aSq (the trust-region factor, Poisson ratio and core
 * radius squared the network was trained for), the f32 parameters, and the
 * CRC-32 (zlib) of everything before it.  load refuses a wrong magic, version,
 * size or CRC with DDD_EINVAL; kappa / nu / aSq may be NULL. */
int ddd_surrogate_save(ddd_surrogate* s, const char* path, double kappa, double nu, double aSq);
int ddd_surrogate_load(ddd_surrogate* s, const char* path, double* kappa, double* nu, double* aSq);

/* Seg-seg forces with the surrogate for far pairs: the same inputs and output
 * as ddd_segseg_force_device (packed 9 x ldSegs device segments n1, n2, b; ext
 * device bytes or NULL; force device 3 x 2 x numSeg), the same pair set as
 * calcSegSegForce (DislocationForces.jl:574-657, every unordered pair of active
 * segments), split into
 *   far pairs  R^2 >= kappa^2 max(L_i, L_j)^2 (R: midpoint separation, L:
 *              lengths) -> the network, fused tcgen05 kernel;
 *   near pairs (every other active pair) -> the exact pair force
 *              (calcSegSegForce's general or near-parallel branch; the general
 *              branch in the arithmetic of opts->exact_mode, strict FP64 by
 *              default), evaluated in full.
 * Segments are Morton-sorted by midpoint first, so near pairs fall in few tile
 * pairs; the result is returned in the caller's order and is deterministic.
 * Audit: a deterministic sample of about audit_fraction of the tile pairs is
 * also evaluated exactly on its far pairs.  From the network's errors there the
 * call estimates the node-force relative RMS error of the whole result
 * (sqrt(sum of squared slot errors / sampled fraction) / ||F||); when that
 * exceeds audit_tol, the whole call is recomputed with the exact FP64 kernel
 * (fallback = 1).
 * Far pairs may instead go to Gauss-Legendre quadrature of the non-singular
 * stress on both segments (far_mode 2 or 3, FP32): the endpoint differences
 * of the analytic form are replaced by integrals of their derivatives, which
 * do not cancel, so a far pair's force carries ~2e-7 relative error (3 points,
 * R >= 20 max(L_i, L_j)) where the analytic FP64 formula loses up to ~1e-3 to
 * cancellation; the near pass, audit and fallback are unchanged.
 * opts may be NULL (kappa 20, audit_fraction 0.01, audit_tol 1e-3, exact_mode
 * DDD_MODE_FP64, far_mode 0, kappa_two 0); rep may be
 * NULL.  Synchronous: the work is queued on `stream` (NULL: the surrogate's own
 * stream, after waiting for all work already queued on the device) and the
 * call returns when the forces are complete. */
typedef struct {
  double kappa;          /* trust-region factor R >= kappa max(L_i, L_j) for far pairs (> 0): the network's
                            training range sets it for far_mode 0 (the checkpoint's kappa); for the
                            3-point quadrature 10 suffices (at the FP32 noise level from 8), for the
                            2-point rule 20 */
  double audit_fraction; /* in [0, 1]; 0 disables the audit */
  double audit_tol;      /* bound of the estimated node-force relative RMS error; <= 0: no fallback */
  int exact_mode;        /* arithmetic of the exact passes (near, audit, fallback): DDD_MODE_FP64 (strict),
                            DDD_MODE_FP64_FAST, DDD_MODE_DF64 or DDD_MODE_F32C for the general branch */
  int far_mode;          /* 0: far pairs through the network; 2 or 3: through Gauss-Legendre quadrature with
                            that many points on each segment, in FP32 (no network involved: the surrogate's
                            weights and trained Poisson ratio are not used) */
  double kappa_two;      /* far_mode 3 only, >= 0: the far pass takes the 2-point rule for a warp's step of
                            32 pairs when each far pair in it lies beyond kappa_two max(L_i, L_j) (the
                            2-point rule's truncation, ~5e-6 per pair at 20 lengths, falls as (L/R)^4;
                            from 30 the node-force errors are those of 3 points); 0: always 3 points */
} ddd_sur_opts;
typedef struct {
  int64_t pairs_total;          /* unordered pairs of active segments */
  int64_t pairs_near_general;   /* near pairs, general branch (exact) */
  int64_t pairs_near_parallel;  /* near pairs, near-parallel branch (exact) */
  int64_t tiles_total;          /* tile pairs (128 x 128) of the network pass */
  int64_t tiles_near;           /* tile pairs visited by the exact near pass */
  int64_t tiles_audit;          /* tile pairs audited */
  double audit_rel_rms;         /* sqrt(sum |net - exact|^2 / sum |exact|^2) over audited tile sums */
  double audit_rel_max;         /* largest per-tile-pair relative error among them */
  double audit_node_rel_rms;    /* estimated node-force relative RMS error of the result */
  int fallback;                 /* 1 when the exact recomputation replaced the network's result */
  double ms_prep, ms_network, ms_audit, ms_near, ms_reduce, ms_total;
} ddd_sur_report;
int ddd_surrogate_force(ddd_surrogate* s, const ddd_consts* k, const double* segs, int64_t ldSegs,
                        const uint8_t* ext, int64_t numSeg, double* force, void* stream, const ddd_sur_opts* opts,
                        ddd_sur_report* rep);
/* The same with the network's own host arrays, in the layout of
 * ddd_segseg_force (calcSegSegForce's all-pairs form: coord 3 x coordCols,
 * bVec 3 x bVecCols, segIdx ldSegIdx x 3 1-based, extSeg per segment row or
 * NULL, force 3 x 2 x numSeg); validated like ddd_segseg_force. */
int ddd_surrogate_force_host(ddd_surrogate* s, const ddd_consts* k, const double* coord, int64_t coordCols,
                             const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                             const uint8_t* extSeg, int64_t numSeg, double* force, const ddd_sur_opts* opts,
                             ddd_sur_report* rep);
const char* ddd_surrogate_last_error(const ddd_surrogate* s);

/* Measurement utility (no reference counterpart): FP64 or FP32 FMA-pipe
 * throughput of this GPU in FLOP/s, measured with CUDA events over an
 * FMA-chain kernel filling every SM; the chain length is calibrated so each
 * timed run lasts about a second (clocks and power settle), best of three.
 * precision: 64 or 32. */
int ddd_probe_fma_peak(ddd_ctx* ctx, int precision, double* flops_per_s);

/* Failure-detection self-test (no reference counterpart: the reference has no
 * device code).  Runs, on the context's device, the bounded mbarrier wait that
 * the tensor-core kernels (ddd_tc_gemm_bf16, the surrogate's network pass) use
 * for every wait, in a one-warp kernel that issues no MMA and holds no tensor
 * memory: with arrive != 0 the barrier receives its arrival and the call
 * returns DDD_OK; with arrive == 0 nothing arrives, the wait gives up after
 * max_clocks SM clocks (1 <= max_clocks <= 2e9, about a second at most), the
 * kernel records the timeout and returns, and the call returns DDD_ETIMEOUT
 * with the context still usable.  Synchronous. */
int ddd_selftest_bounded_wait(ddd_ctx* ctx, long long max_clocks, int arrive);

#ifdef __cplusplus
}
#endif

#endif /* DDD_GB300_H */
