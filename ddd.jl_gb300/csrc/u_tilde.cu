// Displacements of the FE nodes from the dislocation network (calc_uTilde /
// calc_uTilde!, DislocationFEM.jl:355-581) by Barnett triangles
// (calcDisplacementDislocationTriangle!, :600-707; Bromage & Tarleton 2018),
// strict FP64 (compiled with --fmad=false; the host part with
// -ffp-contract=off).
//
// Host: one pass over the segments in order, as the reference's loop, decides
// which triangles each segment contributes: none for a segment joining a
// surface node to an external one (it only records that connection), one full
// triangle (A, B, C) for an internal segment, five solid-angle triangles
// through the points the nodes were projected out from for a segment with an
// external node.  Internal segments are passed by index (the GPU reads their
// nodes), the projected triangles explicitly.
// GPU: tri_prep builds every triangle's vertices and safeNorm'ed edges;
// u_field gives each point one thread that sums the triangles in the
// reference's order, triangles streamed through shared memory.  Its log and
// atan are the integer-pipe functions of intmath_f64.cuh (within 0.51 ulp);
// acos and tan are CUDA's.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include <limits>
#include <vector>

#include "ddd_internal.h"
#include "intmath_f64.cuh"

namespace ddd {
namespace {

constexpr int PT = 128;   // points per CTA of the field kernel
constexpr int TCH = 32;   // triangles per shared-memory chunk
constexpr int TROW = kUTriRows;  // doubles per triangle (layout below)

struct V {
  double x, y, z;
};
__host__ __device__ __forceinline__ V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ V operator*(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ V cross(V a, V b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V ld3(const double* a, int64_t n) { return {a[3 * n], a[3 * n + 1], a[3 * n + 2]}; }

// safeNorm (Misc.jl:289-300): |x| (eps when below eps) and x normalised as
// inv(norm(x)) * x (or zero).
__device__ __forceinline__ double safe_norm(V& x) {
  const double n = sqrt(dot(x, x));
  if (n > DBL_EPSILON) {
    const double inv = 1.0 / n;
    x = {inv * x.x, inv * x.y, inv * x.z};
    return n;
  }
  x = {0.0, 0.0, 0.0};
  return DBL_EPSILON;
}
__device__ __forceinline__ double clamp11(double x) { return x > 1.0 ? 1.0 : (x < -1.0 ? -1.0 : x); }
__device__ __forceinline__ double jl_sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : x); }
// Julia's max(x, 0): negatives and -0.0 give +0.0; NaN stays NaN.
__device__ __forceinline__ double jl_max0(double x) { return isnan(x) ? x : ((x < 0.0 || signbit(x)) ? 0.0 : x); }

// Triangle rows (SoA, T columns): 0-2 A, 3-5 B, 6-8 C, 9-11 b, 12-14 AB,
// 15-17 BC, 18-20 CA, 21 full (1) or solid angle only (0), 22 link flags:
// +1 when C is the closure point, +2 when A is the previous triangle's B (the
// field kernel then reuses R = C - P and the previous R_B, bit for bit), +4 /
// +8 when the BC / CA edge term cancels against the next / previous triangle's
// (the reformulated kernel skips both), 23-31 b x AB, b x BC, b x CA.
// order[t] >= 0: internal segment order[t] (A, B its nodes, C the closure
// point); order[t] < 0: explicit triangle -1 - order[t] (rows A, B, C, b of
// explicit, 13 doubles each, the last the full flag).
__global__ void tri_prep(const int64_t* __restrict__ order, int64_t nTri, const double* __restrict__ coord,
                         const int64_t* __restrict__ links, const double* __restrict__ bVec, V Cl,
                         const double* __restrict__ explicitTri, double* __restrict__ tri) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nTri) return;
  V A, B, C, b;
  double full;
  const int64_t o = order[t];
  if (o >= 0) {
    A = ld3(coord, links[2 * o] - 1);
    B = ld3(coord, links[2 * o + 1] - 1);
    C = Cl;
    b = ld3(bVec, o);
    full = 1.0;
  } else {
    const double* e = explicitTri + 13 * (-1 - o);
    A = {e[0], e[1], e[2]};
    B = {e[3], e[4], e[5]};
    C = {e[6], e[7], e[8]};
    b = {e[9], e[10], e[11]};
    full = e[12];
  }
  V AB = B - A, BC = C - B, CA = A - C;
  safe_norm(AB);
  safe_norm(BC);
  safe_norm(CA);
  const bool closure = C.x == Cl.x && C.y == Cl.y && C.z == Cl.z;
  double link = closure ? 1.0 : 0.0;
  // A pair of consecutive full triangles closed on C with the same b, the
  // second starting where the first ends, share the edge (B_t, C) in opposite
  // directions: its g terms are exact negatives and its f terms cancel
  // (both logs reduce to the distance from P to the same line).
  auto node_of = [&](int64_t tt, int which, V& X, V& bb, bool& isFull, bool& isClosure) {
    const int64_t o = order[tt];
    if (o >= 0) {
      X = ld3(coord, links[2 * o + which] - 1);
      bb = ld3(bVec, o);
      isFull = true;
      isClosure = true;
    } else {
      const double* e = explicitTri + 13 * (-1 - o);
      X = {e[3 * which], e[3 * which + 1], e[3 * which + 2]};
      bb = {e[9], e[10], e[11]};
      isFull = e[12] != 0.0;
      isClosure = e[6] == Cl.x && e[7] == Cl.y && e[8] == Cl.z;
    }
  };
  auto same = [](V x, V y) { return x.x == y.x && x.y == y.y && x.z == y.z; };
  if (t > 0) {  // the previous triangle's B
    V Bp, bp;
    bool fp, cp;
    node_of(t - 1, 1, Bp, bp, fp, cp);
    if (same(Bp, A)) {
      link += 2.0;
      if (fp && cp && full != 0.0 && closure && same(bp, b)) link += 8.0;  // CA cancels the previous BC
    }
  }
  if (t + 1 < nTri) {  // the next triangle's A
    V An, bn;
    bool fn, cn;
    node_of(t + 1, 0, An, bn, fn, cn);
    if (same(An, B) && fn && cn && full != 0.0 && closure && same(bn, b)) link += 4.0;  // BC cancels the next CA
  }
  const V bAB = cross(b, AB), bBC = cross(b, BC), bCA = cross(b, CA);
  const double r[TROW] = {A.x,   A.y,   A.z,   B.x,   B.y,   B.z,   C.x,   C.y,   C.z,   b.x,   b.y,
                          b.z,   AB.x,  AB.y,  AB.z,  BC.x,  BC.y,  BC.z,  CA.x,  CA.y,  CA.z,  full,
                          link,  bAB.x, bAB.y, bAB.z, bBC.x, bBC.y, bBC.z, bCA.x, bCA.y, bCA.z};
#pragma unroll
  for (int k = 0; k < TROW; ++k) tri[k * nTri + t] = r[k];
}

// What a point's previous triangle leaves for the next one (valid once a
// triangle of the thread's range has been evaluated).
struct Chain {
  V RB;
  double RBn, tb;
  bool closure, valid;
};

// One triangle at point P (calcDisplacementDislocationTriangle!, both forms).
// RCc / RCcn: C - P safeNorm'ed for the closure point; ch: the previous
// triangle's R_B, |R_B| and acos(R_B . R_C) (valid when the flags say so).
__device__ __forceinline__ V tri_u(const double* s, double omNuInv8pi, double om2NuOmNuInv8pi, V P, V RCc,
                                   double RCcn, Chain& ch) {
  const V A = {s[0], s[1], s[2]}, B = {s[3], s[4], s[5]}, C = {s[6], s[7], s[8]}, b = {s[9], s[10], s[11]};
  const V AB = {s[12], s[13], s[14]}, BC = {s[15], s[16], s[17]}, CA = {s[18], s[19], s[20]};
  const int link = (int)s[22];
  const bool closure = link & 1, chained = (link & 2) && ch.valid;
  V RA, RB = B - P, RC;
  double RAn, RCn;
  if (chained) {
    RA = ch.RB;
    RAn = ch.RBn;
  } else {
    RA = A - P;
    RAn = safe_norm(RA);
  }
  const double RBn = safe_norm(RB);
  if (closure) {
    RC = RCc;
    RCn = RCcn;
  } else {
    RC = C - P;
    RCn = safe_norm(RC);
  }
  const double RAdRB = clamp11(dot(RA, RB)), RBdRC = clamp11(dot(RB, RC)), RCdRA = clamp11(dot(RC, RA));
  // RC . RA here equals the previous triangle's RB . RC term by term.
  const double ta = acos(RAdRB), tb = acos(RBdRC), tc = (chained && closure && ch.closure) ? ch.tb : acos(RCdRA);
  ch = {RB, RBn, tb, closure, true};
  const double th = (ta + tb + tc) / 2.0;
  const double factor =
      jl_max0(tan(th / 2.0) * tan((th - ta) / 2.0) * tan((th - tb) / 2.0) * tan((th - tc) / 2.0));
  double omega = 4.0 * im::atan(sqrt(factor));
  omega = -jl_sign(dot(RA, cross(CA, AB))) * omega;
  const double fourPi = 4.0 * 3.141592653589793;
  V u = {-b.x * omega / fourPi, -b.y * omega / fourPi, -b.z * omega / fourPi};
  if (s[21] == 0.0) return u;
  const V bAB = {s[23], s[24], s[25]}, bBC = {s[26], s[27], s[28]}, bCA = {s[29], s[30], s[31]};
  const V fAB = bAB * im::log((RBn / RAn) * (1.0 + dot(RB, AB)) / (1.0 + dot(RA, AB)));
  const V fBC = bBC * im::log((RCn / RBn) * (1.0 + dot(RC, BC)) / (1.0 + dot(RB, BC)));
  const V fCA = bCA * im::log((RAn / RCn) * (1.0 + dot(RA, CA)) / (1.0 + dot(RC, CA)));
  const double sAB = dot(b, cross(RA, RB)), sBC = dot(b, cross(RB, RC)), sCA = dot(b, cross(RC, RA));
  const V vAB = RA + RB, vBC = RB + RC, vCA = RC + RA;
  const double dAB = 1.0 + RAdRB, dBC = 1.0 + RBdRC, dCA = 1.0 + RCdRA;
  const V gAB = {sAB * vAB.x / dAB, sAB * vAB.y / dAB, sAB * vAB.z / dAB};
  const V gBC = {sBC * vBC.x / dBC, sBC * vBC.y / dBC, sBC * vBC.z / dBC};
  const V gCA = {sCA * vCA.x / dCA, sCA * vCA.y / dCA, sCA * vCA.z / dCA};
  const V fs = fAB + fBC + fCA, gs = gAB + gBC + gCA;
  return u - V{om2NuOmNuInv8pi * fs.x, om2NuOmNuInv8pi * fs.y, om2NuOmNuInv8pi * fs.z} +
         V{omNuInv8pi * gs.x, omNuInv8pi * gs.y, omNuInv8pi * gs.z};
}

// Block (x, y): points x * PT.., triangles [y * chunk, (y + 1) * chunk), in
// order; partial sums to part[y][p] (the reduce kernel adds them in y order).
__global__ void __launch_bounds__(PT) u_field(const double* __restrict__ tri, int64_t nTri, int64_t chunk,
                                              const double* __restrict__ points, int64_t M, double omNuInv8pi,
                                              double om2NuOmNuInv8pi, V Cl, double* __restrict__ part) {
  __shared__ double sm[TCH][TROW + 1];
  const int64_t p = blockIdx.x * (int64_t)PT + threadIdx.x;
  const bool on = p < M;
  const V P = on ? ld3(points, p) : V{0.0, 0.0, 0.0};
  V RCc = V{Cl.x, Cl.y, Cl.z} - P;
  const double RCcn = safe_norm(RCc);
  Chain ch = {{0.0, 0.0, 0.0}, 0.0, 0.0, false, false};
  V acc = {0.0, 0.0, 0.0};
  const int64_t tBeg = blockIdx.y * chunk, tEnd = tBeg + chunk < nTri ? tBeg + chunk : nTri;
  for (int64_t t0 = tBeg; t0 < tEnd; t0 += TCH) {
    const int n = (int)(tEnd - t0 < TCH ? tEnd - t0 : TCH);
    __syncthreads();
    for (int q = threadIdx.x; q < n * TROW; q += PT) {
      const int tt = q % n, k = q / n;
      sm[tt][k] = tri[k * nTri + t0 + tt];
    }
    __syncthreads();
    if (on)
      for (int tt = 0; tt < n; ++tt) acc = acc + tri_u(sm[tt], omNuInv8pi, om2NuOmNuInv8pi, P, RCc, RCcn, ch);
  }
  if (on) {
    double* u = part + 3 * (blockIdx.y * M + p);
    u[0] = acc.x;
    u[1] = acc.y;
    u[2] = acc.z;
  }
}

// u[p] = sum over k of part[k][p], k in order.
__global__ void u_reduce(const double* __restrict__ part, int64_t K, int64_t M, double* __restrict__ u) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= 3 * M) return;
  double s = part[q];
  for (int64_t k = 1; k < K; ++k) s += part[k * 3 * M + q];
  u[q] = s;
}

// ---- host: the segment pass of _calc_uTilde! -------------------------------

struct HV {
  double x, y, z;
};
inline HV hadd(HV a, HV b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline HV hsub(HV a, HV b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline HV hmul(HV a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double hdot(HV a, HV b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline HV hcol(const double* a, int64_t n) { return {a[3 * n], a[3 * n + 1], a[3 * n + 2]}; }

struct HostMesh {
  HV C, lo, hi;
  double tol;
  const double* faceNorm;
  const double* faceMidPt;
  int64_t nF;
  const double* normals;
  int64_t nN;
  bool inside(HV p) const {
    return p.x >= lo.x - tol && p.x <= hi.x + tol && p.y >= lo.y - tol && p.y <= hi.y + tol && p.z >= lo.z - tol &&
           p.z <= hi.z + tol;
  }
};

// findIntersectVolume (DislocationTopologySpecial.jl:7-34) with
// linePlaneIntersect (Misc.jl:223-235).
double nearest_face_hit(const HostMesh& m, HV dir, HV from, HV& hit) {
  double best = std::numeric_limits<double>::infinity();
  hit = {0.0, 0.0, 0.0};
  for (int64_t f = 0; f < m.nF; ++f) {
    const HV n = hcol(m.faceNorm, f), mid = hcol(m.faceMidPt, f);
    const double den = hdot(dir, n);
    if (den == 0.0) continue;
    const double d = hdot(hsub(mid, from), n) / den;
    const HV x = hadd(from, hmul(dir, d));
    if (std::isinf(x.x) || std::isinf(x.y) || std::isinf(x.z) || !m.inside(x)) continue;
    const HV r = hsub(x, from);
    const double s = r.x * r.x + r.y * r.y + r.z * r.z;
    const double prev = best;
    best = s < prev ? s : prev;
    if (best < prev) hit = x;
  }
  return best;
}

}  // namespace

cudaError_t u_tilde_compute(const UTildeArgs& a, double* u, cudaEvent_t e0, cudaEvent_t e1, cudaStream_t st,
                            UTildeScratch& S) {
  const HostMesh m{{a.C[0], a.C[1], a.C[2]}, {a.lo[0], a.lo[1], a.lo[2]}, {a.hi[0], a.hi[1], a.hi[2]}, a.tol,
                   a.faceNorm, a.faceMidPt, a.numFaces, a.normals, a.numNormals};
  auto srf = [](int32_t l) { return l == 3 || l == 4; };  // srfMobDln, srfFixDln
  constexpr int32_t kExt = 5;                             // extDln
  std::vector<int64_t>& order = S.order;
  std::vector<double>& ex = S.explicitTri;
  order.clear();
  ex.clear();
  std::vector<int64_t> surfCon((size_t)a.numNode, 0);
  auto emit = [&](HV A, HV B, HV C, HV b) {
    const double r[13] = {A.x, A.y, A.z, B.x, B.y, B.z, C.x, C.y, C.z, b.x, b.y, b.z, 0.0};
    order.push_back(-1 - (int64_t)(ex.size() / 13));
    ex.insert(ex.end(), r, r + 13);
  };
  for (int64_t i = 0; i < a.numSeg; ++i) {
    const int64_t n1 = a.links[2 * i], n2 = a.links[2 * i + 1];
    const int32_t l1 = a.label[n1 - 1], l2 = a.label[n2 - 1];
    if (srf(l1) && l2 == kExt) {
      surfCon[n2 - 1] = n1;
      continue;
    }
    if (srf(l2) && l1 == kExt) {
      surfCon[n1 - 1] = n2;
      continue;
    }
    if (l1 != kExt && l2 != kExt) {
      order.push_back(i);
      continue;
    }
    const HV A = hcol(a.coord, n1 - 1), B = hcol(a.coord, n2 - 1), b = hcol(a.bVec, i);
    const double inf = std::numeric_limits<double>::infinity();
    double dA = inf, dB = inf, dC = inf;
    HV pA = {inf, inf, inf}, pB = {inf, inf, inf};
    for (int64_t j = 0; j < m.nN; ++j) {
      const HV dir = hcol(m.normals, j);
      HV hA, hB;
      const double sA = nearest_face_hit(m, dir, A, hA);
      const double sB = nearest_face_hit(m, dir, B, hB);
      if (sA < dA) dA = sA, pA = hA;
      if (sB < dB) dB = sB, pB = hB;
    }
    // No face hit (projected out of an edge or a corner): step through the
    // face planes towards the centroid; the distance record dC is shared by
    // both nodes' walks, as in the reference.
    auto walk = [&](HV P) {
      for (int64_t f = 0; f < m.nF; ++f) {
        const HV n = hcol(m.faceNorm, f);
        const double q = hdot(hadd(P, hcol(m.faceMidPt, f)), n);
        const HV x = hsub(P, hmul(n, std::sqrt(q * q)));
        const HV r = hsub(x, m.C);
        const double dc = std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
        if (dc <= dC) dC = dc, P = x;
      }
      return P;
    };
    if (std::isinf(dA)) pA = walk(A);
    if (std::isinf(dB)) pB = walk(B);
    if (surfCon[n1 - 1] != 0) pA = hcol(a.coord, surfCon[n1 - 1] - 1);
    if (surfCon[n2 - 1] != 0) pB = hcol(a.coord, surfCon[n2 - 1] - 1);
    const HV Cp = {(A.x + pB.x) / 2.0, (A.y + pB.y) / 2.0, (A.z + pB.z) / 2.0};
    emit(pA, pB, m.C, b);
    emit(pA, A, Cp, b);
    emit(A, B, Cp, b);
    emit(B, pB, Cp, b);
    emit(pB, pA, Cp, b);
  }
  const int64_t nTri = (int64_t)order.size();
  S.lastTriangles = nTri;
  cudaError_t e;
  if ((e = S.order_d.ensure((size_t)std::max<int64_t>(nTri, 1) * 8)) != cudaSuccess) return e;
  if ((e = S.ex_d.ensure(std::max<size_t>(ex.size(), 1) * 8)) != cudaSuccess) return e;
  if ((e = S.tri_d.ensure((size_t)std::max<int64_t>(nTri, 1) * TROW * 8)) != cudaSuccess) return e;
  // Triangle chunks of at least 256 triangles; one chunk keeps each point's
  // sum strictly sequential.
  if (!S.sms) {
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&S.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  }
  int& occ = a.fast ? S.occFast : S.occStrict;
  if (!occ) {
    if (a.fast)
      occ = u_field_fast_blocks_per_sm();
    else if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, u_field, PT, 0)) != cudaSuccess)
      return e;
    occ = std::max(occ, 1);
  }
  // As many chunks as fit the resident slots in one wave (equal chunks then
  // finish together); many points alone fill the GPU with one chunk.
  const int64_t bx = (a.numPoints + PT - 1) / PT;
  const int64_t want = std::max<int64_t>(1, (int64_t)S.sms * occ / std::max<int64_t>(bx, 1));
  const int64_t K = std::max<int64_t>(1, std::min<int64_t>({want, (nTri + 255) / 256, 65535}));
  const int64_t chunk = std::max<int64_t>(1, (nTri + K - 1) / K);
  S.lastChunks = K;
  if ((e = S.u_d.ensure((size_t)std::max<int64_t>(a.numPoints, 1) * 3 * 8)) != cudaSuccess) return e;
  if ((e = S.part_d.ensure((size_t)std::max<int64_t>(a.numPoints, 1) * 3 * 8 * K)) != cudaSuccess) return e;
  if (nTri > 0 &&
      (e = cudaMemcpyAsync(S.order_d.p, order.data(), (size_t)nTri * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if (!ex.empty() &&
      (e = cudaMemcpyAsync(S.ex_d.p, ex.data(), ex.size() * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if (e0 && (e = cudaEventRecord(e0, st)) != cudaSuccess) return e;
  if (nTri > 0) {
    tri_prep<<<(int)((nTri + 255) / 256), 256, 0, st>>>((const int64_t*)S.order_d.p, nTri, a.coordDev, a.linksDev,
                                                        a.bVecDev, V{a.C[0], a.C[1], a.C[2]},
                                                        (const double*)S.ex_d.p, (double*)S.tri_d.p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (a.numPoints > 0 && a.fast) {
    if ((e = launch_u_field_fast((const double*)S.tri_d.p, nTri, chunk, K, a.pointsDev, a.numPoints, a.omNuInv8pi,
                                 a.om2NuOmNuInv8pi, a.C, (double*)S.part_d.p, st)) != cudaSuccess)
      return e;
  } else if (a.numPoints > 0) {
    u_field<<<dim3((unsigned)bx, (unsigned)K), PT, 0, st>>>((const double*)S.tri_d.p, nTri, chunk, a.pointsDev,
                                                            a.numPoints, a.omNuInv8pi, a.om2NuOmNuInv8pi,
                                                            V{a.C[0], a.C[1], a.C[2]}, (double*)S.part_d.p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (a.numPoints > 0) {
    u_reduce<<<(int)((3 * a.numPoints + 255) / 256), 256, 0, st>>>((const double*)S.part_d.p, K, a.numPoints,
                                                                   (double*)S.u_d.p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (e1 && (e = cudaEventRecord(e1, st)) != cudaSuccess) return e;
  if (a.numPoints > 0 &&
      (e = cudaMemcpyAsync(u, S.u_d.p, (size_t)a.numPoints * 3 * 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  return cudaStreamSynchronize(st);
}

}  // namespace ddd
