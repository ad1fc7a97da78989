// Displacements of the FE nodes from the dislocation network (calc_uTilde /
// calc_uTilde!, DislocationFEM.jl:354-632) by Barnett triangles
// (calcDisplacementDislocationTriangle!, :634-751; Bromage & Tarleton 2018),
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
// reference's order, triangles streamed through shared memory.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include <limits>
#include <vector>

#include "ddd_internal.h"

namespace ddd {
namespace {

constexpr int PT = 128;   // points per CTA of the field kernel
constexpr int TCH = 32;   // triangles per shared-memory chunk
constexpr int TROW = 22;  // doubles per triangle: A, B, C, b, AB, BC, CA, full flag

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
// 15-17 BC, 18-20 CA, 21 full (1) or solid angle only (0).
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
  const double r[TROW] = {A.x,  A.y,  A.z,  B.x,  B.y,  B.z,  C.x,  C.y,  C.z,  b.x,  b.y,
                          b.z,  AB.x, AB.y, AB.z, BC.x, BC.y, BC.z, CA.x, CA.y, CA.z, full};
#pragma unroll
  for (int k = 0; k < TROW; ++k) tri[k * nTri + t] = r[k];
}

// One triangle at point P (calcDisplacementDislocationTriangle!, both forms).
__device__ __forceinline__ V tri_u(const double* s, double omNuInv8pi, double om2NuOmNuInv8pi, V P) {
  const V A = {s[0], s[1], s[2]}, B = {s[3], s[4], s[5]}, C = {s[6], s[7], s[8]}, b = {s[9], s[10], s[11]};
  const V AB = {s[12], s[13], s[14]}, BC = {s[15], s[16], s[17]}, CA = {s[18], s[19], s[20]};
  V RA = A - P, RB = B - P, RC = C - P;
  const double RAn = safe_norm(RA), RBn = safe_norm(RB), RCn = safe_norm(RC);
  const double RAdRB = clamp11(dot(RA, RB)), RBdRC = clamp11(dot(RB, RC)), RCdRA = clamp11(dot(RC, RA));
  const double ta = acos(RAdRB), tb = acos(RBdRC), tc = acos(RCdRA);
  const double th = (ta + tb + tc) / 2.0;
  const double factor =
      jl_max0(tan(th / 2.0) * tan((th - ta) / 2.0) * tan((th - tb) / 2.0) * tan((th - tc) / 2.0));
  double omega = 4.0 * atan(sqrt(factor));
  omega = -jl_sign(dot(RA, cross(CA, AB))) * omega;
  const double fourPi = 4.0 * 3.141592653589793;
  V u = {-b.x * omega / fourPi, -b.y * omega / fourPi, -b.z * omega / fourPi};
  if (s[21] == 0.0) return u;
  const V fAB = cross(b, AB) * log((RBn / RAn) * (1.0 + dot(RB, AB)) / (1.0 + dot(RA, AB)));
  const V fBC = cross(b, BC) * log((RCn / RBn) * (1.0 + dot(RC, BC)) / (1.0 + dot(RB, BC)));
  const V fCA = cross(b, CA) * log((RAn / RCn) * (1.0 + dot(RA, CA)) / (1.0 + dot(RC, CA)));
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

__global__ void __launch_bounds__(PT) u_field(const double* __restrict__ tri, int64_t nTri,
                                              const double* __restrict__ points, int64_t M, double omNuInv8pi,
                                              double om2NuOmNuInv8pi, double* __restrict__ u) {
  __shared__ double sm[TCH][TROW + 1];
  const int64_t p = blockIdx.x * (int64_t)PT + threadIdx.x;
  const bool on = p < M;
  const V P = on ? ld3(points, p) : V{0.0, 0.0, 0.0};
  V acc = {0.0, 0.0, 0.0};
  for (int64_t t0 = 0; t0 < nTri; t0 += TCH) {
    const int n = (int)(nTri - t0 < TCH ? nTri - t0 : TCH);
    __syncthreads();
    for (int q = threadIdx.x; q < n * TROW; q += PT) {
      const int tt = q % n, k = q / n;
      sm[tt][k] = tri[k * nTri + t0 + tt];
    }
    __syncthreads();
    if (on)
      for (int tt = 0; tt < n; ++tt) acc = acc + tri_u(sm[tt], omNuInv8pi, om2NuOmNuInv8pi, P);
  }
  if (on) {
    u[3 * p] = acc.x;
    u[3 * p + 1] = acc.y;
    u[3 * p + 2] = acc.z;
  }
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
  if ((e = S.u_d.ensure((size_t)std::max<int64_t>(a.numPoints, 1) * 3 * 8)) != cudaSuccess) return e;
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
  if (a.numPoints > 0) {
    u_field<<<(int)((a.numPoints + PT - 1) / PT), PT, 0, st>>>((const double*)S.tri_d.p, nTri, a.pointsDev,
                                                               a.numPoints, a.omNuInv8pi, a.om2NuOmNuInv8pi,
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
