// BCC mobility (dlnMobility / dlnMobility!, DislocationMobility.jl:16-341),
// strict FP64 (compiled with --fmad=false): for each node of the list, the
// forces of its connected segments are summed and a 3×3 drag tensor is built
// from each connection's geometry (edge / climb / line drags, and for
// screw-type Burgers vectors the screw glide and climb drags of Arsenlis et al.
// 2007, eqn 112); the velocity solves drag · v = force (Cramer's rule).
//
// One thread per node; a node's connections are at most maxConnect (4 in the
// reference), so the kernel is a short gather and O(1) arithmetic per node.
#include <cfloat>
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_f64.cuh"

namespace ddd {
namespace {

struct M3 {
  double a[3][3];
};

// M += scale * (diag I + (s x) y'): the reference's `scale * (ξ I + (ξ' - ξ) * x ⊗ y)`.
__device__ __forceinline__ void add_outer(M3& M, double s, D3 x, D3 y, double scale, double diag) {
  const double sx[3] = {s * x.x, s * x.y, s * x.z};
  const double yy[3] = {y.x, y.y, y.z};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) M.a[i][j] = M.a[i][j] + scale * ((i == j ? diag : 0.0) + sx[i] * yy[j]);
}

__device__ __forceinline__ D3 solve3(const M3& M, D3 f) {
  const double(&a)[3][3] = M.a;
  const double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  const double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
  const double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  const double det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
  return {(c00 * f.x + (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * f.y + (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * f.z) /
              det,
          (c01 * f.x + (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * f.y + (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * f.z) /
              det,
          (c02 * f.x + (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * f.y + (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * f.z) /
              det};
}

__global__ void mobility_bcc_f64(MobK P, const double* __restrict__ coord, const double* __restrict__ bVec,
                                 const int64_t* __restrict__ links, const int64_t* __restrict__ conn, int64_t ldConn,
                                 const double* __restrict__ segForce, const int64_t* __restrict__ rows, int64_t n,
                                 double* __restrict__ nodeForce, double* __restrict__ nodeVel) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int64_t node1 = rows ? rows[q] : q;
  const double eps = DBL_EPSILON;
  const double sqrtBType = sqrt(eps);
  M3 drag;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) drag.a[i][j] = 0.0;
  D3 force = {0, 0, 0};
  const D3 x1 = {coord[3 * node1], coord[3 * node1 + 1], coord[3 * node1 + 2]};
  const int64_t numConnect = conn[ldConn * node1];
  for (int64_t c = 1; c <= numConnect; ++c) {
    const int64_t link = conn[ldConn * node1 + 2 * c - 1] - 1;
    const int64_t colLink = conn[ldConn * node1 + 2 * c];
    const int64_t node2 = links[2 * link + (3 - colLink) - 1] - 1;
    D3 t = D3{coord[3 * node2], coord[3 * node2 + 1], coord[3 * node2 + 2]} - x1;
    const double nT = norm(t);
    if (nT < eps) continue;  // zero-length segment
    const double tN = 1.0 / nT;
    t = t * tN;
    const double* fs = segForce + 6 * link + 3 * (colLink - 1);
    D3 f = {fs[0], fs[1], fs[2]};
    if (norm(f) * tN < P.sigmaPN) f = {0, 0, 0};  // below the Peierls-Nabarro stress
    force = force + f;
    D3 b = {bVec[3 * link], bVec[3 * link + 1], bVec[3 * link + 2]};
    const double nB = norm(b);
    const double ab[3] = {fabs(b.x), fabs(b.y), fabs(b.z)};
    const double mn = fmin(fmin(ab[0], ab[1]), ab[2]);
    int type1 = 0, type2 = 0, type3 = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double r = ab[k] / mn;
      type1 += fabs(1.0 - r) < sqrtBType;
      type2 += fabs(2.0 - r) < sqrtBType;
      type3 += fabs(3.0 - r) < sqrtBType;
    }
    const bool screw = 1.0 - nB < sqrtBType;
    b = {b.x / nB, b.y / nB, b.z / nB};
    const double nBnT_2 = nB * nT / 2.0;
    if (!((type1 == 3 && screw) || (type1 == 2 && type2 == 1 && screw) ||
          (type1 == 1 && type2 == 1 && type3 == 1 && screw))) {
      add_outer(drag, P.line - P.climb, t, t, nBnT_2, P.climb);
      continue;
    }
    const double tDb = dot(t, b);
    const double cosSq = tDb * tDb;
    const double sinSq = 1.0 - cosSq;
    add_outer(drag, P.line - P.screw, t, t, nBnT_2, P.screw);
    if (sinSq < eps) continue;  // pure screw
    const double sq = sqrt(sinSq);
    const D3 bt = cross(b, t);
    const D3 p = {bt.x / sq, bt.y / sq, bt.z / sq};
    const D3 qv = cross(p, t);
    const double screwSq = P.screw * P.screw;
    const double glide = 1.0 / sqrt(sinSq / (P.edge * P.edge) + cosSq / screwSq);
    const double climb = sqrt(sinSq * (P.climb * P.climb) + cosSq * screwSq);
    const double gq[3] = {(glide - P.screw) * qv.x, (glide - P.screw) * qv.y, (glide - P.screw) * qv.z};
    const double cp[3] = {(climb - P.screw) * p.x, (climb - P.screw) * p.y, (climb - P.screw) * p.z};
    const double qq[3] = {qv.x, qv.y, qv.z}, pp[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) drag.a[i][j] = drag.a[i][j] + nBnT_2 * (gq[i] * qq[j] + cp[i] * pp[j]);
  }
  const D3 v = solve3(drag, force);
  nodeForce[3 * q] = force.x;
  nodeForce[3 * q + 1] = force.y;
  nodeForce[3 * q + 2] = force.z;
  nodeVel[3 * q] = v.x;
  nodeVel[3 * q + 1] = v.y;
  nodeVel[3 * q + 2] = v.z;
}

}  // namespace

cudaError_t launch_mobility_bcc(const MobK& P, const double* coord, const double* bVec, const int64_t* links,
                                const int64_t* conn, int64_t ldConn, const double* segForce, const int64_t* rows,
                                int64_t n, double* nodeForce, double* nodeVel, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  mobility_bcc_f64<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(P, coord, bVec, links, conn, ldConn, segForce, rows, n,
                                                               nodeForce, nodeVel);
  return cudaGetLastError();
}

}  // namespace ddd
