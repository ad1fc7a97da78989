// Collision detection (detectCollision, DislocationTopologyCollision.jl:1-221)
// and minimumDistance (Misc.jl:314-367), strict FP64 (compiled with
// --fmad=false, every multiply and add rounded as in the reference).
//
// The reference scans every pair of segments serially and keeps the pair with
// the largest 1/distSq among those closer than collisionDist and approaching;
// a later pair replaces the kept one only when strictly better, so ties go to
// the first pair in (i, j) order.  Here:
//   * hinge pass: one thread per node, its pairs of connections in the
//     reference's order (including the swap that keeps link1 on the longer
//     connection for the rest of the k loop);
//   * two-line pass: segments Morton-sorted into 128-segment tiles; a
//     persistent kernel takes the tile pairs from a counter, rejects a pair of tiles whose
//     bounding boxes are farther apart than collisionDist and then, per pair of
//     segments, rejects by bounding spheres in FP32 (radii rounded outward with
//     a 1e-5 relative and 1e-5 * max|coord| margin, so no pair whose FP64
//     distance is below collisionDist is ever rejected); survivors go through
//     the reference's filters and minimumDistance in FP64, the segment with the
//     lower index taking the reference's "i" role;
//   * the reference returns L1, L2 of the LAST pair its loops evaluated (its
//     loop variables), not of the reported pair: a third kernel finds, per row
//     i, the largest j that passes the filters, and the last pair is the
//     largest such (i, j);
//   * one block combines the per-block results with the reference's order
//     (largest key, then the smallest index), deterministic, no atomics.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "ddd_internal.h"

namespace ddd {
namespace {

constexpr int T = 128;        // segments per tile and threads per CTA of the pair kernel
constexpr int RB = 256;       // threads per CTA of the per-node / per-row kernels
constexpr double kEps = DBL_EPSILON;

struct V {
  double x, y, z;
};
__device__ __forceinline__ V ld3(const double* a, int64_t n) { return {a[3 * n], a[3 * n + 1], a[3 * n + 2]}; }
__device__ __forceinline__ V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V operator*(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V twice(V a) { return {2.0 * a.x, 2.0 * a.y, 2.0 * a.z}; }
// StaticArrays' dot: (x1*y1 + x2*y2) + x3*y3.
__device__ __forceinline__ double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double clamp01(double x) { return x > 1.0 ? 1.0 : (x < 0.0 ? 0.0 : x); }

struct MD {
  double distSq, dDistSqDt, L1, L2;
};

// minimumDistance(x0, x1, y0, y1, vx0, vx1, vy0, vy1), Misc.jl:314-367, with its
// operation order; the near-parallel branch keeps L1 = floor(idx / 2).
__device__ MD min_dist(V x0, V x1, V y0, V y1, V vx0, V vx1, V vy0, V vy1) {
  const V seg1 = x1 - x0, seg2 = y1 - y0, vseg1 = vx1 - vx0, vseg2 = vy1 - vy0;
  const double A = dot(seg1, seg1);
  const double B = dot(twice(seg1), x0 - y0);
  const double C = dot(twice(seg1), seg2);
  const double D = dot(twice(seg2), y0 - x0);
  const double E = dot(seg2, seg2);
  const double G = C * C - 4.0 * A * E;
  double L1, L2;
  if (A < kEps) {
    L1 = 0.0;
    L2 = E < kEps ? 0.0 : -D / E / 2.0;
  } else if (E < kEps) {
    L2 = 0.0;
    L1 = -B / A / 2.0;
  } else if (fabs(G) < kEps) {
    const double d[4] = {dot(y0 - x0, y0 - x0), dot(y1 - x0, y1 - x0), dot(y0 - x1, y0 - x1), dot(y1 - x1, y1 - x1)};
    int idx = 1;  // findmin: the first minimum, a NaN counting as the smallest
    for (int k = 1; k < 4 && !isnan(d[idx - 1]); ++k)
      if (isnan(d[k]) || d[k] < d[idx - 1]) idx = k + 1;
    L1 = floor((double)idx / 2.0);
    L2 = (double)((idx - 1) % 2);
  } else {
    L2 = (2.0 * A * D + B * C) / G;
    L1 = (C * L2 - B) / A / 2.0;
  }
  L1 = clamp01(L1);
  L2 = clamp01(L2);
  const V P = x0 + seg1 * L1 - y0 - seg2 * L2;
  const V W = vx0 + vseg1 * L1 - vy0 - vseg2 * L2;
  return {dot(P, P), 2.0 * dot(W, P), L1, L2};
}

__device__ __forceinline__ bool mobile(int32_t l) { return l == 1 || l == 3; }  // intMobDln, srfMobDln

// Canonical (a <= b) link pairs, sorted: binary search.
__device__ bool skipped(const int64_t* __restrict__ sk, int64_t n, int64_t a, int64_t b) {
  if (a > b) {
    const int64_t t = a;
    a = b;
    b = t;
  }
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    const int64_t p = sk[2 * mid], q = sk[2 * mid + 1];
    if (p < a || (p == a && q < b))
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < n && sk[2 * lo] == a && sk[2 * lo + 1] == b;
}

// The two-line filters other than mobility (DislocationTopologyCollision.jl:
// 150-193): no shared node, no superdislocation in the making, not skipped.
// Segment i < j (0-based), nodes 0-based.
__device__ __forceinline__ bool pair_passes(int64_t i, int64_t j, int32_t a1, int32_t a2, int32_t c1, int32_t c2,
                                            const double* __restrict__ coord, const double* __restrict__ bVec,
                                            const int64_t* __restrict__ skip, int64_t nSkip) {
  if (a1 == c1 || a1 == c2 || a2 == c1 || a2 == c2) return false;
  const V bi = ld3(bVec, i), bj = ld3(bVec, j);
  const V bm = bi - bj, bp = bi + bj;
  const double tt = dot(ld3(coord, a2) - ld3(coord, a1), ld3(coord, c2) - ld3(coord, c1));
  if ((dot(bm, bm) < kEps && tt > kEps) || (dot(bp, bp) < kEps && tt < kEps)) return false;
  return !(nSkip > 0 && skipped(skip, nSkip, i + 1, j + 1));
}

// (key, lo, hi) order of the reference's scan: larger key first, then the
// earlier pair.  key < 0: no candidate.
__device__ __forceinline__ bool better(double k1, int64_t a1, int64_t b1, double k2, int64_t a2, int64_t b2) {
  return k1 > k2 || (k1 == k2 && (a1 < a2 || (a1 == a2 && b1 < b2)));
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

struct Box {
  double lo[3];
  double scale;  // 1023 / largest extent
};

// Per segment (original order): node ids, mobility, Morton key of the midpoint.
__global__ void seg_prep(const double* __restrict__ coord, const int32_t* __restrict__ label,
                         const int64_t* __restrict__ links, int64_t numSeg, Box box, uint32_t* __restrict__ keys,
                         int32_t* __restrict__ vals, int2* __restrict__ ids, uint8_t* __restrict__ mob) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= numSeg) return;
  const int32_t a1 = (int32_t)(links[2 * i] - 1), a2 = (int32_t)(links[2 * i + 1] - 1);
  ids[i] = make_int2(a1, a2);
  mob[i] = mobile(label[a1]) && mobile(label[a2]);
  const V m = (ld3(coord, a1) + ld3(coord, a2)) * 0.5;
  const double c[3] = {m.x, m.y, m.z};
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double u = (c[k] - box.lo[k]) * box.scale;
    q[k] = u > 0.0 ? (uint32_t)fmin(u, 1023.0) : 0u;
  }
  keys[i] = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
  vals[i] = (int32_t)i;
}

// Sorted slot s: bounding sphere (FP32 centre, radius rounded up with margins)
// and meta (original index, node ids, mobile); padding is not mobile.
__global__ void gather(const double* __restrict__ coord, const int32_t* __restrict__ perm,
                       const int2* __restrict__ ids, const uint8_t* __restrict__ mob, int64_t numSeg, int64_t npad,
                       double maxAbs, float4* __restrict__ sph, int4* __restrict__ meta) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= npad) return;
  if (s >= numSeg) {
    sph[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    meta[s] = make_int4(-1, -1, -1, 0);
    return;
  }
  const int32_t i = perm[s];
  const int2 a = ids[i];
  const V x0 = ld3(coord, a.x), x1 = ld3(coord, a.y);
  const V m = (x0 + x1) * 0.5;
  const V d = x1 - x0;
  const double h = 0.5 * sqrt(dot(d, d));
  const float r = __double2float_ru(h * (1.0 + 1e-5) + 1e-5 * maxAbs);
  sph[s] = make_float4(__double2float_rn(m.x), __double2float_rn(m.y), __double2float_rn(m.z), r);
  meta[s] = make_int4(i, a.x, a.y, mob[i] ? 1 : 0);
}

// Per tile: box of its mobile segments' spheres, rounded outward (8 floats: lo
// xyz, hi xyz, any-mobile flag, unused).
__global__ void tile_boxes(const float4* __restrict__ sph, const int4* __restrict__ meta, float* __restrict__ box) {
  __shared__ float sm[6][T];
  const int t = threadIdx.x;
  const int64_t s = blockIdx.x * (int64_t)T + t;
  const float4 c = sph[s];
  const bool on = meta[s].w != 0;
  sm[0][t] = on ? __fsub_rd(c.x, c.w) : INFINITY;
  sm[1][t] = on ? __fsub_rd(c.y, c.w) : INFINITY;
  sm[2][t] = on ? __fsub_rd(c.z, c.w) : INFINITY;
  sm[3][t] = on ? __fadd_ru(c.x, c.w) : -INFINITY;
  sm[4][t] = on ? __fadd_ru(c.y, c.w) : -INFINITY;
  sm[5][t] = on ? __fadd_ru(c.z, c.w) : -INFINITY;
  const int any = __syncthreads_or(on);
  for (int w = T / 2; w > 0; w >>= 1) {
    if (t < w) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        sm[k][t] = fminf(sm[k][t], sm[k][t + w]);
        sm[3 + k][t] = fmaxf(sm[3 + k][t], sm[3 + k][t + w]);
      }
    }
    __syncthreads();
  }
  if (t < 6) box[8 * blockIdx.x + t] = sm[t][0];
  if (t == 6) box[8 * blockIdx.x + 6] = any ? 1.f : 0.f;
  if (t == 7) box[8 * blockIdx.x + 7] = 0.f;
}

struct Cand {
  double key;
  int64_t lo, hi;
};

template <int N>
__device__ void block_best(Cand& c, Cand* sm) {
  const int t = threadIdx.x;
  sm[t] = c;
  __syncthreads();
  for (int w = N / 2; w > 0; w >>= 1) {
    if (t < w) {
      const Cand o = sm[t + w];
      if (better(o.key, o.lo, o.hi, sm[t].key, sm[t].lo, sm[t].hi)) sm[t] = o;
    }
    __syncthreads();
  }
  c = sm[0];
}

// Two-line pass over the tile pairs (I <= J) of the sorted segments,
// persistent; each CTA takes the next tile pair from a counter (most tile
// pairs are rejected by their boxes at once, a few carry all the work).
__global__ void __launch_bounds__(T) two_line(const float4* __restrict__ sph, const int4* __restrict__ meta,
                                               const float* __restrict__ tbox, int64_t nTP, float Rf, double cd2,
                                               const double* __restrict__ coord, const double* __restrict__ vel,
                                               const double* __restrict__ bVec, const int64_t* __restrict__ skip,
                                               int64_t nSkip, unsigned long long* __restrict__ next,
                                               Cand* __restrict__ part) {
  __shared__ float4 s_sph[T];
  __shared__ int4 s_meta[T];
  __shared__ Cand s_red[T];
  __shared__ unsigned long long s_tp;
  const int t = threadIdx.x;
  Cand best = {-1.0, INT64_MAX, INT64_MAX};
  for (;;) {
    __syncthreads();  // the previous tile pair's shared data and s_tp are no longer read
    if (t == 0) s_tp = atomicAdd(next, 1ull);
    __syncthreads();
    const int64_t tp = (int64_t)s_tp;
    if (tp >= nTP) break;
    int64_t J = (int64_t)((sqrt(8.0 * (double)tp + 1.0) - 1.0) * 0.5);
    while (J * (J + 1) / 2 > tp) --J;
    while ((J + 1) * (J + 2) / 2 <= tp) ++J;
    const int64_t I = tp - J * (J + 1) / 2;
    const float* bI = tbox + 8 * I;
    const float* bJ = tbox + 8 * J;
    if (bI[6] == 0.f || bJ[6] == 0.f) continue;
    float gap = -INFINITY;
#pragma unroll
    for (int k = 0; k < 3; ++k) gap = fmaxf(gap, fmaxf(__fsub_rd(bJ[k], bI[3 + k]), __fsub_rd(bI[k], bJ[3 + k])));
    if (gap > Rf) continue;  // uniform over the block: no pair of these tiles is within reach
    s_sph[t] = sph[J * T + t];
    s_meta[t] = meta[J * T + t];
    __syncthreads();
    const int4 mi = meta[I * T + t];
    if (!mi.w) continue;
    const float4 si = sph[I * T + t];
    for (int jj = (I == J) ? t + 1 : 0; jj < T; ++jj) {
      const int4 mj = s_meta[jj];
      if (!mj.w) continue;
      const float4 sj = s_sph[jj];
      const float dx = si.x - sj.x, dy = si.y - sj.y, dz = si.z - sj.z;
      const float lim = Rf + si.w + sj.w;
      if (dx * dx + dy * dy + dz * dz > lim * lim) continue;
      const bool iFirst = mi.x < mj.x;
      const int4 lo = iFirst ? mi : mj, hi = iFirst ? mj : mi;
      if (!pair_passes(lo.x, hi.x, lo.y, lo.z, hi.y, hi.z, coord, bVec, skip, nSkip)) continue;
      const MD m = min_dist(ld3(coord, lo.y), ld3(coord, lo.z), ld3(coord, hi.y), ld3(coord, hi.z), ld3(vel, lo.y),
                            ld3(vel, lo.z), ld3(vel, hi.y), ld3(vel, hi.z));
      if (m.distSq < cd2 && m.dDistSqDt < -kEps) {
        const double key = 1.0 / m.distSq;
        if (better(key, lo.x, hi.x, best.key, best.lo, best.hi)) best = {key, lo.x, hi.x};
      }
    }
  }
  __syncthreads();
  block_best<T>(best, s_red);
  if (t == 0) part[blockIdx.x] = best;
}

struct HingeRec {
  double key;                            // best candidate of the block (< 0: none)
  int64_t node, node1, node2, link1, link2;
  int64_t last;                          // largest node with an evaluated pair (-1: none)
  double lastL1, lastL2;
};

// Hinge pass: node i's pairs of connections (DislocationTopologyCollision.jl:24-127).
__global__ void __launch_bounds__(RB) hinge(const double* __restrict__ coord, const double* __restrict__ vel,
                                            const int32_t* __restrict__ label, const int64_t* __restrict__ links,
                                            const int64_t* __restrict__ conn, int64_t ldConn, int64_t numNode,
                                            double cd2, const int64_t* __restrict__ skip, int64_t nSkip,
                                            HingeRec* __restrict__ part) {
  __shared__ HingeRec sm[RB];
  const int t = threadIdx.x;
  const int64_t i = blockIdx.x * (int64_t)RB + t;
  HingeRec r = {-1.0, -1, 0, 0, 0, 0, -1, 0.0, 0.0};
  if (i < numNode && mobile(label[i])) {
    const int64_t* c = conn + ldConn * i;
    const int64_t nc = c[0];
    const V xi = ld3(coord, i), vi = ld3(vel, i);
    for (int64_t j = 1; j <= nc; ++j) {
      int64_t link1 = c[2 * j - 1];
      int64_t node1 = links[2 * (link1 - 1) + (3 - c[2 * j]) - 1];
      V tv = xi - ld3(coord, node1 - 1);
      double tN1 = dot(tv, tv);
      for (int64_t k = j + 1; k <= nc; ++k) {
        int64_t link2 = c[2 * k - 1];
        int64_t node2 = links[2 * (link2 - 1) + (3 - c[2 * k]) - 1];
        tv = xi - ld3(coord, node2 - 1);
        double tN2 = dot(tv, tv);
        if (tN1 < tN2) {  // the reference swaps its j-loop variables here
          const int64_t l = link1, n = node1;
          const double q = tN1;
          link1 = link2, node1 = node2, tN1 = tN2;
          link2 = l, node2 = n, tN2 = q;
        }
        if (nSkip > 0 && skipped(skip, nSkip, link1, link2)) continue;
        const V y0 = ld3(coord, node2 - 1), vy0 = ld3(vel, node2 - 1);
        const MD m = min_dist(xi, ld3(coord, node1 - 1), y0, y0, vi, ld3(vel, node1 - 1), vy0, vy0);
        r.last = i;
        r.lastL1 = m.L1;
        r.lastL2 = m.L2;
        if (m.distSq < cd2 && m.dDistSqDt < -kEps) {
          const double key = 1.0 / m.distSq;
          if (key > r.key) {
            r.key = key;
            r.node = i;
            r.node1 = node1;
            r.node2 = node2;
            r.link1 = link1;
            r.link2 = link2;
          }
        }
      }
    }
  }
  sm[t] = r;
  __syncthreads();
  for (int w = RB / 2; w > 0; w >>= 1) {
    if (t < w) {
      const HingeRec o = sm[t + w];
      HingeRec& a = sm[t];
      if (o.key > a.key || (o.key == a.key && o.key >= 0.0 && o.node < a.node)) {
        a.key = o.key, a.node = o.node, a.node1 = o.node1, a.node2 = o.node2, a.link1 = o.link1, a.link2 = o.link2;
      }
      if (o.last > a.last) a.last = o.last, a.lastL1 = o.lastL1, a.lastL2 = o.lastL2;
    }
    __syncthreads();
  }
  if (t == 0) part[blockIdx.x] = sm[0];
}

// Last evaluated two-line pair: per row i, the largest j > i that passes every
// filter (scanned downward, so usually found at once); per block the largest
// (i, j) as i * numSeg + j.
__global__ void __launch_bounds__(RB) row_last(const double* __restrict__ coord, const double* __restrict__ bVec,
                                               const int2* __restrict__ ids, const uint8_t* __restrict__ mob,
                                               int64_t numSeg, const int64_t* __restrict__ skip, int64_t nSkip,
                                               int64_t* __restrict__ part) {
  __shared__ int64_t sm[RB];
  const int t = threadIdx.x;
  const int64_t i = blockIdx.x * (int64_t)RB + t;
  int64_t best = -1;
  if (i < numSeg && mob[i]) {
    const int2 a = ids[i];
    for (int64_t j = numSeg - 1; j > i; --j) {
      if (!mob[j]) continue;
      const int2 c = ids[j];
      if (pair_passes(i, j, a.x, a.y, c.x, c.y, coord, bVec, skip, nSkip)) {
        best = i * numSeg + j;
        break;
      }
    }
  }
  sm[t] = best;
  __syncthreads();
  for (int w = RB / 2; w > 0; w >>= 1) {
    if (t < w) sm[t] = max(sm[t], sm[t + w]);
    __syncthreads();
  }
  if (t == 0) part[blockIdx.x] = sm[0];
}

// Combines the partial results in the reference's order and writes the answer.
__global__ void __launch_bounds__(RB) resolve(const HingeRec* __restrict__ hp, int nH, const Cand* __restrict__ tp,
                                              int nT, const int64_t* __restrict__ rp, int nR,
                                              const double* __restrict__ coord, const double* __restrict__ vel,
                                              const int2* __restrict__ ids, int64_t numSeg,
                                              CollisionOut* __restrict__ out) {
  __shared__ HingeRec sh[RB];
  __shared__ Cand sc[RB];
  __shared__ int64_t sr[RB];
  const int t = threadIdx.x;
  HingeRec h = {-1.0, -1, 0, 0, 0, 0, -1, 0.0, 0.0};
  for (int q = t; q < nH; q += RB) {
    const HingeRec o = hp[q];
    if (o.key > h.key || (o.key == h.key && o.key >= 0.0 && o.node < h.node))
      h.key = o.key, h.node = o.node, h.node1 = o.node1, h.node2 = o.node2, h.link1 = o.link1, h.link2 = o.link2;
    if (o.last > h.last) h.last = o.last, h.lastL1 = o.lastL1, h.lastL2 = o.lastL2;
  }
  Cand c = {-1.0, INT64_MAX, INT64_MAX};
  for (int q = t; q < nT; q += RB) {
    const Cand o = tp[q];
    if (better(o.key, o.lo, o.hi, c.key, c.lo, c.hi)) c = o;
  }
  int64_t last = -1;
  for (int q = t; q < nR; q += RB) last = max(last, rp[q]);
  sh[t] = h;
  sr[t] = last;
  __syncthreads();
  for (int w = RB / 2; w > 0; w >>= 1) {
    if (t < w) {
      const HingeRec o = sh[t + w];
      HingeRec& a = sh[t];
      if (o.key > a.key || (o.key == a.key && o.key >= 0.0 && o.node < a.node))
        a.key = o.key, a.node = o.node, a.node1 = o.node1, a.node2 = o.node2, a.link1 = o.link1, a.link2 = o.link2;
      if (o.last > a.last) a.last = o.last, a.lastL1 = o.lastL1, a.lastL2 = o.lastL2;
      sr[t] = max(sr[t], sr[t + w]);
    }
    __syncthreads();
  }
  block_best<RB>(c, sc);
  if (t != 0) return;
  h = sh[0];
  last = sr[0];
  CollisionOut r = {};
  if (h.key >= 0.0) {
    r.collision = 1;
    r.type = 1;
    r.n1s1 = h.node + 1;
    r.n2s1 = h.node1;
    r.n1s2 = h.node2;
    r.n2s2 = h.node2;
    r.s1 = h.link1;
    r.s2 = h.link2;
    const V x0 = ld3(coord, h.node), y0 = ld3(coord, h.node2 - 1), vy0 = ld3(vel, h.node2 - 1);
    const MD m = min_dist(x0, ld3(coord, h.node1 - 1), y0, y0, ld3(vel, h.node), ld3(vel, h.node1 - 1), vy0, vy0);
    r.pairDistSq = m.distSq, r.pairL1 = m.L1, r.pairL2 = m.L2;
    r.L1 = h.lastL1;
    r.L2 = h.lastL2;
    *out = r;
    return;
  }
  if (c.key >= 0.0) {
    const int2 a = ids[c.lo], b = ids[c.hi];
    r.collision = 1;
    r.type = 2;
    r.n1s1 = a.x + 1, r.n2s1 = a.y + 1, r.n1s2 = b.x + 1, r.n2s2 = b.y + 1;
    r.s1 = c.lo + 1;
    r.s2 = c.hi + 1;
    const MD m = min_dist(ld3(coord, a.x), ld3(coord, a.y), ld3(coord, b.x), ld3(coord, b.y), ld3(vel, a.x),
                          ld3(vel, a.y), ld3(vel, b.x), ld3(vel, b.y));
    r.pairDistSq = m.distSq, r.pairL1 = m.L1, r.pairL2 = m.L2;
  }
  if (last >= 0) {
    const int64_t i = last / numSeg, j = last % numSeg;
    const int2 a = ids[i], b = ids[j];
    const MD m = min_dist(ld3(coord, a.x), ld3(coord, a.y), ld3(coord, b.x), ld3(coord, b.y), ld3(vel, a.x),
                          ld3(vel, a.y), ld3(vel, b.x), ld3(vel, b.y));
    r.L1 = m.L1;
    r.L2 = m.L2;
  } else if (h.last >= 0) {
    r.L1 = h.lastL1;
    r.L2 = h.lastL2;
  }
  *out = r;
}

__global__ void min_dist_batch(const double* __restrict__ pts, int64_t n, double* __restrict__ out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double* p = pts + 24 * q;
  const MD m = min_dist(ld3(p, 0), ld3(p, 1), ld3(p, 2), ld3(p, 3), ld3(p, 4), ld3(p, 5), ld3(p, 6), ld3(p, 7));
  out[4 * q] = m.distSq;
  out[4 * q + 1] = m.dDistSqDt;
  out[4 * q + 2] = m.L1;
  out[4 * q + 3] = m.L2;
}

using Buf = GrowBuf;

}  // namespace

struct CollisionPlan {
  Buf keysIn, keysOut, valsIn, valsOut, cub, ids, mob, sph, meta, tbox, hpart, tpart, rpart, out, next;
  int twoLineGrid = 0;
};

CollisionPlan* collision_plan_create() { return new CollisionPlan(); }
void collision_plan_destroy(CollisionPlan* p) { delete p; }

#define CCK(x)                              \
  do {                                      \
    cudaError_t e_ = (x);                   \
    if (e_ != cudaSuccess) return e_;       \
  } while (0)

cudaError_t collision_detect(CollisionPlan* P, double cd2, const double* coord, const double* vel, const int32_t* label,
                             const int64_t* links, const double* bVec, const int64_t* conn, int64_t ldConn,
                             int64_t numNode, int64_t numSeg, const int64_t* skip, int64_t nSkip, const double box[6],
                             double maxAbs, CollisionOut* out, cudaEvent_t e0, cudaEvent_t e1, cudaStream_t st) {
  const int64_t nt = (numSeg + T - 1) / T;
  const int64_t npad = nt * T;
  const int64_t nTP = nt * (nt + 1) / 2;
  const int nH = (int)std::max<int64_t>(1, (numNode + RB - 1) / RB);
  const int nR = (int)std::max<int64_t>(1, (numSeg + RB - 1) / RB);
  if (!P->twoLineGrid) {
    int dev = 0, sms = 0, occ = 0;
    CCK(cudaGetDevice(&dev));
    CCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, two_line, T, 0));
    P->twoLineGrid = sms * std::max(occ, 1);
  }
  const int gT = (int)std::max<int64_t>(1, std::min<int64_t>(nTP, P->twoLineGrid));
  size_t cubBytes = 0;
  if (numSeg > 0)
    CCK(cub::DeviceRadixSort::SortPairs(nullptr, cubBytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                        (const int32_t*)nullptr, (int32_t*)nullptr, (int)numSeg, 0, 30, st));
  const size_t ns = (size_t)std::max<int64_t>(numSeg, 1), np = (size_t)std::max<int64_t>(npad, T);
  CCK(P->keysIn.ensure(ns * 4));
  CCK(P->keysOut.ensure(ns * 4));
  CCK(P->valsIn.ensure(ns * 4));
  CCK(P->valsOut.ensure(ns * 4));
  CCK(P->cub.ensure(cubBytes + 16));
  CCK(P->ids.ensure(ns * sizeof(int2)));
  CCK(P->mob.ensure(ns));
  CCK(P->sph.ensure(np * sizeof(float4)));
  CCK(P->meta.ensure(np * sizeof(int4)));
  CCK(P->tbox.ensure((size_t)std::max<int64_t>(nt, 1) * 8 * sizeof(float)));
  CCK(P->hpart.ensure((size_t)nH * sizeof(HingeRec)));
  CCK(P->tpart.ensure((size_t)gT * sizeof(Cand)));
  CCK(P->rpart.ensure((size_t)nR * sizeof(int64_t)));
  CCK(P->out.ensure(sizeof(CollisionOut)));
  CCK(P->next.ensure(sizeof(unsigned long long)));

  Box bx;
  const double ext = std::max(std::max(box[3] - box[0], box[4] - box[1]), box[5] - box[2]);
  for (int k = 0; k < 3; ++k) bx.lo[k] = box[k];
  bx.scale = ext > 0.0 ? 1023.0 / ext : 0.0;
  const double R = cd2 > 0.0 ? sqrt(cd2) : 0.0;
  // Coordinates beyond 1e15 would overflow the FP32 squares of the prefilter:
  // an infinite reach turns both prefilters off (every pair goes to FP64).
  float Rf = INFINITY;
  if (maxAbs < 1e15) {  // R * (1 + 1e-5), rounded up to a float
    const double want = R * (1.0 + 1e-5);
    Rf = (float)want;
    if ((double)Rf < want) Rf = std::nextafter(Rf, INFINITY);
  }

  if (e0) CCK(cudaEventRecord(e0, st));
  // Hinge pass (also for an empty node list: one block writes "none").
  hinge<<<nH, RB, 0, st>>>(coord, vel, label, links, conn, ldConn, numNode, cd2, skip, nSkip, P->hpart.as<HingeRec>());
  CCK(cudaGetLastError());
  int nTparts = 0, nRparts = 0;
  if (numSeg > 1) {
    const int gs = (int)((numSeg + RB - 1) / RB);
    seg_prep<<<gs, RB, 0, st>>>(coord, label, links, numSeg, bx, P->keysIn.as<uint32_t>(), P->valsIn.as<int32_t>(),
                                P->ids.as<int2>(), P->mob.as<uint8_t>());
    CCK(cudaGetLastError());
    CCK(cub::DeviceRadixSort::SortPairs(P->cub.p, cubBytes, P->keysIn.as<uint32_t>(), P->keysOut.as<uint32_t>(),
                                        P->valsIn.as<int32_t>(), P->valsOut.as<int32_t>(), (int)numSeg, 0, 30, st));
    gather<<<(int)((npad + RB - 1) / RB), RB, 0, st>>>(coord, P->valsOut.as<int32_t>(), P->ids.as<int2>(),
                                                       P->mob.as<uint8_t>(), numSeg, npad, maxAbs,
                                                       P->sph.as<float4>(), P->meta.as<int4>());
    CCK(cudaGetLastError());
    tile_boxes<<<(int)nt, T, 0, st>>>(P->sph.as<float4>(), P->meta.as<int4>(), P->tbox.as<float>());
    CCK(cudaGetLastError());
    CCK(cudaMemsetAsync(P->next.p, 0, sizeof(unsigned long long), st));
    two_line<<<gT, T, 0, st>>>(P->sph.as<float4>(), P->meta.as<int4>(), P->tbox.as<float>(), nTP, Rf, cd2, coord, vel,
                               bVec, skip, nSkip, P->next.as<unsigned long long>(), P->tpart.as<Cand>());
    CCK(cudaGetLastError());
    row_last<<<nR, RB, 0, st>>>(coord, bVec, P->ids.as<int2>(), P->mob.as<uint8_t>(), numSeg, skip, nSkip,
                                P->rpart.as<int64_t>());
    CCK(cudaGetLastError());
    nTparts = gT;
    nRparts = nR;
  }
  resolve<<<1, RB, 0, st>>>(P->hpart.as<HingeRec>(), nH, P->tpart.as<Cand>(), nTparts, P->rpart.as<int64_t>(), nRparts,
                            coord, vel, P->ids.as<int2>(), numSeg, P->out.as<CollisionOut>());
  CCK(cudaGetLastError());
  if (e1) CCK(cudaEventRecord(e1, st));
  CCK(cudaMemcpyAsync(out, P->out.p, sizeof(CollisionOut), cudaMemcpyDeviceToHost, st));
  return cudaStreamSynchronize(st);
}

cudaError_t launch_minimum_distance(const double* pts, int64_t n, double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  min_dist_batch<<<(int)((n + 255) / 256), 256, 0, st>>>(pts, n, out);
  return cudaGetLastError();
}

}  // namespace ddd
