// Seg-seg forces with the learned surrogate for far pairs (ddd_surrogate_force).
//
// Order of work on the caller's stream:
//   1. prep: bounding box of the midpoints, 30-bit Morton keys, radix sort
//      (CUB), gather of the segments into sorted order (FP64 SoA, skip flags,
//      FP32 surrogate data), per-tile boxes, and the list of tile pairs whose
//      boxes are close enough to hold a pair outside the trust region;
//   2. network pass (surrogate_infer.cu): every tile pair I <= J, far pairs
//      through the MLP, partial forces written to the tile pair's slot;
//   3. near pass: the listed tile pairs, every pair outside the trust region
//      evaluated exactly (tile_body MODE 2: the reference's general or
//      near-parallel branch, the general branch in the caller's exact_mode
//      arithmetic: strict FP64, df64 or f32c) and added to the slot;
//   4. audit: a fixed, hashed ~audit_fraction of the tile pairs re-evaluated
//      exactly over all their pairs (tile_body MODE 0, the all-pairs body in
//      the same arithmetic), compared with their slots (network far pairs +
//      exact near pairs): the difference is the network's error;
//   5. reduction of each segment's slots in a fixed order, written back in the
//      caller's order.
// If the audited error exceeds the caller's bound, steps 2-5 are replaced by
// the exact all-pairs tile kernel on the same sorted data.  Every sum has a
// fixed order: the forces are deterministic.
//
// Compiled with --fmad=false: the exact passes round as the reference does.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ddd_gb300.h"
#include "ddd_internal.h"
#include "net_check.h"
#include "pair_f64.cuh"
#include "surrogate.cuh"
#include "surrogate_state.h"
#include "tile_body.cuh"
#include "tile_pol_df.cuh"
#include "tile_pol_fx.cuh"

namespace ddd {

size_t mlp_seg_bytes(int64_t npad);
cudaError_t launch_prep_mlp_seg(const double* soa, const uint8_t* skip, int64_t npad, float* ms, cudaStream_t st);
cudaError_t launch_mlp_far_tiles(const float* ms, int64_t npad, const int4* items, int32_t nItems, int32_t* next,
                                 const void* const* W, const float* params, float mu4pi, float kappa2,
                                 double* partial, int32_t* err, int grid, cudaStream_t st);
// farfield_quad.cu: the far pairs by Gauss-Legendre quadrature in FP32 instead of the network.
size_t quad_seg_bytes(int64_t npad);
cudaError_t launch_prep_quad_seg(const double* soa, const float* ms, int64_t npad, float* qs, cudaStream_t st);
int quad_far_blocks_per_sm(int nq);
cudaError_t launch_quad_far_tiles(const float* ms, const float* qs, const double* soa, int64_t npad, const int4* items,
                                  int32_t nItems, int nq, const KConsts& K, float kappa2, float kappaTwo2,
                                  double* partial, int grid, cudaStream_t st);

namespace sf {

constexpr int T = 128;

// Per-block min / max of the midpoints of segments [0, n) of the packed array.
__global__ void mid_minmax_part(const double* __restrict__ segs, int64_t ld, int64_t n, double* __restrict__ part) {
  __shared__ double sm[6][256];
  double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double m = 0.5 * (segs[c * ld + i] + segs[(3 + c) * ld + i]);
      v[c] = fmin(v[c], m);
      v[3 + c] = fmax(v[3 + c], m);
    }
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) sm[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sm[c][threadIdx.x] = fmin(sm[c][threadIdx.x], sm[c][threadIdx.x + s]);
        sm[3 + c][threadIdx.x] = fmax(sm[3 + c][threadIdx.x], sm[3 + c][threadIdx.x + s]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = sm[threadIdx.x][0];
}

__global__ void mid_minmax_final(const double* __restrict__ part, int nb, double* __restrict__ box) {
  if (threadIdx.x >= 6) return;
  const int c = threadIdx.x;
  double v = c < 3 ? INFINITY : -INFINITY;
  for (int b = 0; b < nb; ++b) v = c < 3 ? fmin(v, part[b * 6 + c]) : fmax(v, part[b * 6 + c]);
  box[c] = v;
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

// Morton key of each midpoint on a 1024^3 grid over the bounding cube.
__global__ void morton_keys(const double* __restrict__ segs, int64_t ld, int64_t n, const double* __restrict__ box,
                            uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ext = fmax(fmax(box[3] - box[0], box[4] - box[1]), box[5] - box[2]);
  const double sc = ext > 0.0 ? 1023.0 / ext : 0.0;
  uint32_t q[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double m = 0.5 * (segs[c * ld + i] + segs[(3 + c) * ld + i]);
    const double u = (m - box[c]) * sc;
    q[c] = u > 0.0 ? (uint32_t)fmin(u, 1023.0) : 0u;  // NaN -> 0
  }
  keys[i] = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
  vals[i] = (int32_t)i;
}

// Sorted FP64 SoA (13 rows, as the tile kernels read it), skip flags and the
// source column of each sorted position (-1 for padding); counts active segments.
__global__ void gather_sorted(const double* __restrict__ segs, int64_t ld, const uint8_t* __restrict__ ext,
                              const int32_t* __restrict__ perm, int64_t numSeg, int64_t npad, double* __restrict__ soa,
                              uint8_t* __restrict__ skip, int32_t* __restrict__ src,
                              unsigned long long* __restrict__ active) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= npad) return;
  double v[13];
  uint8_t sk = 1;
  int32_t i = -1;
  if (s < numSeg) {
    i = perm[s];
    const D3 n1 = {segs[i], segs[ld + i], segs[2 * ld + i]};
    const D3 n2 = {segs[3 * ld + i], segs[4 * ld + i], segs[5 * ld + i]};
    const D3 bv = {segs[6 * ld + i], segs[7 * ld + i], segs[8 * ld + i]};
    D3 t;
    double tN;
    seg_direction(n1, n2, t, tN);
    v[0] = n1.x; v[1] = n1.y; v[2] = n1.z;
    v[3] = n2.x; v[4] = n2.y; v[5] = n2.z;
    v[6] = bv.x; v[7] = bv.y; v[8] = bv.z;
    v[9] = t.x; v[10] = t.y; v[11] = t.z; v[12] = tN;
    sk = ext ? (ext[i] ? 1 : 0) : 0;
  } else {
#pragma unroll
    for (int k = 0; k < 13; ++k) v[k] = 0.0;
    v[3] = 1.0;
    v[9] = 1.0;
    v[12] = 1.0;
  }
#pragma unroll
  for (int k = 0; k < 13; ++k) soa[k * npad + s] = v[k];
  skip[s] = sk;
  src[s] = i;
  const unsigned m = __ballot_sync(__activemask(), sk == 0);
  if ((threadIdx.x & 31) == __ffs(__activemask()) - 1 && m) atomicAdd(active, (unsigned long long)__popc(m));
}

// Per tile: bounding box of the active midpoints and the longest active segment
// (8 floats: min xyz, max xyz, Lmax, any-active flag).
__global__ void tile_boxes(const float* __restrict__ ms, int64_t npad, float* __restrict__ box) {
  __shared__ float sm[7][T];
  const int t = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * T + t;
  const float L = ms[sur::kMsL * npad + i];
  const bool act = L > 0.0f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float m = ms[(sur::kMsM + c) * npad + i];
    sm[c][t] = act ? m : INFINITY;
    sm[3 + c][t] = act ? m : -INFINITY;
  }
  sm[6][t] = act ? L : 0.0f;
  __syncthreads();
  for (int s = T / 2; s > 0; s >>= 1) {
    if (t < s) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sm[c][t] = fminf(sm[c][t], sm[c][t + s]);
        sm[3 + c][t] = fmaxf(sm[3 + c][t], sm[3 + c][t + s]);
      }
      sm[6][t] = fmaxf(sm[6][t], sm[6][t + s]);
    }
    __syncthreads();
  }
  if (t < 7) box[blockIdx.x * 8 + t] = sm[t][0];
  if (t == 7) box[blockIdx.x * 8 + 7] = sm[6][0] > 0.0f ? 1.0f : 0.0f;
}

// Tile pairs that may hold a pair outside the trust region: box gap below
// kappa * max(Lmax_I, Lmax_J) (with a relative margin far above the FP32
// rounding of the pairwise test, so the list is a superset of what the pairwise
// test selects).  List order is arbitrary; each item owns its slot.
__global__ void near_items(const int4* __restrict__ all, int32_t nAll, const float* __restrict__ box, float kappa,
                           int4* __restrict__ out, int32_t* __restrict__ count) {
  const int32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nAll) return;
  const int4 it = all[w];
  const float* bI = box + (it.y / T) * 8;
  const float* bJ = box + (it.z / T) * 8;
  if (bI[7] == 0.0f || bJ[7] == 0.0f) return;
  float d2 = 0.0f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float g = fmaxf(0.0f, fmaxf(bJ[c] - bI[3 + c], bI[c] - bJ[3 + c]));
    d2 += g * g;
  }
  const float cut = kappa * fmaxf(bI[6], bJ[6]) * 1.001f + 1e-3f;
  if (d2 < cut * cut) out[atomicAdd(count, 1)] = it;
}

// Persistent loop of the exact tile body (arithmetic policy P) over a work
// list; the item count is read from the device (nDev) when given.
template <int MODE, class P>
__global__ void __launch_bounds__(T, 2)
exact_tiles(TileArgs A, typename P::Consts KP, const int4* __restrict__ items, const int32_t* __restrict__ nDev,
            int32_t nHost, int32_t* __restrict__ next, double* __restrict__ partial,
            unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& sm = *reinterpret_cast<TileSmemT<T, P>*>(smem_raw);
  __shared__ int32_t s_item;
  const int32_t nItems = nDev ? *nDev : nHost;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int32_t w = s_item;
    if (w >= nItems) break;
    const int4 it = items[w];
    tile_body<T, MODE, P>(A, KP, sm, it.y, it.z, it.w != 0, nullptr, 0, partial + (int64_t)it.x * 12 * T, counters);
  }
}

// Per audited tile pair: squared error of the network's slot against the exact
// far-pair slot, and the squared norm of the exact one (fixed-order tree).
__global__ void audit_compare(const double* __restrict__ partial, const double* __restrict__ abuf,
                              const int32_t* __restrict__ aslot, double* __restrict__ astat) {
  __shared__ double se[T], sr[T];
  const int a = blockIdx.x, t = threadIdx.x;
  const double* p = partial + (int64_t)aslot[a] * 12 * T;
  const double* e = abuf + (int64_t)a * 12 * T;
  double e2 = 0.0, r2 = 0.0;
#pragma unroll
  for (int c = 0; c < 12; ++c) {
    const double x = e[c * T + t], d = p[c * T + t] - x;
    e2 += d * d;
    r2 += x * x;
  }
  se[t] = e2;
  sr[t] = r2;
  __syncthreads();
  for (int s = T / 2; s > 0; s >>= 1) {
    if (t < s) {
      se[t] += se[t + s];
      sr[t] += sr[t + s];
    }
    __syncthreads();
  }
  if (t == 0) {
    astat[2 * a] = se[0];
    astat[2 * a + 1] = sr[0];
  }
}

// out = {sum e2, sum r2, max e2 / r2} over the audited tile pairs (fixed order).
__global__ void audit_final(const double* __restrict__ astat, int32_t nA, double* __restrict__ out) {
  __shared__ double se[256], sr[256], sx[256];
  const int t = threadIdx.x;
  double e2 = 0.0, r2 = 0.0, mx = 0.0;
  for (int a = t; a < nA; a += 256) {
    e2 += astat[2 * a];
    r2 += astat[2 * a + 1];
    if (astat[2 * a + 1] > 0.0) mx = fmax(mx, astat[2 * a] / astat[2 * a + 1]);
  }
  se[t] = e2;
  sr[t] = r2;
  sx[t] = mx;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (t < s) {
      se[t] += se[t + s];
      sr[t] += sr[t + s];
      sx[t] = fmax(sx[t], sx[t + s]);
    }
    __syncthreads();
  }
  if (t == 0) {
    out[0] = se[0];
    out[1] = sr[0];
    out[2] = sx[0];
  }
}

// Per-block sums of squares of v[0, n) (fixed order), then their total.
__global__ void sumsq_part(const double* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double sm[256];
  double a = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a += v[i] * v[i];
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void sumsq_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double a = 0.0;
  for (int b = 0; b < nb; ++b) a += part[b];
  *out = a;
}

// Each sorted segment's row and column slots, summed in a fixed order, written
// to the caller's position src[s].
__global__ void reduce_unpermute(const double* __restrict__ partial, const int32_t* __restrict__ src, int64_t npad,
                                 int64_t nt, double* __restrict__ out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= npad) return;
  const int32_t i = src[s];
  if (i < 0) return;
  const int64_t Ab = s / T;
  const int t = (int)(s % T);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t Jt = Ab; Jt < nt; ++Jt) {
    const double* p = partial + (Jt * (Jt + 1) / 2 + Ab) * 12 * T;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[c * T + t];
  }
  for (int64_t It = 0; It <= Ab; ++It) {
    const double* p = partial + (Ab * (Ab + 1) / 2 + It) * 12 * T;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[(6 + c) * T + t];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) out[6 * (int64_t)i + c] = acc[c];
}

}  // namespace sf

// Device buffers of the force path for one segment count.
struct SurForcePlan {
  using Buf = GrowBuf;
  int64_t numSeg = -1, npad = 0, nt = 0, nItems = 0;
  int32_t nAudit = 0;
  double auditFraction = -1.0;
  size_t cubBytes = 0;
  int sms = 0, gridExact = 0, gridQuad = 0;
  Buf soa, soadf, skip, ms, qs, keysIn, keysOut, valsIn, perm, src, cubTmp, minmaxPart, box, tbox, allItems, nearItems, partial,
      auditItems, auditSlots, abuf, astat, small;
  Buf hostSegs, hostExt, hostForce;  // device copies for the host-array entry point
  cudaEvent_t ev[6] = {};
  ~SurForcePlan() {
    for (Buf* b : {&soa, &soadf, &skip, &ms, &qs, &keysIn, &keysOut, &valsIn, &perm, &src, &cubTmp, &minmaxPart, &box, &tbox,
                   &allItems, &nearItems, &partial, &auditItems, &auditSlots, &abuf, &astat, &small, &hostSegs,
                   &hostExt, &hostForce})
      b->release();
    for (cudaEvent_t& e : ev)
      if (e) cudaEventDestroy(e);
  }
};

// Layout of the `small` buffer: counters and flags reset at every call.
struct SmallDev {
  int32_t next[4];               // work counters: network, audit, near, fallback
  int32_t nearCount;             // near-pass list length
  int32_t err;                   // bounded-wait timeout flag
  unsigned long long active;     // active segments
  unsigned long long counts[3];  // near pass: general, near-parallel, core
  double audit[3];               // sum e2, sum r2, max e2 / r2
  double fnorm2;                 // sum of squares of the output forces
};

void destroy_force_plan(SurForcePlan* p) { delete p; }

namespace {

constexpr int kMinmaxBlocks = 256;

// 32-bit mix of the slot index: the audit takes the slots whose hash falls
// below fraction * 2^32 (about that fraction, spread over the network).
uint32_t slot_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

template <int MODE, class P>
cudaError_t set_exact_attr() {
  static std::atomic<uint64_t> done{0};
  return set_smem_once(sf::exact_tiles<MODE, P>, (int)sizeof(TileSmemT<sf::T, P>), done);
}

template <int MODE, class P>
cudaError_t launch_exact_p(const TileArgs& A, const typename P::Consts& KP, const int4* items, const int32_t* nDev,
                           int32_t nHost, int32_t* next, double* partial, unsigned long long* counters, int grid,
                           cudaStream_t st) {
  cudaError_t e = set_exact_attr<MODE, P>();
  if (e != cudaSuccess) return e;
  sf::exact_tiles<MODE, P><<<grid, sf::T, sizeof(TileSmemT<sf::T, P>), st>>>(A, KP, items, nDev, nHost, next,
                                                                             partial, counters);
  return cudaGetLastError();
}

// The exact tile pass in the arithmetic of `mode` (DDD_MODE_FP64 strict,
// DDD_MODE_FP64_FAST, DDD_MODE_DF64 or DDD_MODE_F32C for the general branch).
template <int MODE>
cudaError_t launch_exact(int mode, const TileArgs& A, const int4* items, const int32_t* nDev, int32_t nHost,
                         int32_t* next, double* partial, unsigned long long* counters, int grid, cudaStream_t st) {
  if (mode == DDD_MODE_FP64)
    return launch_exact_p<MODE, PolF64>(A, PolF64::Consts{}, items, nDev, nHost, next, partial, counters, grid, st);
  if (mode == DDD_MODE_FP64_FAST)
    return launch_exact_p<MODE, PolF64Fast>(A, PolF64Fast::Consts{}, items, nDev, nHost, next, partial, counters, grid,
                                            st);
  const typename PolDF<0>::Consts KP{kconsts_df(A.K), kconsts_f(A.K)};
  if (mode == DDD_MODE_DF64)
    return launch_exact_p<MODE, PolDF<0>>(A, KP, items, nDev, nHost, next, partial, counters, grid, st);
  return launch_exact_p<MODE, PolDF<1>>(A, typename PolDF<1>::Consts{KP.K, KP.KF}, items, nDev, nHost, next, partial,
                                        counters, grid, st);
}

cudaError_t ensure_plan(ddd_surrogate* s, int64_t numSeg, double auditFraction) {
  if (!s->plan) s->plan = new SurForcePlan();
  SurForcePlan& P = *s->plan;
  cudaError_t e;
  if (P.numSeg != numSeg) {
    const int64_t T = sf::T;
    P.numSeg = numSeg;
    P.npad = (numSeg + T - 1) / T * T;
    P.nt = P.npad / T;
    P.nItems = P.nt * (P.nt + 1) / 2;
    P.auditFraction = -1.0;
    if ((e = cudaDeviceGetAttribute(&P.sms, cudaDevAttrMultiProcessorCount, s->device)) != cudaSuccess) return e;
    if ((e = set_exact_attr<2, PolF64>()) != cudaSuccess) return e;
    int per = 0;  // the df64 policies use the same shared memory and register budget
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sf::exact_tiles<2, PolF64>, sf::T,
                                                           sizeof(TileSmemT<sf::T, PolF64>))) != cudaSuccess)
      return e;
    P.gridExact = P.sms * std::max(1, per);
    P.gridQuad = P.sms * quad_far_blocks_per_sm(3);
    const size_t n = (size_t)numSeg, np = (size_t)P.npad;
    if ((e = P.soa.ensure(np * 13 * sizeof(double))) != cudaSuccess) return e;
    if ((e = P.skip.ensure(np)) != cudaSuccess) return e;
    if ((e = P.ms.ensure(mlp_seg_bytes(P.npad))) != cudaSuccess) return e;
    if ((e = P.keysIn.ensure(n * 4)) != cudaSuccess) return e;
    if ((e = P.keysOut.ensure(n * 4)) != cudaSuccess) return e;
    if ((e = P.valsIn.ensure(n * 4)) != cudaSuccess) return e;
    if ((e = P.perm.ensure(n * 4)) != cudaSuccess) return e;
    if ((e = P.src.ensure(np * 4)) != cudaSuccess) return e;
    size_t cb = 0;
    if ((e = cub::DeviceRadixSort::SortPairs(nullptr, cb, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                             (const int32_t*)nullptr, (int32_t*)nullptr, (int)numSeg, 0, 30)) !=
        cudaSuccess)
      return e;
    P.cubBytes = cb;
    if ((e = P.cubTmp.ensure(cb)) != cudaSuccess) return e;
    if ((e = P.minmaxPart.ensure(kMinmaxBlocks * 6 * sizeof(double))) != cudaSuccess) return e;
    if ((e = P.box.ensure(6 * sizeof(double))) != cudaSuccess) return e;
    if ((e = P.tbox.ensure((size_t)P.nt * 8 * sizeof(float))) != cudaSuccess) return e;
    if ((e = P.allItems.ensure((size_t)P.nItems * sizeof(int4))) != cudaSuccess) return e;
    if ((e = P.nearItems.ensure((size_t)P.nItems * sizeof(int4))) != cudaSuccess) return e;
    if ((e = P.partial.ensure((size_t)P.nItems * 12 * T * sizeof(double))) != cudaSuccess) return e;
    if ((e = P.small.ensure(sizeof(SmallDev))) != cudaSuccess) return e;
    std::vector<int4> items((size_t)P.nItems);
    size_t w = 0;
    for (int64_t J = 0; J < P.nt; ++J)
      for (int64_t I = 0; I <= J; ++I)
        items[w++] = make_int4((int)(J * (J + 1) / 2 + I), (int)(I * T), (int)(J * T), I == J ? 1 : 0);
    if ((e = cudaMemcpy(P.allItems.p, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      return e;
    for (cudaEvent_t& ev : P.ev)
      if (!ev && (e = cudaEventCreate(&ev)) != cudaSuccess) return e;
  }
  if (P.auditFraction != auditFraction) {
    P.auditFraction = auditFraction;
    std::vector<int4> aitems;
    std::vector<int32_t> aslot;
    const double thr = auditFraction * 4294967296.0;
    for (int64_t J = 0; J < P.nt; ++J)
      for (int64_t I = 0; I <= J; ++I) {
        const int64_t slot = J * (J + 1) / 2 + I;
        if ((double)slot_hash((uint32_t)slot) < thr) {
          aitems.push_back(make_int4((int)aslot.size(), (int)(I * sf::T), (int)(J * sf::T), I == J ? 1 : 0));
          aslot.push_back((int32_t)slot);
        }
      }
    P.nAudit = (int32_t)aslot.size();
    if (P.nAudit > 0) {
      if ((e = P.auditItems.ensure(aitems.size() * sizeof(int4))) != cudaSuccess) return e;
      if ((e = P.auditSlots.ensure(aslot.size() * 4)) != cudaSuccess) return e;
      if ((e = P.abuf.ensure((size_t)P.nAudit * 12 * sf::T * sizeof(double))) != cudaSuccess) return e;
      if ((e = P.astat.ensure((size_t)P.nAudit * 2 * sizeof(double))) != cudaSuccess) return e;
      if ((e = cudaMemcpy(P.auditItems.p, aitems.data(), aitems.size() * sizeof(int4), cudaMemcpyHostToDevice)) !=
          cudaSuccess)
        return e;
      if ((e = cudaMemcpy(P.auditSlots.p, aslot.data(), aslot.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    }
  }
  return cudaSuccess;
}

int sfail(ddd_surrogate* s, int code, const std::string& m) {
  s->lastError = m;
  return code;
}

}  // namespace
}  // namespace ddd

using namespace ddd;

#define SCK(x, what)                                                                                     \
  do {                                                                                                   \
    cudaError_t _e = (x);                                                                                \
    if (_e != cudaSuccess)                                                                               \
      return sfail(s, _e == cudaErrorMemoryAllocation ? DDD_ENOMEM : DDD_EDEVICE,                        \
                   std::string(what) + ": " + cudaGetErrorString(_e));                                   \
  } while (0)

extern "C" {

const char* ddd_surrogate_last_error(const ddd_surrogate* s) { return s ? s->lastError.c_str() : "null surrogate"; }

int ddd_surrogate_force(ddd_surrogate* s, const ddd_consts* k, const double* segs, int64_t ldSegs,
                        const uint8_t* ext, int64_t numSeg, double* force, void* stream, const ddd_sur_opts* opts,
                        ddd_sur_report* rep) {
  DDD_NVTX("ddd_surrogate_force");
  if (!s) return DDD_EINVAL;
  ddd_sur_opts o{20.0, 0.01, 1e-3, DDD_MODE_FP64, 0, 0.0};
  if (opts) o = *opts;
  if (o.exact_mode != DDD_MODE_FP64 && o.exact_mode != DDD_MODE_FP64_FAST && o.exact_mode != DDD_MODE_DF64 &&
      o.exact_mode != DDD_MODE_F32C)
    return sfail(s, DDD_EINVAL, "exact_mode must be DDD_MODE_FP64, DDD_MODE_FP64_FAST, DDD_MODE_DF64 or DDD_MODE_F32C");
  if (o.far_mode != 0 && o.far_mode != 2 && o.far_mode != 3)
    return sfail(s, DDD_EINVAL, "far_mode must be 0 (network) or 2 / 3 (Gauss points of the quadrature)");
  if (!k) return sfail(s, DDD_EINVAL, "consts is NULL");
  const double kv[5] = {k->aSq, k->mu4pi, k->mu8pi, k->mu4pinu, k->nuMu4pinu};
  for (double x : kv)
    if (!std::isfinite(x)) return sfail(s, DDD_ENONFINITE, "non-finite material/core constant");
  if (!(k->aSq > 0.0)) return sfail(s, DDD_EINVAL, "aSq (coreRadSq) must be > 0");
  if (!(o.kappa > 0.0) || !std::isfinite(o.kappa)) return sfail(s, DDD_EINVAL, "kappa must be > 0");
  if (!(o.kappa_two >= 0.0) || !std::isfinite(o.kappa_two))
    return sfail(s, DDD_EINVAL, "kappa_two must be >= 0 (0: no 2-point switch)");
  if (!(o.audit_fraction >= 0.0 && o.audit_fraction <= 1.0)) return sfail(s, DDD_EINVAL, "audit_fraction in [0, 1]");
  if (numSeg < 0 || ldSegs < numSeg) return sfail(s, DDD_EINVAL, "numSeg < 0 or ldSegs < numSeg");
  if (numSeg > ((int64_t)1 << 24)) return sfail(s, DDD_ETOOBIG, "numSeg above 2^24");
  if (numSeg > 0 && (!segs || !force)) return sfail(s, DDD_EINVAL, "segs or force is NULL");
  if (rep) std::memset(rep, 0, sizeof *rep);
  if (numSeg == 0) return DDD_OK;

  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  // No stream given: the inputs may come from any stream; wait for all queued work.
  if (!stream) SCK(cudaDeviceSynchronize(), "wait for the caller's device inputs");
  cudaStream_t st = stream ? (cudaStream_t)stream : s->own;
  SCK(ensure_plan(s, numSeg, o.audit_fraction), "allocate force-path buffers");
  SurForcePlan& P = *s->plan;
  const int64_t npad = P.npad, nt = P.nt;
  SmallDev* dv = P.small.as<SmallDev>();
  KConsts K;
  K.aSq = k->aSq;
  K.mu4pi = k->mu4pi;
  K.mu8pi = k->mu8pi;
  K.mu4pinu = k->mu4pinu;
  K.nuMu4pinu = k->nuMu4pinu;
  K.mu8piaSq = k->aSq * k->mu8pi;
  K.mu4pinuaSq = k->aSq * k->mu4pinu;
  const float kappa = (float)o.kappa;
  const int xm = o.exact_mode;
  const bool dfx = xm == DDD_MODE_DF64 || xm == DDD_MODE_F32C;  // the exact passes read df64 segment data
  if (dfx) SCK(P.soadf.ensure((size_t)npad * 26 * sizeof(float)), "allocate df64 segments");
  if (o.far_mode) SCK(P.qs.ensure(quad_seg_bytes(npad)), "allocate quadrature segment data");
  TileArgs A{K, P.soa.as<double>(), P.skip.as<uint8_t>(), npad, P.soadf.as<float>(), nullptr};
  A.ms = P.ms.as<float>();
  A.farK2 = kappa * kappa;
  const unsigned nb = (unsigned)((npad + 255) / 256);

  // 1. prep
  SCK(cudaEventRecord(P.ev[0], st), "event");
  SCK(cudaMemsetAsync(dv, 0, sizeof(SmallDev), st), "memset");
  sf::mid_minmax_part<<<kMinmaxBlocks, 256, 0, st>>>(segs, ldSegs, numSeg, P.minmaxPart.as<double>());
  sf::mid_minmax_final<<<1, 32, 0, st>>>(P.minmaxPart.as<double>(), kMinmaxBlocks, P.box.as<double>());
  sf::morton_keys<<<(unsigned)((numSeg + 255) / 256), 256, 0, st>>>(segs, ldSegs, numSeg, P.box.as<double>(),
                                                                    P.keysIn.as<uint32_t>(), P.valsIn.as<int32_t>());
  SCK(cudaGetLastError(), "morton keys");
  size_t cb = P.cubBytes;
  SCK(cub::DeviceRadixSort::SortPairs(P.cubTmp.p, cb, P.keysIn.as<uint32_t>(), P.keysOut.as<uint32_t>(),
                                      P.valsIn.as<int32_t>(), P.perm.as<int32_t>(), (int)numSeg, 0, 30, st),
      "radix sort");
  sf::gather_sorted<<<nb, 256, 0, st>>>(segs, ldSegs, ext, P.perm.as<int32_t>(), numSeg, npad, P.soa.as<double>(),
                                        P.skip.as<uint8_t>(), P.src.as<int32_t>(), &dv->active);
  SCK(cudaGetLastError(), "gather");
  SCK(launch_prep_mlp_seg(P.soa.as<double>(), P.skip.as<uint8_t>(), npad, P.ms.as<float>(), st), "prep_mlp_seg");
  if (o.far_mode)
    SCK(launch_prep_quad_seg(P.soa.as<double>(), P.ms.as<float>(), npad, P.qs.as<float>(), st), "prep_quad_seg");
  if (dfx) SCK(launch_prep_df(P.soa.as<double>(), npad, P.soadf.as<float>(), st), "prep_df");
  sf::tile_boxes<<<(unsigned)nt, sf::T, 0, st>>>(P.ms.as<float>(), npad, P.tbox.as<float>());
  sf::near_items<<<(unsigned)((P.nItems + 255) / 256), 256, 0, st>>>(
      P.allItems.as<int4>(), (int32_t)P.nItems, P.tbox.as<float>(), kappa, P.nearItems.as<int4>(), &dv->nearCount);
  SCK(cudaGetLastError(), "tile classification");
  SCK(cudaEventRecord(P.ev[1], st), "event");

  // 2. far pass over every tile pair: the network, or Gauss-Legendre quadrature
  if (o.far_mode) {
    const float kappaTwo = (float)o.kappa_two;
    const float kappaTwo2 = o.far_mode == 3 && o.kappa_two > 0.0 ? kappaTwo * kappaTwo : INFINITY;
    SCK(launch_quad_far_tiles(P.ms.as<float>(), P.qs.as<float>(), P.soa.as<double>(), npad, P.allItems.as<int4>(),
                              (int32_t)P.nItems,
                              o.far_mode, K, kappa * kappa, kappaTwo2, P.partial.as<double>(),
                              (int)std::min<int64_t>(P.gridQuad, P.nItems), st),
        "quadrature pass");
  } else {
    const void* W[4] = {s->W1, s->W2, s->W3, s->W4};
    const int gridNet = (int)std::min<int64_t>(P.sms, P.nItems);
    SCK(launch_mlp_far_tiles(P.ms.as<float>(), npad, P.allItems.as<int4>(), (int32_t)P.nItems, &dv->next[0], W, s->P,
                             (float)k->mu4pi, kappa * kappa, P.partial.as<double>(), &dv->err, gridNet, st),
        "network pass");
  }
  SCK(cudaEventRecord(P.ev[2], st), "event");

  // 3. near pass (in place)
  SCK(launch_exact<2>(xm, A, P.nearItems.as<int4>(), &dv->nearCount, 0, &dv->next[2], P.partial.as<double>(),
                      dv->counts, P.gridExact, st),
      "near pass");
  SCK(cudaEventRecord(P.ev[3], st), "event");

  // 4. audit: the sampled tile pairs exactly over all their pairs (the plain
  // all-pairs tile body), against their slots, which now hold the network's
  // far pairs plus the exact near pairs: the difference is the network's
  // error on the far pairs (the near pairs agree up to summation order).
  if (P.nAudit > 0) {
    SCK(launch_exact<0>(xm, A, P.auditItems.as<int4>(), nullptr, P.nAudit, &dv->next[1], P.abuf.as<double>(), nullptr,
                        (int)std::min<int64_t>(P.gridExact, P.nAudit), st),
        "audit pass");
    sf::audit_compare<<<P.nAudit, sf::T, 0, st>>>(P.partial.as<double>(), P.abuf.as<double>(),
                                                   P.auditSlots.as<int32_t>(), P.astat.as<double>());
    sf::audit_final<<<1, 256, 0, st>>>(P.astat.as<double>(), P.nAudit, dv->audit);
    SCK(cudaGetLastError(), "audit compare");
  }
  SCK(cudaEventRecord(P.ev[4], st), "event");

  // 5. reduction into the caller's order
  sf::reduce_unpermute<<<nb, 256, 0, st>>>(P.partial.as<double>(), P.src.as<int32_t>(), npad, nt, force);
  sf::sumsq_part<<<kMinmaxBlocks, 256, 0, st>>>(force, numSeg * 6, P.minmaxPart.as<double>());
  sf::sumsq_final<<<1, 32, 0, st>>>(P.minmaxPart.as<double>(), kMinmaxBlocks, &dv->fnorm2);
  SCK(cudaGetLastError(), "reduce");
  SCK(cudaEventRecord(P.ev[5], st), "event");

  SmallDev h;
  SCK(cudaMemcpyAsync(&h, dv, sizeof h, cudaMemcpyDeviceToHost, st), "copy counters");
  SCK(cudaStreamSynchronize(st), "surrogate force");
  if (h.err) return sfail(s, DDD_ETIMEOUT, "network pass: mbarrier wait timed out");

  const double relRms = h.audit[1] > 0.0 ? std::sqrt(h.audit[0] / h.audit[1]) : 0.0;
  // Node-level estimate: every tile pair adds its slot error to the node forces
  // of its 256 segments, so the squared error over all nodes is the sum of the
  // tile pairs' squared slot errors, estimated from the audited sample.
  const double frac = (double)P.nAudit / (double)P.nItems;
  const double nodeRel =
      (P.nAudit > 0 && h.fnorm2 > 0.0) ? std::sqrt(h.audit[0] / frac) / std::sqrt(h.fnorm2) : 0.0;
  int fallback = 0;
  float msFallback = 0.0f;
  if (o.audit_tol > 0.0 && P.nAudit > 0 && nodeRel > o.audit_tol) {
    // The audit exceeded its bound: exact forces for every pair.
    cudaEvent_t e0 = P.ev[1], e1 = P.ev[2];
    SCK(cudaEventRecord(e0, st), "event");
    SCK(launch_exact<0>(xm, A, P.allItems.as<int4>(), nullptr, (int32_t)P.nItems, &dv->next[3], P.partial.as<double>(),
                        nullptr, P.gridExact, st),
        "exact fallback");
    sf::reduce_unpermute<<<nb, 256, 0, st>>>(P.partial.as<double>(), P.src.as<int32_t>(), npad, nt, force);
    SCK(cudaGetLastError(), "reduce");
    SCK(cudaEventRecord(e1, st), "event");
    SCK(cudaEventSynchronize(e1), "exact fallback");
    cudaEventElapsedTime(&msFallback, e0, e1);
    fallback = 1;
  }
  if (rep) {
    const int64_t na = (int64_t)h.active;
    rep->pairs_total = na * (na - 1) / 2;
    rep->pairs_near_general = (int64_t)h.counts[0];
    rep->pairs_near_parallel = (int64_t)h.counts[1];
    rep->tiles_total = P.nItems;
    rep->tiles_near = h.nearCount;
    rep->tiles_audit = P.nAudit;
    rep->audit_rel_rms = relRms;
    rep->audit_rel_max = std::sqrt(h.audit[2]);
    rep->audit_node_rel_rms = nodeRel;
    rep->fallback = fallback;
    float m[5] = {0, 0, 0, 0, 0};
    if (!fallback)
      for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&m[i], P.ev[i], P.ev[i + 1]);
    rep->ms_prep = m[0];
    rep->ms_network = m[1];
    rep->ms_near = m[2];
    rep->ms_audit = m[3];
    rep->ms_reduce = m[4];
    rep->ms_total = fallback ? (double)msFallback : (double)(m[0] + m[1] + m[2] + m[3] + m[4]);
  }
  return DDD_OK;
}

// The network's own host arrays (the layout of ddd_segseg_force): validated and
// packed on the host, copied in, ddd_surrogate_force on the surrogate's stream,
// forces copied out.
int ddd_surrogate_force_host(ddd_surrogate* s, const ddd_consts* k, const double* coord, int64_t coordCols,
                             const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                             const uint8_t* extSeg, int64_t numSeg, double* force, const ddd_sur_opts* opts,
                             ddd_sur_report* rep) {
  DDD_NVTX("ddd_surrogate_force_host");
  if (!s) return DDD_EINVAL;
  if (numSeg < 0 || coordCols < 0 || bVecCols < 0 || ldSegIdx < numSeg)
    return sfail(s, DDD_EINVAL, "negative size or numSeg exceeds the rows of segIdx");
  if (numSeg > 0 && (!coord || !bVec || !segIdx || !force)) return sfail(s, DDD_EINVAL, "network array is NULL");
  if (numSeg > ((int64_t)1 << 24)) return sfail(s, DDD_ETOOBIG, "numSeg above 2^24");
  std::vector<double> packed((size_t)numSeg * 9);
  for (int64_t r = 0; r < numSeg; ++r) {
    std::string msg;
    const int rc = check_segment_row(coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, r, msg);
    if (rc) return sfail(s, rc, msg);
    const double* p1 = coord + 3 * (segIdx[r + ldSegIdx] - 1);
    const double* p2 = coord + 3 * (segIdx[r + 2 * ldSegIdx] - 1);
    const double* bv = bVec + 3 * (segIdx[r] - 1);
    for (int c = 0; c < 3; ++c) {
      packed[(size_t)c * numSeg + r] = p1[c];
      packed[(size_t)(3 + c) * numSeg + r] = p2[c];
      packed[(size_t)(6 + c) * numSeg + r] = bv[c];
    }
  }
  if (rep) std::memset(rep, 0, sizeof *rep);
  if (numSeg == 0) return DDD_OK;
  SCK(cudaSetDevice(s->device), "cudaSetDevice");
  if (!s->plan) s->plan = new SurForcePlan();
  SurForcePlan& P = *s->plan;
  SCK(P.hostSegs.ensure(packed.size() * sizeof(double)), "allocate segments");
  SCK(P.hostForce.ensure((size_t)numSeg * 6 * sizeof(double)), "allocate forces");
  if (extSeg) SCK(P.hostExt.ensure((size_t)numSeg), "allocate extSeg");
  cudaStream_t st = s->own;
  SCK(cudaMemcpyAsync(P.hostSegs.p, packed.data(), packed.size() * sizeof(double), cudaMemcpyHostToDevice, st),
      "copy segments");
  if (extSeg) SCK(cudaMemcpyAsync(P.hostExt.p, extSeg, (size_t)numSeg, cudaMemcpyHostToDevice, st), "copy extSeg");
  const int rc = ddd_surrogate_force(s, k, P.hostSegs.as<double>(), numSeg, extSeg ? P.hostExt.as<uint8_t>() : nullptr,
                                     numSeg, P.hostForce.as<double>(), st, opts, rep);
  if (rc) return rc;
  SCK(cudaMemcpyAsync(force, P.hostForce.p, (size_t)numSeg * 6 * sizeof(double), cudaMemcpyDeviceToHost, st),
      "copy forces");
  SCK(cudaStreamSynchronize(st), "surrogate force");
  return DDD_OK;
}

}  // extern "C"
