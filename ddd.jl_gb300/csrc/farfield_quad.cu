// Far-pair pass of the seg-seg force by Gauss-Legendre quadrature in FP32
// (farfield_quad.cuh): the alternative to the network pass in the surrogate
// force path (ddd_surrogate_force with far_mode = 2 or 3).  Same routing: the
// Morton-sorted segments, every tile pair I <= J, the FP32 trust test
// pair_is_far deciding which pairs are far (the near pass takes the others),
// and the same per-tile-pair slot of 12 x 128 partial forces (row segments'
// then column segments' node forces), so the near pass, audit and reduction
// run unchanged after it.
//
// One CTA of 128 threads per tile pair (grid-stride over the items).  Thread t
// owns row segment i in registers; the column tile sits in shared memory; at
// step k thread t pairs with column (t + k) mod 128, so a warp's lanes never
// share a column and column forces accumulate race-free in per-warp arrays.
// Per-segment FP32 data (qs, built by prep_quad_seg from the sorted FP64
// segments): the low part of the midpoint (the FP32 midpoint of the trust test
// plus this part gives the midpoint to ~2^-48), the segment vector n2 - n1,
// the unit direction, the length and the Burgers vector.
//
// With 3 points (far_mode 3) a warp's step of 32 pairs takes the 2-point rule
// instead when each far pair it holds lies beyond kappaTwo max(L_i, L_j)
// (ddd_sur_opts.kappa_two): the 2-point rule's truncation error falls as
// (L/R)^4 (~5e-6 per pair at 20 lengths, ~1e-6 at 30; from 30 the node-force
// errors measure as with 3 points everywhere), and it costs 4 + 2 instead of
// 9 + 3 stress evaluations per side.  The choice
// is a warp vote on values fixed by the tile layout, so results stay
// deterministic; the dense near-parallel pass votes the same way over its
// listed pairs.
//
// Near-parallel pairs (1 - c^2 <= sqrt(eps) by the reference's FP64 test on
// the FP64 directions; an FP32 pre-test with a wide margin picks the
// candidates) are flagged during the sweep and evaluated afterwards in a
// compacted dense pass (fixed order, so the sums stay deterministic), with the
// reference's construction of calcParSegSegForce
// (DislocationForces.jl:1167-1442): each side's source segment projected onto
// the field segment's direction and pulled in by the critical angle, plus the
// two connector segments where its core-correction test holds
// (qf::par_sources); the quadrature then integrates that geometry, so these
// pairs get the force the reference assigns them.
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "farfield_quad.cuh"
#include "pair_f64.cuh"
#include "surrogate.cuh"

namespace ddd {

namespace {

constexpr int TQ = 128;
constexpr int kQsRows = 13;  // midpoint low part xyz, segment vector xyz, direction xyz, length, Burgers xyz
constexpr int kQLo = 0, kQL = 3, kQT = 6, kQLen = 9, kQB = 10;

__global__ void prep_quad_seg(const double* __restrict__ soa, const float* __restrict__ ms, int64_t npad,
                              float* __restrict__ qs) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= npad) return;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double n1 = soa[k * npad + i], n2 = soa[(3 + k) * npad + i];
    const double m = 0.5 * (n1 + n2);
    qs[(kQLo + k) * npad + i] = (float)(m - (double)ms[(sur::kMsM + k) * npad + i]);
    qs[(kQL + k) * npad + i] = (float)(n2 - n1);
    qs[(kQT + k) * npad + i] = (float)soa[(9 + k) * npad + i];
    qs[(kQB + k) * npad + i] = (float)soa[(6 + k) * npad + i];
  }
  qs[kQLen * npad + i] = (float)(1.0 / soa[12 * npad + i]);
}

// FP64 record of segment g of the sorted SoA (rows n1, n2, t).
__device__ __forceinline__ qf::SegD seg_d(const double* __restrict__ soa, int64_t npad, int64_t g) {
  qf::SegD d;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    d.n1[k] = soa[k * npad + g];
    d.l[k] = soa[(3 + k) * npad + g] - d.n1[k];
    d.t[k] = soa[(9 + k) * npad + g];
  }
  return d;
}

// R^2 >= kappaTwo2 max(L_i, L_j)^2 for the midpoint difference d, rounded as
// the trust test (sur::pair_is_far) rounds it; false when kappaTwo2 is
// infinite (rule switch off).
__device__ __forceinline__ bool beyond(float dx, float dy, float dz, float Li, float Lj, float kappaTwo2) {
  const float R2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  const float Lm = fmaxf(Li, Lj);
  return R2 >= __fmul_rn(kappaTwo2, __fmul_rn(Lm, Lm));
}

// Near-parallel pairs listed per round: a tile pair with more (up to 128 x 128)
// takes several rounds.  The cap keeps the shared memory at four CTAs per SM.
constexpr int kPCap = 8192;

// Shared memory of one CTA: the column tile, per-warp column forces, and the
// compaction state of the near-parallel pairs.
struct QuadSmem {
  float cM[3][TQ], cLen[TQ];      // trust-test data of the column tile
  float cQ[kQsRows][TQ];          // quadrature data of the column tile
  float sFJ[TQ / 32][6][TQ];      // per-warp column forces
  float cf[TQ][12];               // dense pass: one pair's four node forces per thread
  uint16_t plist[kPCap];          // near-parallel pairs (row << 8 | column), by row then step: one round
  int cnt[TQ];
  int total;
};

// Four CTAs of 128 threads per SM (128 registers per thread, 43 KB of shared
// memory each); the near-parallel pairs run in a dense pass after the sweep (as
// in tile_body.cuh), so a warp never waits on one lane's FP64 branch.
template <int NQ>
__global__ void __launch_bounds__(TQ, 4)
quad_far_tiles(const float* __restrict__ ms, const float* __restrict__ qs, const double* __restrict__ soa, int64_t npad,
               const int4* __restrict__ items, int32_t nItems, qf::QConst K, float kappa2, float kappaTwo2,
               double* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char qsm_raw[];
  QuadSmem& sm = *reinterpret_cast<QuadSmem*>(qsm_raw);
  constexpr int NW = TQ / 32;
  const int t = threadIdx.x, warp = t >> 5;
  for (int32_t w = blockIdx.x; w < nItems; w += gridDim.x) {
    const int4 it = items[w];
    const int64_t i0 = it.y, i = it.y + t, j0 = it.z;
    const bool diag = it.w != 0;
    __syncthreads();  // the previous item's readers are done with the tile
#pragma unroll
    for (int k = 0; k < 3; ++k) sm.cM[k][t] = ms[(sur::kMsM + k) * npad + j0 + t];
    sm.cLen[t] = ms[sur::kMsL * npad + j0 + t];
#pragma unroll
    for (int k = 0; k < kQsRows; ++k) sm.cQ[k][t] = qs[k * npad + j0 + t];
#pragma unroll
    for (int q = 0; q < NW; ++q)
#pragma unroll
      for (int c = 0; c < 6; ++c) sm.sFJ[q][c][t] = 0.0f;
    const float mi[3] = {ms[(sur::kMsM + 0) * npad + i], ms[(sur::kMsM + 1) * npad + i],
                         ms[(sur::kMsM + 2) * npad + i]};
    const float Li = ms[sur::kMsL * npad + i];
    const float loi[3] = {qs[(kQLo + 0) * npad + i], qs[(kQLo + 1) * npad + i], qs[(kQLo + 2) * npad + i]};
    const qf::V3f li = {qs[(kQL + 0) * npad + i], qs[(kQL + 1) * npad + i], qs[(kQL + 2) * npad + i]};
    const qf::V3f ti = {qs[(kQT + 0) * npad + i], qs[(kQT + 1) * npad + i], qs[(kQT + 2) * npad + i]};
    const float Lni = qs[kQLen * npad + i];
    const qf::V3f bi = {qs[(kQB + 0) * npad + i], qs[(kQB + 1) * npad + i], qs[(kQB + 2) * npad + i]};
    __syncthreads();

    // ---- Sweep: general far pairs by quadrature; near-parallel ones flagged. ----
    qf::V3f f1 = {0.f, 0.f, 0.f}, f2 = {0.f, 0.f, 0.f};
    uint32_t pmask[NW];
#pragma unroll
    for (int q = 0; q < NW; ++q) pmask[q] = 0;
    for (int k = 0; k < TQ; ++k) {
      const int jl = (t + k) & (TQ - 1);
      float dx, dy, dz, R2, Lm2;
      const bool far = sur::pair_is_far(mi[0], mi[1], mi[2], Li, sm.cM[0][jl], sm.cM[1][jl], sm.cM[2][jl],
                                        sm.cLen[jl], kappa2, dx, dy, dz, R2, Lm2);
      const bool take = far && (!diag || jl > t);
      // 2-point rule for this step when every pair the warp takes lies beyond
      // kappaTwo max(L_i, L_j) (a warp-uniform choice, fixed by the tile layout).
      const bool two = NQ == 2 || !__any_sync(0xffffffffu, take && !(R2 >= __fmul_rn(kappaTwo2, Lm2)));
      if (take) {
        const qf::V3f tj = {sm.cQ[kQT + 0][jl], sm.cQ[kQT + 1][jl], sm.cQ[kQT + 2][jl]};
        const float c32 = qf::dot(ti, tj);
        bool par = false;
        if (1.0f - c32 * c32 <= 1e-5f) {  // FP32 error of 1 - c^2 < 1e-6: only these can be near-parallel
          const int64_t gj = j0 + jl;
          const double ti64[3] = {soa[9 * npad + i], soa[10 * npad + i], soa[11 * npad + i]};
          const double tj64[3] = {soa[9 * npad + gj], soa[10 * npad + gj], soa[11 * npad + gj]};
          double c64;
          par = qf::par_decision(ti64, tj64, c64);
        }
        if (par) {
          pmask[jl >> 5] |= 1u << (jl & 31);
        } else {
          // m_i - m_j from the FP32 midpoints and their low parts.
          const qf::V3f dm = {(mi[0] - sm.cM[0][jl]) + (loi[0] - sm.cQ[kQLo + 0][jl]),
                              (mi[1] - sm.cM[1][jl]) + (loi[1] - sm.cQ[kQLo + 1][jl]),
                              (mi[2] - sm.cM[2][jl]) + (loi[2] - sm.cQ[kQLo + 2][jl])};
          const qf::V3f lj = {sm.cQ[kQL + 0][jl], sm.cQ[kQL + 1][jl], sm.cQ[kQL + 2][jl]};
          const qf::V3f bj = {sm.cQ[kQB + 0][jl], sm.cQ[kQB + 1][jl], sm.cQ[kQB + 2][jl]};
          const float Lnj = sm.cQ[kQLen][jl];
          qf::V3f Fa, Fb, Fc, Fd;
          if (two) {
            qf::side<2>(K, dm, li, bi, tj, Lnj, bj, Fa, Fb);
            qf::side<2>(K, {-dm.x, -dm.y, -dm.z}, lj, bj, ti, Lni, bi, Fc, Fd);
          } else {
            qf::side<NQ>(K, dm, li, bi, tj, Lnj, bj, Fa, Fb);
            qf::side<NQ>(K, {-dm.x, -dm.y, -dm.z}, lj, bj, ti, Lni, bi, Fc, Fd);
          }
          f1 = f1 + Fa;
          f2 = f2 + Fb;
          float* fj = &sm.sFJ[warp][0][0];
          fj[0 * TQ + jl] += Fc.x;
          fj[1 * TQ + jl] += Fc.y;
          fj[2 * TQ + jl] += Fc.z;
          fj[3 * TQ + jl] += Fd.x;
          fj[4 * TQ + jl] += Fd.y;
          fj[5 * TQ + jl] += Fd.z;
        }
      }
      __syncwarp();
    }

    // ---- Near-parallel pairs: compact in a fixed order, evaluate densely. ----
    int myCnt = 0;
#pragma unroll
    for (int q = 0; q < NW; ++q) myCnt += __popc(pmask[q]);
    sm.cnt[t] = myCnt;
    __syncthreads();
    if (warp == 0) {  // exclusive prefix sum over the 128 counts, 4 per lane
      int v[NW], s4 = 0;
#pragma unroll
      for (int q = 0; q < NW; ++q) {
        v[q] = sm.cnt[NW * t + q];
        s4 += v[q];
      }
      int incl = s4;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int nb = __shfl_up_sync(0xffffffffu, incl, o);
        if ((t & 31) >= o) incl += nb;
      }
      int excl = incl - s4;
#pragma unroll
      for (int q = 0; q < NW; ++q) {
        sm.cnt[NW * t + q] = excl;
        excl += v[q];
      }
    }
    __syncthreads();
    const int myOff = sm.cnt[t];
    if (t == TQ - 1) sm.total = myOff + myCnt;
    __syncthreads();
    const int nPar = sm.total;
    qf::V3f fc3 = {0.f, 0.f, 0.f}, fc4 = {0.f, 0.f, 0.f};  // this thread's column segment
    for (int r0 = 0; r0 < nPar; r0 += kPCap) {  // rounds of at most kPCap listed pairs
      const int rEnd = min(nPar, r0 + kPCap);
      {
        int o = myOff;
        for (int k = 0; k < TQ; ++k) {
          const int jl = (t + k) & (TQ - 1);
          if (pmask[jl >> 5] & (1u << (jl & 31))) {
            if (o >= r0 && o < rEnd) sm.plist[o - r0] = (uint16_t)((t << 8) | jl);
            ++o;
          }
        }
      }
      __syncthreads();
      for (int base = r0; base < rEnd; base += TQ) {
        const int e = base + t;
        const bool has = e < rEnd;
        const int il = has ? sm.plist[e - r0] >> 8 : 0, jl = has ? sm.plist[e - r0] & 0xff : 0;
        const int64_t gi = i0 + il, gj = j0 + jl;
        const float mi2[3] = {ms[(sur::kMsM + 0) * npad + gi], ms[(sur::kMsM + 1) * npad + gi],
                              ms[(sur::kMsM + 2) * npad + gi]};
        // The same warp-uniform choice of rule as the sweep's, over this warp's listed pairs.
        const bool two =
            NQ == 2 || !__any_sync(0xffffffffu, has && !beyond(__fsub_rn(sm.cM[0][jl], mi2[0]),
                                                               __fsub_rn(sm.cM[1][jl], mi2[1]),
                                                               __fsub_rn(sm.cM[2][jl], mi2[2]),
                                                               ms[sur::kMsL * npad + gi], sm.cLen[jl], kappaTwo2));
        if (has) {
          const qf::SegD si = seg_d(soa, npad, gi), sj = seg_d(soa, npad, gj);
          const qf::V3f dm = {(mi2[0] - sm.cM[0][jl]) + (qs[(kQLo + 0) * npad + gi] - sm.cQ[kQLo + 0][jl]),
                              (mi2[1] - sm.cM[1][jl]) + (qs[(kQLo + 1) * npad + gi] - sm.cQ[kQLo + 1][jl]),
                              (mi2[2] - sm.cM[2][jl]) + (qs[(kQLo + 2) * npad + gi] - sm.cQ[kQLo + 2][jl])};
          const qf::V3f la = {qs[(kQL + 0) * npad + gi], qs[(kQL + 1) * npad + gi], qs[(kQL + 2) * npad + gi]};
          const qf::V3f ba = {qs[(kQB + 0) * npad + gi], qs[(kQB + 1) * npad + gi], qs[(kQB + 2) * npad + gi]};
          const qf::V3f lb = {sm.cQ[kQL + 0][jl], sm.cQ[kQL + 1][jl], sm.cQ[kQL + 2][jl]};
          const qf::V3f bb = {sm.cQ[kQB + 0][jl], sm.cQ[kQB + 1][jl], sm.cQ[kQB + 2][jl]};
          const qf::V3f ta = {qs[(kQT + 0) * npad + gi], qs[(kQT + 1) * npad + gi], qs[(kQT + 2) * npad + gi]};
          const qf::V3f tb = {sm.cQ[kQT + 0][jl], sm.cQ[kQT + 1][jl], sm.cQ[kQT + 2][jl]};
          const qf::V3f ma = {mi2[0], mi2[1], mi2[2]}, mb = {sm.cM[0][jl], sm.cM[1][jl], sm.cM[2][jl]};
          const bool flip = qf::dot(ta, tb) < 0.0f;  // the sign of the FP64 t_i.t_j (|c| > 1 - 1e-8 here)
          qf::V3f Fa, Fb, Fc, Fd;
          if (two)
            qf::par_pair<2>(K, si, sj, flip, dm, ma, mb, ta, tb, la, ba, lb, bb, Fa, Fb, Fc, Fd);
          else
            qf::par_pair<NQ>(K, si, sj, flip, dm, ma, mb, ta, tb, la, ba, lb, bb, Fa, Fb, Fc, Fd);
          const float v[12] = {Fa.x, Fa.y, Fa.z, Fb.x, Fb.y, Fb.z, Fc.x, Fc.y, Fc.z, Fd.x, Fd.y, Fd.z};
#pragma unroll
          for (int c2 = 0; c2 < 12; ++c2) sm.cf[t][c2] = v[c2];
        }
        __syncthreads();
        const int lim = min(TQ, rEnd - base);
        // Row forces: this thread's own entries, in list order.
        const int lo = max(myOff, base), hi = min(myOff + myCnt, base + lim);
        for (int e2 = lo; e2 < hi; ++e2) {
          const float* f = sm.cf[e2 - base];
          f1 = f1 + qf::V3f{f[0], f[1], f[2]};
          f2 = f2 + qf::V3f{f[3], f[4], f[5]};
        }
        // Column forces: the entries whose column is this thread's, in list order.
        for (int q = 0; q < lim; ++q) {
          if ((sm.plist[base - r0 + q] & 0xff) == t) {
            const float* f = sm.cf[q];
            fc3 = fc3 + qf::V3f{f[6], f[7], f[8]};
            fc4 = fc4 + qf::V3f{f[9], f[10], f[11]};
          }
        }
        __syncthreads();
      }
    }

    // ---- Partials: row segments' then column segments' node forces. ----
    double* p = partial + (int64_t)it.x * 12 * TQ;
    const float row[6] = {f1.x, f1.y, f1.z, f2.x, f2.y, f2.z};
    const float colp[6] = {fc3.x, fc3.y, fc3.z, fc4.x, fc4.y, fc4.z};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      p[c * TQ + t] = (double)row[c];
      double v = (double)colp[c];
#pragma unroll
      for (int q = 0; q < NW; ++q) v += (double)sm.sFJ[q][c][t];
      p[(6 + c) * TQ + t] = v;
    }
  }
}

template <int NQ>
cudaError_t set_attr_quad() {
  static std::atomic<uint64_t> done{0};
  return set_smem_once(quad_far_tiles<NQ>, (int)sizeof(QuadSmem), done);
}

}  // namespace

size_t quad_seg_bytes(int64_t npad) { return (size_t)npad * kQsRows * sizeof(float); }

cudaError_t launch_prep_quad_seg(const double* soa, const float* ms, int64_t npad, float* qs, cudaStream_t st) {
  prep_quad_seg<<<(unsigned)((npad + 255) / 256), 256, 0, st>>>(soa, ms, npad, qs);
  return cudaGetLastError();
}

int quad_far_blocks_per_sm(int nq) {
  int per = 0;
  if (nq == 2) {
    if (set_attr_quad<2>() == cudaSuccess)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, quad_far_tiles<2>, TQ, sizeof(QuadSmem));
  } else {
    if (set_attr_quad<3>() == cudaSuccess)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, quad_far_tiles<3>, TQ, sizeof(QuadSmem));
  }
  return per > 0 ? per : 1;
}

cudaError_t launch_quad_far_tiles(const float* ms, const float* qs, const double* soa, int64_t npad, const int4* items,
                                  int32_t nItems, int nq, const KConsts& K, float kappa2, float kappaTwo2,
                                  double* partial, int grid, cudaStream_t st) {
  if (nItems <= 0) return cudaSuccess;
  const qf::QConst Q{(float)K.aSq, (float)K.mu4pi, (float)K.mu4pinu, (float)K.nuMu4pinu, (float)(K.aSq * K.mu8pi)};
  cudaError_t e = nq == 2 ? set_attr_quad<2>() : set_attr_quad<3>();
  if (e != cudaSuccess) return e;
  if (nq == 2)
    quad_far_tiles<2><<<grid, TQ, sizeof(QuadSmem), st>>>(ms, qs, soa, npad, items, nItems, Q, kappa2, kappaTwo2,
                                                                 partial);
  else
    quad_far_tiles<3><<<grid, TQ, sizeof(QuadSmem), st>>>(ms, qs, soa, npad, items, nItems, Q, kappa2, kappaTwo2,
                                                                 partial);
  return cudaGetLastError();
}

}  // namespace ddd
