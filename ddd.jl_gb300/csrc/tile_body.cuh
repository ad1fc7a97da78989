// One tile pair of the seg-seg force: the body shared by every seg-seg kernel
// (all-pairs, index rows, batched persistent), templated on
//   T     tile size (segments per side = threads per CTA; 64 or 128),
//   MODE  0 = unordered pairs i < j (both sides' forces), 1 = index rows (all
//         j != i, forces on the row segment only), 2 = the pairs i < j outside
//         the surrogate's trust region (near pairs; forces added to `p`),
//   P     arithmetic policy (FP64, df64, mixed FP32; pair_f64.cuh / pair_df.cuh).
//
// Thread t owns row segment i (registers); the column tile sits in shared
// memory.  At step k thread t pairs with column j = (t + k) mod T, so a warp's
// lanes never share a column and column forces accumulate race-free in
// per-warp shared arrays.  Near-parallel pairs (1 - c^2 <= sqrt(eps)) are only
// flagged during the sweep, then compacted in a fixed order (by row, then by
// step) and evaluated densely, T at a time, with the FP64 calcParSegSegForce.
// The block's partial forces — 6 per row segment, and in MODE 0 6 per column
// segment — are written to `p` as [side][component][T] doubles.  No
// floating-point atomics: the result is deterministic.
//
// In MODE 2 every selected pair goes through the compacted dense pass.  The
// sweep takes the reference's FP64 branch decision for each selected pair and
// compacts the general-branch pairs (policy arithmetic, P::dense_general) and
// the near-parallel ones (FP64) into two runs of the list, so that no warp runs
// both branches.
//
// Data: `soa` is the FP64 structure of arrays (13 rows of npad doubles: n1xyz,
// n2xyz, bxyz, txyz, 1/|l|), `skip` one byte per segment (external or padding).
#pragma once
#include <cstdint>

#include "pair_f64.cuh"
#include "surrogate.cuh"

namespace ddd {

struct TileArgs {
  KConsts K;             // FP64 constants
  const double* soa;     // FP64 SoA
  const uint8_t* skip;   // skip flags
  int64_t npad;          // row stride of the SoA
  const float* soadf;    // df64 SoA (policies that use it)
  const void* kd;        // policy constants (df64 / FP32), device-side copy in the kernel parameters
  const float* ms = nullptr;  // MODES 2-3: FP32 segment data of the trust-region test (surrogate.cuh)
  float farK2 = 0.0f;         // MODES 2-3: kappa^2 of the trust region
};

__device__ __forceinline__ SegF64 tb_load_seg64(const double* __restrict__ soa, int64_t npad, int64_t i) {
  SegF64 s;
  s.n1 = {soa[i], soa[npad + i], soa[2 * npad + i]};
  s.n2 = {soa[3 * npad + i], soa[4 * npad + i], soa[5 * npad + i]};
  s.b = {soa[6 * npad + i], soa[7 * npad + i], soa[8 * npad + i]};
  s.t = {soa[9 * npad + i], soa[10 * npad + i], soa[11 * npad + i]};
  s.tN = soa[12 * npad + i];
  return s;
}

// Shared memory of one tile: the policy's column tile and column accumulators,
// plus the near-parallel compaction state.
template <int T, class P>
struct TileSmemT {
  typename P::template Tile<T> pol;
  double cf[T][12];
  uint16_t plist[T * T];
  int cnt[T];
  uint8_t skip[T];
  int total;
};

template <int T, int MODE, class P>
__device__ __forceinline__ void tile_body(const TileArgs& A, const typename P::Consts& KP, TileSmemT<T, P>& sm,
                                          int64_t iBase, int64_t j0, bool diag, const int64_t* __restrict__ rows,
                                          int64_t nRows, double* __restrict__ p,
                                          unsigned long long* __restrict__ counters) {
  constexpr int NW = T / 32;
  constexpr int CH = T;
  const int t = threadIdx.x;
  const int warp = t >> 5;

  int64_t gi;
  bool iActive;
  if (MODE != 1) {
    gi = iBase + t;
    iActive = A.skip[gi] == 0;
  } else {
    const int64_t r = iBase + t;
    iActive = r < nRows;
    gi = iActive ? rows[r] : 0;
    iActive = iActive && A.skip[gi] == 0;
  }
  constexpr bool CLS = MODE == 2;  // classified mode: dense pass only
  typename P::Seg si;
  if (!CLS) si = P::load_global(A, gi);
  float mi[3] = {0, 0, 0}, Li = 0.0f;
  D3 ti = {0, 0, 0};  // MODE 2: the row's FP64 direction for the branch decision
  if (CLS) {
    const int64_t n = A.npad;
    mi[0] = A.ms[(sur::kMsM + 0) * n + gi];
    mi[1] = A.ms[(sur::kMsM + 1) * n + gi];
    mi[2] = A.ms[(sur::kMsM + 2) * n + gi];
    Li = A.ms[sur::kMsL * n + gi];
    ti = {A.soa[9 * n + gi], A.soa[10 * n + gi], A.soa[11 * n + gi]};
  }

  if (!CLS) {
    P::template load_tile<T>(A, sm.pol, j0, t);
    P::template zero_cols<T>(sm.pol, t);
  }
  sm.skip[t] = A.skip[j0 + t];
  __syncthreads();

  typename P::Acc fi1 = P::acc_zero(), fi2 = P::acc_zero();
  uint32_t pmask[NW], gmask[NW];  // near-parallel pairs; MODE 2: general-branch pairs
#pragma unroll
  for (int w = 0; w < NW; ++w) pmask[w] = gmask[w] = 0;
  unsigned long long nGeneral = 0, nDenseParallel = 0;

  for (int k = 0; k < T; ++k) {
    const int jl = (t + k) & (T - 1);
    bool act = iActive && sm.skip[jl] == 0;
    if (MODE != 1) act = act && (!diag || jl > t);
    if (MODE == 1) act = act && (j0 + jl != gi);
    if (CLS) {
      if (act) {
        const int64_t n = A.npad, gj = j0 + jl;
        float dx, dy, dz;
        const bool far = sur::pair_is_far(mi[0], mi[1], mi[2], Li, A.ms[(sur::kMsM + 0) * n + gj],
                                          A.ms[(sur::kMsM + 1) * n + gj], A.ms[(sur::kMsM + 2) * n + gj],
                                          A.ms[sur::kMsL * n + gj], A.farK2, dx, dy, dz);
        if (!far) {
          const D3 tj = {A.soa[9 * n + gj], A.soa[10 * n + gj], A.soa[11 * n + gj]};
          const double c = dot(ti, tj);
          if (1.0 - c * c > kSqrtEps)
            gmask[jl >> 5] |= 1u << (jl & 31);
          else
            pmask[jl >> 5] |= 1u << (jl & 31);
        }
      }
    } else if (act) {
      typename P::Seg sj = P::template load_smem<T>(sm.pol, jl);
      typename P::Scalar c;
      if (P::is_general(A, si, sj, gi, j0 + jl, c)) {
        typename P::Vec F1, F2, F3, F4;
        if (MODE == 0) {
          P::template general<true>(KP, A, si, sj, c, F1, F2, F3, F4);
          P::template add_col<T>(sm.pol, warp, jl, F3, F4);
        } else {
          P::template general<false>(KP, A, si, sj, c, F1, F2, F3, F4);
        }
        P::acc_add(fi1, F1);
        P::acc_add(fi2, F2);
        ++nGeneral;
      } else {
        pmask[jl >> 5] |= 1u << (jl & 31);
      }
    }
    __syncwarp();
  }

  // ---- Compact the listed pairs (fixed order: by row, then by step) and
  // evaluate them densely: MODE 2 lists its general-branch pairs first, then its
  // near-parallel ones; the other modes list only near-parallel pairs. ----
  int myCntG = 0, myCnt = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    myCntG += __popc(gmask[w]);
    myCnt += __popc(pmask[w]);
  }
  int myOffG = 0, myOff = 0;
#pragma unroll
  for (int run = CLS ? 0 : 1; run < 2; ++run) {
    sm.cnt[t] = run == 0 ? myCntG : myCnt;
    __syncthreads();
    if (warp == 0) {
      constexpr int PER = T / 32;
      int v[PER];
      int s = 0;
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        v[q] = sm.cnt[PER * t + q];
        s += v[q];
      }
      int incl = s;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(0xffffffffu, incl, o);
        if ((t & 31) >= o) incl += n;
      }
      int excl = incl - s;
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        sm.cnt[PER * t + q] = excl;
        excl += v[q];
      }
    }
    __syncthreads();
    if (run == 0) {
      myOffG = sm.cnt[t];
      if (t == T - 1) sm.total = myOffG + myCntG;
    } else {
      myOff = sm.cnt[t];
    }
    __syncthreads();
  }
  const int nGen = CLS ? sm.total : 0;  // the general run, then the near-parallel run
  myOff += nGen;
  __syncthreads();
  if (t == T - 1) sm.total = myOff + myCnt;
  {
    int og = myOffG, o = myOff;
    for (int k = 0; k < T; ++k) {
      const int jl = (t + k) & (T - 1);
      const uint32_t bit = 1u << (jl & 31);
      if (CLS && (gmask[jl >> 5] & bit)) sm.plist[og++] = (uint16_t)((t << 8) | jl);
      if (pmask[jl >> 5] & bit) sm.plist[o++] = (uint16_t)((t << 8) | jl);
    }
  }
  __syncthreads();
  const int nPar = sm.total;
  D3 fp1 = {0, 0, 0}, fp2 = {0, 0, 0}, fjp3 = {0, 0, 0}, fjp4 = {0, 0, 0};
  unsigned long long nCore = 0;
  // Chunks of CH never straddle the two runs, so a warp runs one branch.
  for (int base = 0; base < nPar;) {
    const bool genRun = base < nGen;
    const int end = genRun ? nGen : nPar;
    const int e = base + t;
    if (e < end) {
      const int il = sm.plist[e] >> 8, jl = sm.plist[e] & 0xff;
      D3 F1, F2, F3 = {0, 0, 0}, F4 = {0, 0, 0};
      if (genRun) {
        P::dense_general(KP, A, iBase + il, j0 + jl, F1, F2, F3, F4);
        ++nGeneral;
      } else {
        SegF64 a = tb_load_seg64(A.soa, A.npad, MODE != 1 ? iBase + il : rows[iBase + il]);
        SegF64 b = tb_load_seg64(A.soa, A.npad, j0 + jl);
        double c = dot(a.t, b.t);
        if (MODE != 1) {
          ++nDenseParallel;
          nCore += parallel_pair<true>(A.K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
        } else {
          nCore += parallel_pair<false>(A.K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
        }
      }
      sm.cf[t][0] = F1.x; sm.cf[t][1] = F1.y; sm.cf[t][2] = F1.z;
      sm.cf[t][3] = F2.x; sm.cf[t][4] = F2.y; sm.cf[t][5] = F2.z;
      sm.cf[t][6] = F3.x; sm.cf[t][7] = F3.y; sm.cf[t][8] = F3.z;
      sm.cf[t][9] = F4.x; sm.cf[t][10] = F4.y; sm.cf[t][11] = F4.z;
    }
    __syncthreads();
    const int lim = min(CH, end - base);
    // This thread's own entries of the chunk: its general run, then its near-parallel run.
    {
      const int lo = max(myOffG, base), hi = min(myOffG + myCntG, base + lim);
      for (int e2 = lo; e2 < hi; ++e2) {
        const double* f = sm.cf[e2 - base];
        fp1 = fp1 + D3{f[0], f[1], f[2]};
        fp2 = fp2 + D3{f[3], f[4], f[5]};
      }
    }
    {
      const int lo = max(myOff, base), hi = min(myOff + myCnt, base + lim);
      for (int e2 = lo; e2 < hi; ++e2) {
        const double* f = sm.cf[e2 - base];
        fp1 = fp1 + D3{f[0], f[1], f[2]};
        fp2 = fp2 + D3{f[3], f[4], f[5]};
      }
    }
    if (MODE != 1) {
      for (int q = 0; q < lim; ++q) {
        if ((sm.plist[base + q] & 0xff) == t) {
          const double* f = sm.cf[q];
          fjp3 = fjp3 + D3{f[6], f[7], f[8]};
          fjp4 = fjp4 + D3{f[9], f[10], f[11]};
        }
      }
    }
    __syncthreads();
    base += lim;
  }

  // ---- Partials: [side][component][T]; side 0 = row segments, 1 = column segments. ----
  if (CLS) {
    const double v[12] = {fp1.x, fp1.y, fp1.z, fp2.x, fp2.y, fp2.z, fjp3.x, fjp3.y, fjp3.z, fjp4.x, fjp4.y, fjp4.z};
#pragma unroll
    for (int c = 0; c < 12; ++c) p[c * T + t] = p[c * T + t] + v[c];
  }
  if (counters && CLS) {
    unsigned long long g = nGeneral, pp = nDenseParallel, cc = nCore;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      g += __shfl_down_sync(0xffffffffu, g, o);
      pp += __shfl_down_sync(0xffffffffu, pp, o);
      cc += __shfl_down_sync(0xffffffffu, cc, o);
    }
    if ((t & 31) == 0) {
      atomicAdd(&counters[0], g);
      atomicAdd(&counters[1], pp);
      atomicAdd(&counters[2], cc);
    }
  }
  if (CLS) return;
  const D3 r1 = P::acc_to_d3(fi1), r2 = P::acc_to_d3(fi2);
  p[0 * T + t] = r1.x + fp1.x;
  p[1 * T + t] = r1.y + fp1.y;
  p[2 * T + t] = r1.z + fp1.z;
  p[3 * T + t] = r2.x + fp2.x;
  p[4 * T + t] = r2.y + fp2.y;
  p[5 * T + t] = r2.z + fp2.z;
  if (MODE == 0) {
    const double add[6] = {fjp3.x, fjp3.y, fjp3.z, fjp4.x, fjp4.y, fjp4.z};
#pragma unroll
    for (int c = 0; c < 6; ++c) p[(6 + c) * T + t] = P::template col_sum<T>(sm.pol, c, t) + add[c];
  }

  if (counters) {
    unsigned long long g = nGeneral, cc = nCore;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      g += __shfl_down_sync(0xffffffffu, g, o);
      cc += __shfl_down_sync(0xffffffffu, cc, o);
    }
    if ((t & 31) == 0) {
      atomicAdd(&counters[0], g);
      atomicAdd(&counters[2], cc);
    }
    if (t == 0) atomicAdd(&counters[1], (unsigned long long)nPar);
  }
}

// ---------------------------------------------------------------------------
// FP64 policy: the reference arithmetic (strict or FMA, by the translation
// unit's compile flags).
struct PolF64 {
  using Seg = SegF64;
  using Scalar = double;
  using Vec = D3;
  using Acc = D3;
  struct Consts {};
  template <int T>
  struct Tile {
    double seg[13][T];
    double fj[T / 32][6][T];
  };
  static __device__ __forceinline__ Seg load_global(const TileArgs& A, int64_t i) {
    return tb_load_seg64(A.soa, A.npad, i);
  }
  template <int T>
  static __device__ __forceinline__ void load_tile(const TileArgs& A, Tile<T>& s, int64_t j0, int t) {
#pragma unroll
    for (int k = 0; k < 13; ++k) s.seg[k][t] = A.soa[k * A.npad + j0 + t];
  }
  template <int T>
  static __device__ __forceinline__ void zero_cols(Tile<T>& s, int t) {
#pragma unroll
    for (int w = 0; w < T / 32; ++w)
#pragma unroll
      for (int c = 0; c < 6; ++c) s.fj[w][c][t] = 0.0;
  }
  template <int T>
  static __device__ __forceinline__ Seg load_smem(const Tile<T>& s, int j) {
    Seg r;
    r.n1 = {s.seg[0][j], s.seg[1][j], s.seg[2][j]};
    r.n2 = {s.seg[3][j], s.seg[4][j], s.seg[5][j]};
    r.b = {s.seg[6][j], s.seg[7][j], s.seg[8][j]};
    r.t = {s.seg[9][j], s.seg[10][j], s.seg[11][j]};
    r.tN = s.seg[12][j];
    return r;
  }
  static __device__ __forceinline__ bool is_general(const TileArgs&, const Seg& a, const Seg& b, int64_t, int64_t,
                                                    double& c) {
    c = dot(a.t, b.t);
    return 1.0 - c * c > kSqrtEps;
  }
  template <bool BOTH>
  static __device__ __forceinline__ void general(const Consts&, const TileArgs& A, const Seg& a, const Seg& b, double c,
                                                 D3& F1, D3& F2, D3& F3, D3& F4) {
    general_pair<true, BOTH>(A.K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
  }
  // Dense pass of the classified modes: one general-branch pair, both sides.
  static __device__ __forceinline__ void dense_general(const Consts& KP, const TileArgs& A, int64_t gi, int64_t gj,
                                                       D3& F1, D3& F2, D3& F3, D3& F4) {
    const SegF64 a = tb_load_seg64(A.soa, A.npad, gi), b = tb_load_seg64(A.soa, A.npad, gj);
    general<true>(KP, A, a, b, dot(a.t, b.t), F1, F2, F3, F4);
  }
  template <int T>
  static __device__ __forceinline__ void add_col(Tile<T>& s, int warp, int j, const D3& F3, const D3& F4) {
    double* fj = &s.fj[warp][0][0];
    fj[0 * T + j] += F3.x;
    fj[1 * T + j] += F3.y;
    fj[2 * T + j] += F3.z;
    fj[3 * T + j] += F4.x;
    fj[4 * T + j] += F4.y;
    fj[5 * T + j] += F4.z;
  }
  static __device__ __forceinline__ D3 acc_zero() { return {0, 0, 0}; }
  static __device__ __forceinline__ void acc_add(D3& a, const D3& v) { a = a + v; }
  static __device__ __forceinline__ D3 acc_to_d3(const D3& a) { return a; }
  template <int T>
  static __device__ __forceinline__ double col_sum(const Tile<T>& s, int c, int t) {
    double v = s.fj[0][c][t];
#pragma unroll
    for (int w = 1; w < T / 32; ++w) v += s.fj[w][c][t];
    return v;
  }
};

}  // namespace ddd
