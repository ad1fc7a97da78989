// Precision forms of the all-pairs and index-list seg-seg force: the general
// branch (the bulk of the pair arithmetic, ~95% of pairs) in df64 — pairs of
// FP32 on the FP32 pipes, ~48-bit significands — while FP64 is kept for
//   * the near-parallel branch (calcParSegSegForce, the strict FP64 code),
//   * the branch decision (computed in df64, settled in FP64 whenever it falls
//     within 1e-5 of the sqrt(eps) threshold, so pairs take exactly the branch
//     the FP64 kernel gives them),
//   * the per-node accumulation across tiles (partials and reduction in FP64).
// Within a tile a thread's 128 general-pair contributions add in df64.
// Tiling, scheduling, near-parallel compaction and the deterministic
// reduction are those of the FP64 kernel (segseg_f64.cu).
//
// Compiled with --fmad=false: df64 needs exact TwoSum/TwoProd, and the FP64
// near-parallel code then rounds as the strict kernel does.
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_df.cuh"
#include "pair_f64.cuh"

namespace ddd {

namespace {

constexpr int TILE = 128;
constexpr int NWARP = TILE / 32;
constexpr int CHUNK = TILE;
// Band around sqrt(eps) inside which the df64 value of 1 - c^2 is not trusted
// to decide the branch; there the FP64 value decides.
constexpr float kThrHi = 1.4901312e-08f;  // sqrt(eps) * (1 + 1e-5)
constexpr float kThrLo = 1.4901012e-08f;  // sqrt(eps) * (1 - 1e-5)

struct SegDF {
  DV3 b, n1, n2, t;
  df64 tN;
};

// soadf: 26 float rows of npad: row 2k = hi, row 2k+1 = lo of FP64 row k.
__global__ void prep_df(const double* __restrict__ soa, int64_t npad, float* __restrict__ soadf) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= npad) return;
#pragma unroll
  for (int k = 0; k < 13; ++k) {
    df64 v = df_from_double(soa[k * npad + i]);
    soadf[(2 * k) * npad + i] = v.hi;
    soadf[(2 * k + 1) * npad + i] = v.lo;
  }
}

__device__ __forceinline__ SegDF load_seg_df(const float* __restrict__ s, int64_t ld, int64_t i) {
  auto g = [&](int k) { return df64{s[(2 * k) * ld + i], s[(2 * k + 1) * ld + i]}; };
  SegDF r;
  r.n1 = {g(0), g(1), g(2)};
  r.n2 = {g(3), g(4), g(5)};
  r.b = {g(6), g(7), g(8)};
  r.t = {g(9), g(10), g(11)};
  r.tN = g(12);
  return r;
}

__device__ __forceinline__ SegF64 load_seg64(const double* __restrict__ soa, int64_t npad, int64_t i) {
  SegF64 s;
  s.n1 = {soa[i], soa[npad + i], soa[2 * npad + i]};
  s.n2 = {soa[3 * npad + i], soa[4 * npad + i], soa[5 * npad + i]};
  s.b = {soa[6 * npad + i], soa[7 * npad + i], soa[8 * npad + i]};
  s.t = {soa[9 * npad + i], soa[10 * npad + i], soa[11 * npad + i]};
  s.tN = soa[12 * npad + i];
  return s;
}

struct TileSmemDF {
  float seg[26][TILE];
  float2 fj[NWARP][6][TILE];
  double cf[CHUNK][12];
  uint16_t plist[TILE * TILE];
  int cnt[TILE];
  uint8_t skip[TILE];
};

__device__ __forceinline__ void tile_index_df(int64_t b, int64_t& I, int64_t& J) {
  int64_t Jc = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while (Jc * (Jc + 1) / 2 > b) --Jc;
  while ((Jc + 1) * (Jc + 2) / 2 <= b) ++Jc;
  J = Jc;
  I = b - Jc * (Jc + 1) / 2;
}

__device__ __forceinline__ void add_df(float2& acc, df64 v) {
  df64 s = df64{acc.x, acc.y} + v;
  acc.x = s.hi;
  acc.y = s.lo;
}

// FORM 0: every general-pair operation in df64.  FORM 1 (mixed): the corner
// antiderivatives and their moments in df64, V-vector assembly and node sums
// in FP32 (general_pair_mixed).
template <int MODE, int FORM>
__global__ void __launch_bounds__(TILE, 2)
segseg_tile_df(KConsts K64, KConstsDF K, KConstsF KF, const double* __restrict__ soa, const float* __restrict__ soadf,
               const uint8_t* __restrict__ skipArr, int64_t npad, const int64_t* __restrict__ rows, int64_t nRows,
               int64_t nJt, double* __restrict__ partial, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmemDF& sm = *reinterpret_cast<TileSmemDF*>(smem_raw);
  const int t = threadIdx.x;
  const int warp = t >> 5;

  int64_t I, J;
  if (MODE == 0) {
    tile_index_df(blockIdx.x, I, J);
  } else {
    I = blockIdx.x / nJt;
    J = blockIdx.x % nJt;
  }
  const bool diag = (MODE == 0) && (I == J);

  int64_t gi;
  bool iActive;
  if (MODE == 0) {
    gi = I * TILE + t;
    iActive = skipArr[gi] == 0;
  } else {
    int64_t r = I * TILE + t;
    iActive = r < nRows;
    gi = iActive ? rows[r] : 0;
    iActive = iActive && skipArr[gi] == 0;
  }
  SegDF si = load_seg_df(soadf, npad, gi);

  const int64_t j0 = J * TILE;
#pragma unroll
  for (int k = 0; k < 26; ++k) sm.seg[k][t] = soadf[k * npad + j0 + t];
  sm.skip[t] = skipArr[j0 + t];
#pragma unroll
  for (int w = 0; w < NWARP; ++w)
#pragma unroll
    for (int c = 0; c < 6; ++c) sm.fj[w][c][t] = make_float2(0.0f, 0.0f);
  __syncthreads();

  DV3 fi1 = {df(0.f), df(0.f), df(0.f)}, fi2 = {df(0.f), df(0.f), df(0.f)};
  uint32_t pmask[TILE / 32] = {0, 0, 0, 0};
  unsigned long long nGeneral = 0;

  for (int k = 0; k < TILE; ++k) {
    const int jl = (t + k) & (TILE - 1);
    bool act = iActive && sm.skip[jl] == 0;
    if (MODE == 0) act = act && (!diag || jl > t);
    if (MODE == 1) act = act && (j0 + jl != gi);
    if (act) {
      SegDF sj;
      {
        auto g = [&](int q) { return df64{sm.seg[2 * q][jl], sm.seg[2 * q + 1][jl]}; };
        sj.n1 = {g(0), g(1), g(2)};
        sj.n2 = {g(3), g(4), g(5)};
        sj.b = {g(6), g(7), g(8)};
        sj.t = {g(9), g(10), g(11)};
        sj.tN = g(12);
      }
      df64 c = dot(si.t, sj.t);
      df64 omc = df(1.0f) - c * c;
      bool general;
      if (omc.hi > kThrHi) {
        general = true;
      } else if (omc.hi < kThrLo) {
        general = false;
      } else {
        // Within the band: the FP64 value of 1 - c^2, as the FP64 kernel computes it.
        D3 ti = {soa[9 * npad + gi], soa[10 * npad + gi], soa[11 * npad + gi]};
        D3 tj = {soa[9 * npad + j0 + jl], soa[10 * npad + j0 + jl], soa[11 * npad + j0 + jl]};
        double c64 = dot(ti, tj);
        general = (1.0 - c64 * c64) > kSqrtEps;
      }
      if (general) {
        DV3 F1, F2, F3, F4;
        if (MODE == 0) {
          if (FORM == 0)
            general_pair_df<true, true>(K, si.b, si.n1, si.n2, si.t, si.tN, sj.b, sj.n1, sj.n2, sj.t, sj.tN, c, F1,
                                        F2, F3, F4);
          else
            general_pair_mixed<true, true, true>(K, KF, f3(si.b), si.n1, si.n2, si.t, si.tN.hi, f3(sj.b), sj.n1,
                                                 sj.n2, sj.t, sj.tN.hi, c, F1, F2, F3, F4);
          add_df(sm.fj[warp][0][jl], F3.x);
          add_df(sm.fj[warp][1][jl], F3.y);
          add_df(sm.fj[warp][2][jl], F3.z);
          add_df(sm.fj[warp][3][jl], F4.x);
          add_df(sm.fj[warp][4][jl], F4.y);
          add_df(sm.fj[warp][5][jl], F4.z);
        } else {
          if (FORM == 0)
            general_pair_df<true, false>(K, si.b, si.n1, si.n2, si.t, si.tN, sj.b, sj.n1, sj.n2, sj.t, sj.tN, c, F1,
                                         F2, F3, F4);
          else
            general_pair_mixed<true, false, true>(K, KF, f3(si.b), si.n1, si.n2, si.t, si.tN.hi, f3(sj.b), sj.n1,
                                                  sj.n2, sj.t, sj.tN.hi, c, F1, F2, F3, F4);
        }
        fi1 = fi1 + F1;
        fi2 = fi2 + F2;
        ++nGeneral;
      } else {
        pmask[jl >> 5] |= 1u << (jl & 31);
      }
    }
    __syncwarp();
  }

  // ---- Near-parallel pairs: compact, then evaluate densely in FP64. ----
  int myCnt = __popc(pmask[0]) + __popc(pmask[1]) + __popc(pmask[2]) + __popc(pmask[3]);
  sm.cnt[t] = myCnt;
  __syncthreads();
  if (warp == 0) {
    int v[4];
    int s = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[q] = sm.cnt[4 * t + q];
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
    for (int q = 0; q < 4; ++q) {
      sm.cnt[4 * t + q] = excl;
      excl += v[q];
    }
  }
  __syncthreads();
  const int myOff = sm.cnt[t];
  __shared__ int sTotal;
  if (t == TILE - 1) sTotal = myOff + myCnt;
  {
    int o = myOff;
    for (int k = 0; k < TILE; ++k) {
      const int jl = (t + k) & (TILE - 1);
      if (pmask[jl >> 5] & (1u << (jl & 31))) sm.plist[o++] = (uint16_t)((t << 8) | jl);
    }
  }
  __syncthreads();
  const int nPar = sTotal;
  D3 fp1 = {0, 0, 0}, fp2 = {0, 0, 0}, fjp3 = {0, 0, 0}, fjp4 = {0, 0, 0};
  unsigned long long nCore = 0;
  for (int base = 0; base < nPar; base += CHUNK) {
    const int e = base + t;
    if (e < nPar) {
      const int il = sm.plist[e] >> 8, jl = sm.plist[e] & 0xff;
      SegF64 a = load_seg64(soa, npad, MODE == 0 ? I * TILE + il : rows[I * TILE + il]);
      SegF64 b = load_seg64(soa, npad, j0 + jl);
      double c = dot(a.t, b.t);
      D3 F1, F2, F3 = {0, 0, 0}, F4 = {0, 0, 0};
      if (MODE == 0)
        nCore += parallel_pair<true>(K64, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
      else
        nCore += parallel_pair<false>(K64, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
      sm.cf[t][0] = F1.x; sm.cf[t][1] = F1.y; sm.cf[t][2] = F1.z;
      sm.cf[t][3] = F2.x; sm.cf[t][4] = F2.y; sm.cf[t][5] = F2.z;
      sm.cf[t][6] = F3.x; sm.cf[t][7] = F3.y; sm.cf[t][8] = F3.z;
      sm.cf[t][9] = F4.x; sm.cf[t][10] = F4.y; sm.cf[t][11] = F4.z;
    }
    __syncthreads();
    const int lim = min(CHUNK, nPar - base);
    int lo = max(myOff, base), hi = min(myOff + myCnt, base + lim);
    for (int e2 = lo; e2 < hi; ++e2) {
      const double* f = sm.cf[e2 - base];
      fp1 = fp1 + D3{f[0], f[1], f[2]};
      fp2 = fp2 + D3{f[3], f[4], f[5]};
    }
    if (MODE == 0) {
      for (int q = 0; q < lim; ++q) {
        if ((sm.plist[base + q] & 0xff) == t) {
          const double* f = sm.cf[q];
          fjp3 = fjp3 + D3{f[6], f[7], f[8]};
          fjp4 = fjp4 + D3{f[9], f[10], f[11]};
        }
      }
    }
    __syncthreads();
  }

  // ---- FP64 partials: df64 tile sums converted, near-parallel sums added. ----
  double* p = partial + (int64_t)blockIdx.x * (MODE == 0 ? 12 : 6) * TILE;
  p[0 * TILE + t] = df_to_double(fi1.x) + fp1.x;
  p[1 * TILE + t] = df_to_double(fi1.y) + fp1.y;
  p[2 * TILE + t] = df_to_double(fi1.z) + fp1.z;
  p[3 * TILE + t] = df_to_double(fi2.x) + fp2.x;
  p[4 * TILE + t] = df_to_double(fi2.y) + fp2.y;
  p[5 * TILE + t] = df_to_double(fi2.z) + fp2.z;
  if (MODE == 0) {
    const double add[6] = {fjp3.x, fjp3.y, fjp3.z, fjp4.x, fjp4.y, fjp4.z};
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < NWARP; ++w) s += (double)sm.fj[w][c][t].x + (double)sm.fj[w][c][t].y;
      p[(6 + c) * TILE + t] = s + add[c];
    }
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

KConstsDF to_df(const KConsts& K) {
  // Host-side split of the FP64 constants into (hi, lo) floats.
  auto s = [](double d) {
    float hi = (float)d;
    return df64{hi, (float)(d - (double)hi)};
  };
  return KConstsDF{s(K.aSq), s(K.mu4pi), s(K.mu4pinu), s(K.mu8piaSq), s(K.mu4pinuaSq)};
}

KConstsF to_f(const KConsts& K) {
  return KConstsF{(float)K.mu4pi, (float)K.mu4pinu, (float)K.mu8piaSq, (float)K.mu4pinuaSq};
}

bool g_attr_df[2][2] = {{false, false}, {false, false}};

template <int MODE, int FORM>
cudaError_t set_attr_df() {
  if (!g_attr_df[MODE][FORM]) {
    cudaError_t e = cudaFuncSetAttribute(segseg_tile_df<MODE, FORM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TileSmemDF));
    if (e != cudaSuccess) return e;
    g_attr_df[MODE][FORM] = true;
  }
  return cudaSuccess;
}

}  // namespace

size_t segseg_df_soa_bytes(int64_t npad) { return (size_t)npad * 26 * sizeof(float); }

cudaError_t launch_prep_df(const double* soa, int64_t npad, float* soadf, cudaStream_t st) {
  prep_df<<<(unsigned)((npad + 255) / 256), 256, 0, st>>>(soa, npad, soadf);
  return cudaGetLastError();
}

cudaError_t launch_segseg_all_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                 int64_t npad, double* partial, double* out, int64_t numSeg,
                                 unsigned long long* counters, cudaStream_t st, int form) {
  cudaError_t e = form ? set_attr_df<0, 1>() : set_attr_df<0, 0>();
  if (e != cudaSuccess) return e;
  const int64_t nt = npad / TILE;
  const int64_t nb = nt * (nt + 1) / 2;
  if (form)
    segseg_tile_df<0, 1><<<(unsigned)nb, TILE, sizeof(TileSmemDF), st>>>(K, to_df(K), to_f(K), soa, soadf, skip, npad,
                                                                         nullptr, 0, 0, partial, counters);
  else
    segseg_tile_df<0, 0><<<(unsigned)nb, TILE, sizeof(TileSmemDF), st>>>(K, to_df(K), to_f(K), soa, soadf, skip, npad,
                                                                         nullptr, 0, 0, partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return strict::launch_reduce_all(partial, npad, numSeg, out, st);
}

cudaError_t launch_segseg_rows_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                  int64_t npad, const int64_t* rows, int64_t nRows, double* partial, double* out,
                                  unsigned long long* counters, cudaStream_t st, int form) {
  cudaError_t e = form ? set_attr_df<1, 1>() : set_attr_df<1, 0>();
  if (e != cudaSuccess) return e;
  const int64_t nJt = npad / TILE;
  const int64_t nrt = (nRows + TILE - 1) / TILE;
  const unsigned grid = (unsigned)(nrt * nJt);
  if (form)
    segseg_tile_df<1, 1><<<grid, TILE, sizeof(TileSmemDF), st>>>(K, to_df(K), to_f(K), soa, soadf, skip, npad, rows,
                                                                 nRows, nJt, partial, counters);
  else
    segseg_tile_df<1, 0><<<grid, TILE, sizeof(TileSmemDF), st>>>(K, to_df(K), to_f(K), soa, soadf, skip, npad, rows,
                                                                 nRows, nJt, partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return strict::launch_reduce_rows(partial, npad, nRows, out, st);
}

}  // namespace ddd
