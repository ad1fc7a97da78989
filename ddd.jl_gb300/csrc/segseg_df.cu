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
#include "tile_pol_df.cuh"
#include "tile_body.cuh"

namespace ddd {

namespace {

constexpr int TILE = 128;

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

__device__ __forceinline__ void tile_index_df(int64_t b, int64_t& I, int64_t& J) {
  int64_t Jc = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while (Jc * (Jc + 1) / 2 > b) --Jc;
  while ((Jc + 1) * (Jc + 2) / 2 <= b) ++Jc;
  J = Jc;
  I = b - Jc * (Jc + 1) / 2;
}

template <int MODE, int FORM>
__global__ void __launch_bounds__(TILE, 2)
segseg_tile_df(TileArgs A, typename PolDF<FORM>::Consts KP, const int64_t* __restrict__ rows, int64_t nRows,
               int64_t nJt, int64_t base, double* __restrict__ partial, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& sm = *reinterpret_cast<TileSmemT<TILE, PolDF<FORM>>*>(smem_raw);
  int64_t I, J;
  if (MODE == 0) {
    tile_index_df(base + blockIdx.x, I, J);  // slots base.. (a band of J columns)
  } else {
    I = blockIdx.x / nJt;
    J = blockIdx.x % nJt;
  }
  tile_body<TILE, MODE, PolDF<FORM>>(A, KP, sm, I * TILE, J * TILE, MODE == 0 && I == J, rows, nRows,
                                     partial + (int64_t)blockIdx.x * (MODE == 0 ? 12 : 6) * TILE, counters);
}

template <int MODE, int FORM>
cudaError_t set_attr_df() {
  static std::atomic<uint64_t> done{0};
  return set_smem_once(segseg_tile_df<MODE, FORM>, (int)sizeof(TileSmemT<TILE, PolDF<FORM>>), done);
}

// σ̃ in the mixed form (sigma_point_mixed, pair_df.cuh): one thread per point,
// segments streamed through shared memory as df64 pairs (n1, n2, t) and FP32
// (b), six df64 accumulators per point in the segment order of the FP64 kernel.
constexpr int SIG_TILE = 128;
__global__ void __launch_bounds__(SIG_TILE)
sigma_tilde_mixed(KConstsSig K, const float* __restrict__ soadf, int64_t npad, int64_t nSeg,
                  const double* __restrict__ x0, int64_t M, double* __restrict__ sigma) {
  __shared__ float seg[21][SIG_TILE];  // n1 hi/lo (6), n2 hi/lo (6), b hi (3), t hi/lo (6)
  const int t = threadIdx.x;
  const int64_t j = blockIdx.x * (int64_t)SIG_TILE + t;
  DV3 x = {df(0.f), df(0.f), df(0.f)};
  if (j < M) x = {df_from_double(x0[3 * j]), df_from_double(x0[3 * j + 1]), df_from_double(x0[3 * j + 2])};
  df64 sig[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) sig[c] = df(0.f);
  for (int64_t s0 = 0; s0 < nSeg; s0 += SIG_TILE) {
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 12; ++k) seg[k][t] = soadf[k * npad + s0 + t];  // rows 0-11: n1, n2 (hi, lo)
#pragma unroll
    for (int k = 0; k < 3; ++k) seg[12 + k][t] = soadf[(12 + 2 * k) * npad + s0 + t];  // b hi
#pragma unroll
    for (int k = 0; k < 6; ++k) seg[15 + k][t] = soadf[(18 + k) * npad + s0 + t];  // t (hi, lo)
    __syncthreads();
    const int n = (int)min((int64_t)SIG_TILE, nSeg - s0);
    if (j < M) {
      for (int q = 0; q < n; ++q) {
        const DV3 n1 = {df64{seg[0][q], seg[1][q]}, df64{seg[2][q], seg[3][q]}, df64{seg[4][q], seg[5][q]}};
        const DV3 n2 = {df64{seg[6][q], seg[7][q]}, df64{seg[8][q], seg[9][q]}, df64{seg[10][q], seg[11][q]}};
        const F3 b = {seg[12][q], seg[13][q], seg[14][q]};
        const DV3 tt = {df64{seg[15][q], seg[16][q]}, df64{seg[17][q], seg[18][q]}, df64{seg[19][q], seg[20][q]}};
        sigma_point_mixed(K, b, n1, n2, tt, x, sig);
      }
    }
  }
  if (j < M) {
#pragma unroll
    for (int c = 0; c < 6; ++c) sigma[6 * j + c] = df_to_double(sig[c]);
  }
}

}  // namespace

size_t segseg_df_soa_bytes(int64_t npad) { return (size_t)npad * 26 * sizeof(float); }

cudaError_t launch_sigma_mixed(const KConsts& K, const float* soadf, int64_t npad, int64_t nSeg, const double* x0,
                               int64_t M, double* sigma, cudaStream_t st) {
  if (M == 0) return cudaSuccess;
  KConstsSig KS;
  KS.aSq = kconsts_df(K).aSq;
  KS.mu4pi = (float)K.mu4pi;
  KS.mu4pinu = (float)K.mu4pinu;
  KS.nuMu4pinu = (float)K.nuMu4pinu;
  KS.aSq32 = (float)K.aSq;
  KS.aSqMu8pi = (float)(K.aSq * K.mu8pi);
  sigma_tilde_mixed<<<(unsigned)((M + SIG_TILE - 1) / SIG_TILE), SIG_TILE, 0, st>>>(KS, soadf, npad, nSeg, x0, M,
                                                                                     sigma);
  return cudaGetLastError();
}

cudaError_t launch_prep_df(const double* soa, int64_t npad, float* soadf, cudaStream_t st) {
  prep_df<<<(unsigned)((npad + 255) / 256), 256, 0, st>>>(soa, npad, soadf);
  return cudaGetLastError();
}

cudaError_t launch_segseg_all_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                 int64_t npad, double* partial, double* out, int64_t numSeg,
                                 unsigned long long* counters, cudaStream_t st, int form, int64_t capSlots) {
  cudaError_t e = form ? set_attr_df<0, 1>() : set_attr_df<0, 0>();
  if (e != cudaSuccess) return e;
  const int64_t nt = npad / TILE;
  const int64_t nb = nt * (nt + 1) / 2;
  const TileArgs A{K, soa, skip, npad, soadf, nullptr};
  // One launch over all slots, or (partial sums larger than capSlots slots)
  // bands of J columns in order, each reduced into the running output.
  for (int64_t J0 = 0; J0 < nt;) {
    const int64_t J1 = capSlots >= nb ? nt : strict::segseg_band_end(J0, nt, capSlots);
    const int64_t b0 = J0 * (J0 + 1) / 2, nbb = J1 * (J1 + 1) / 2 - b0;
    if (form)
      segseg_tile_df<0, 1><<<(unsigned)nbb, TILE, sizeof(TileSmemT<TILE, PolDF<1>>), st>>>(
          A, PolDF<1>::Consts{kconsts_df(K), kconsts_f(K)}, nullptr, 0, 0, b0, partial, counters);
    else
      segseg_tile_df<0, 0><<<(unsigned)nbb, TILE, sizeof(TileSmemT<TILE, PolDF<0>>), st>>>(
          A, PolDF<0>::Consts{kconsts_df(K), kconsts_f(K)}, nullptr, 0, 0, b0, partial, counters);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = capSlots >= nb ? strict::launch_reduce_all(partial, npad, numSeg, out, st)
                       : strict::launch_reduce_band(partial, J0, J1, numSeg, out, st);
    if (e != cudaSuccess) return e;
    J0 = J1;
  }
  return cudaSuccess;
}

cudaError_t launch_segseg_rows_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                  int64_t npad, const int64_t* rows, int64_t nRows, double* partial, double* out,
                                  unsigned long long* counters, cudaStream_t st, int form) {
  cudaError_t e = form ? set_attr_df<1, 1>() : set_attr_df<1, 0>();
  if (e != cudaSuccess) return e;
  const int64_t nJt = npad / TILE;
  const int64_t nrt = (nRows + TILE - 1) / TILE;
  const unsigned grid = (unsigned)(nrt * nJt);
  const TileArgs A{K, soa, skip, npad, soadf, nullptr};
  if (form)
    segseg_tile_df<1, 1><<<grid, TILE, sizeof(TileSmemT<TILE, PolDF<1>>), st>>>(
        A, PolDF<1>::Consts{kconsts_df(K), kconsts_f(K)}, rows, nRows, nJt, 0, partial, counters);
  else
    segseg_tile_df<1, 0><<<grid, TILE, sizeof(TileSmemT<TILE, PolDF<0>>), st>>>(
        A, PolDF<0>::Consts{kconsts_df(K), kconsts_f(K)}, rows, nRows, nJt, 0, partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return strict::launch_reduce_rows(partial, npad, nRows, out, st);
}

}  // namespace ddd
