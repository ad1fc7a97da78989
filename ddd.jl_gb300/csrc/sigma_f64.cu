// FP64 field-point stress σ̃ (calc_σTilde, DislocationFEM.jl:86-303).
//
// One thread per field point; segments stream through shared memory in tiles
// of SIG_TILE, every thread reading the same segment at the same time (a
// broadcast).  Each point's six components accumulate in registers over the
// segments in list order — the same per-point summation order as the
// reference's segment-outer loop — and are written once (48 B/point), so σ
// never round-trips through memory per segment as it does on the CPU.
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_f64.cuh"

// Compiled twice, like segseg_f64.cu: strict (--fmad=false) and fast (FMA).
#ifndef DDD_VARIANT
#define DDD_VARIANT strict
#endif

namespace ddd {
namespace DDD_VARIANT {

// One warp per CTA: each thread owns a point and the CTA's 32 points share a
// 32-segment tile in shared memory.  Small CTAs spread a small point set evenly
// over the SMs (32,768 points: 1,024 CTAs, 6.7 per SM, where 128-thread CTAs
// left 48 SMs with one CTA and 104 with two); each point still adds the
// segments in order 0..nSeg-1.  24 resident CTAs per SM cap registers at 85,
// the budget the 128-thread form ran at (80).
constexpr int SIG_TILE = 32;

__global__ void __launch_bounds__(SIG_TILE, 24)
sigma_tilde_f64(KConsts K, const double* __restrict__ soa, int64_t npad, int64_t nSeg, const double* __restrict__ x0,
                int64_t M, double* __restrict__ sigma) {
  __shared__ double seg[15][SIG_TILE];  // n1, n2, b, t, t x b
  const int t = threadIdx.x;
  const int64_t j = blockIdx.x * (int64_t)SIG_TILE + t;
  D3 x = {0, 0, 0};
  if (j < M) x = {x0[3 * j], x0[3 * j + 1], x0[3 * j + 2]};
  double sig[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t s0 = 0; s0 < nSeg; s0 += SIG_TILE) {
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 12; ++k) seg[k][t] = soa[k * npad + s0 + t];
    {
      const D3 tx = cross(D3{seg[9][t], seg[10][t], seg[11][t]}, D3{seg[6][t], seg[7][t], seg[8][t]});
      seg[12][t] = tx.x;
      seg[13][t] = tx.y;
      seg[14][t] = tx.z;
    }
    __syncthreads();
    const int n = (int)min((int64_t)SIG_TILE, nSeg - s0);
    if (j < M) {
      for (int q = 0; q < n; ++q) {
        D3 n1 = {seg[0][q], seg[1][q], seg[2][q]};
        D3 n2 = {seg[3][q], seg[4][q], seg[5][q]};
        D3 b = {seg[6][q], seg[7][q], seg[8][q]};
        D3 tt = {seg[9][q], seg[10][q], seg[11][q]};
        D3 txb = {seg[12][q], seg[13][q], seg[14][q]};
        sigma_point(K, b, n1, n2, tt, txb, x, sig);
      }
    }
  }
  if (j < M) {
#pragma unroll
    for (int c = 0; c < 6; ++c) sigma[6 * j + c] = sig[c];
  }
}

cudaError_t launch_sigma_f64(const KConsts& K, const double* soa, int64_t npad, int64_t nSeg, const double* x0,
                             int64_t M, double* sigma, cudaStream_t st) {
  if (M == 0) return cudaSuccess;
  sigma_tilde_f64<<<(unsigned)((M + SIG_TILE - 1) / SIG_TILE), SIG_TILE, 0, st>>>(K, soa, npad, nSeg, x0, M, sigma);
  return cudaGetLastError();
}

}  // namespace DDD_VARIANT
}  // namespace ddd
