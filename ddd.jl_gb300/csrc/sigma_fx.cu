// The fast FP64 form of the field-point stress σ̃ (DDD_MODE_FP64_FAST):
// sigma_fx.cuh's regrouped evaluation in sigma_f64.cu's layout.  One thread per
// field point in one-warp CTAs; 32-segment tiles stream through shared memory,
// each segment with its direction, t x b and length computed once per tile;
// each point sums the segments in order (DislocationFEM.jl:129-299's order) and
// writes its six components once.
//
// Compiled with --fmad=false: the only fused operations are sigma_fx.cuh's.
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_f64.cuh"
#include "sigma_fx.cuh"

namespace ddd {

namespace {

constexpr int SIG_TILE = 32;

__global__ void __launch_bounds__(SIG_TILE, 24)
sigma_tilde_fx(sx::KS K, const double* __restrict__ soa, int64_t npad, int64_t nSeg, const double* __restrict__ x0,
               int64_t M, double* __restrict__ sigma) {
  __shared__ double seg[13][SIG_TILE];  // n1 xyz, t xyz, b xyz, t x b xyz, length
  const int t = threadIdx.x;
  const int64_t j = blockIdx.x * (int64_t)SIG_TILE + t;
  sx::X3 x = {0, 0, 0};
  if (j < M) x = {x0[3 * j], x0[3 * j + 1], x0[3 * j + 2]};
  double sig[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t s0 = 0; s0 < nSeg; s0 += SIG_TILE) {
    __syncthreads();
    {
      const int64_t i = s0 + t;  // < npad (a multiple of the tile)
      const double n1x = soa[i], n1y = soa[npad + i], n1z = soa[2 * npad + i];
      const double vx = soa[3 * npad + i] - n1x, vy = soa[4 * npad + i] - n1y, vz = soa[5 * npad + i] - n1z;
      const double bx = soa[6 * npad + i], by = soa[7 * npad + i], bz = soa[8 * npad + i];
      const double tx = soa[9 * npad + i], ty = soa[10 * npad + i], tz = soa[11 * npad + i];
      seg[0][t] = n1x;
      seg[1][t] = n1y;
      seg[2][t] = n1z;
      seg[3][t] = tx;
      seg[4][t] = ty;
      seg[5][t] = tz;
      seg[6][t] = bx;
      seg[7][t] = by;
      seg[8][t] = bz;
      seg[9][t] = fm::fma_(ty, bz, -(tz * by));
      seg[10][t] = fm::fma_(tz, bx, -(tx * bz));
      seg[11][t] = fm::fma_(tx, by, -(ty * bx));
      seg[12][t] = sqrt(fm::fma_(vz, vz, fm::fma_(vy, vy, vx * vx)));
    }
    __syncthreads();
    const int n = (int)min((int64_t)SIG_TILE, nSeg - s0);
    if (j < M) {
      for (int q = 0; q < n; ++q) {
        const sx::SegS sg = {{seg[0][q], seg[1][q], seg[2][q]},
                             {seg[3][q], seg[4][q], seg[5][q]},
                             {seg[6][q], seg[7][q], seg[8][q]},
                             {seg[9][q], seg[10][q], seg[11][q]},
                             seg[12][q]};
        sx::sigma_point(K, sg, x, sig);
      }
    }
  }
  if (j < M) {
#pragma unroll
    for (int c = 0; c < 6; ++c) sigma[6 * j + c] = sig[c];
  }
}

}  // namespace

cudaError_t launch_sigma_fx(const KConsts& K, const double* soa, int64_t npad, int64_t nSeg, const double* x0,
                            int64_t M, double* sigma, cudaStream_t st) {
  if (M == 0) return cudaSuccess;
  const sx::KS KS{K.aSq, K.mu4pi, K.mu4pinu, K.nuMu4pinu, K.aSq * K.mu8pi};
  sigma_tilde_fx<<<(unsigned)((M + SIG_TILE - 1) / SIG_TILE), SIG_TILE, 0, st>>>(KS, soa, npad, nSeg, x0, M, sigma);
  return cudaGetLastError();
}

}  // namespace ddd
