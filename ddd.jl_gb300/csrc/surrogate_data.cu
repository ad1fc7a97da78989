// Training data of the far-field surrogate: for a list of segment pairs, the
// layer-1 operand (hi and lo FP16 parts of the geometric features), the
// Burgers-vector products, and the exact node forces from the FP64 analytic
// kernel (general or near-parallel branch, DislocationForces.jl :879-1442)
// expressed as the surrogate's scaled local outputs (surrogate.cuh).  Compiled
// with --fmad=false so the forces are the strict FP64 ones.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_f64.cuh"
#include "surrogate.cuh"

namespace ddd {

namespace {

__device__ __forceinline__ SegF64 seg_at(const double* __restrict__ soa, int64_t npad, int64_t i) {
  SegF64 s;
  s.n1 = {soa[i], soa[npad + i], soa[2 * npad + i]};
  s.n2 = {soa[3 * npad + i], soa[4 * npad + i], soa[5 * npad + i]};
  s.b = {soa[6 * npad + i], soa[7 * npad + i], soa[8 * npad + i]};
  s.t = {soa[9 * npad + i], soa[10 * npad + i], soa[11 * npad + i]};
  s.tN = soa[12 * npad + i];
  return s;
}

// pairs: 2 x P int32 (row i, then row j; 0-based segment indices of the SoA).
// X [P x 16] FP16, Bp [P x 16] FP32 (9 used), T [P x 16] FP32 (12 used), F [P x 12].
__global__ void pair_data(KConsts K, const double* __restrict__ soa, int64_t npad, const int32_t* __restrict__ pairs,
                          int64_t P, __half* __restrict__ X, float* __restrict__ Bp, float* __restrict__ T,
                          double* __restrict__ F) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= P) return;
  const SegF64 a = seg_at(soa, npad, pairs[p]);
  const SegF64 b = seg_at(soa, npad, pairs[P + p]);
  const double c = dot(a.t, b.t);
  D3 F1, F2, F3, F4;
  if (1.0 - c * c > kSqrtEps)
    general_pair<true, true>(K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
  else
    parallel_pair<true>(K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
  const D3 ma = 0.5 * (a.n1 + a.n2), mb = 0.5 * (b.n1 + b.n2);
  const D3 rd = mb - ma;
  const float r[3] = {(float)rd.x, (float)rd.y, (float)rd.z};
  const float ti[3] = {(float)a.t.x, (float)a.t.y, (float)a.t.z}, tj[3] = {(float)b.t.x, (float)b.t.y, (float)b.t.z};
  const float bi[3] = {(float)a.b.x, (float)a.b.y, (float)a.b.z}, bj[3] = {(float)b.b.x, (float)b.b.y, (float)b.b.z};
  float f[sur::kGeo], bp[sur::kBProd], row[sur::kFeatIn];
  sur::Frame fr;
  sur::pair_features(r, ti, tj, bi, bj, (float)(1.0 / a.tN), (float)(1.0 / b.tN), (float)K.mu4pi, f, bp, fr);
  sur::split_features(f, row);
#pragma unroll
  for (int k = 0; k < sur::kFeatIn; ++k) X[p * sur::kFeatIn + k] = __float2half_rn(row[k]);
#pragma unroll
  for (int k = 0; k < sur::kRow; ++k) Bp[p * sur::kRow + k] = k < sur::kBProd ? bp[k] : 0.0f;
  const D3 Fs[4] = {F1, F2, F3, F4};
  float* tp = T + p * sur::kRow;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double g[3] = {Fs[q].x, Fs[q].y, Fs[q].z};
    sur::to_local(fr, g, tp + 3 * q);
    if (F) {
      F[p * 12 + 3 * q + 0] = g[0];
      F[p * 12 + 3 * q + 1] = g[1];
      F[p * 12 + 3 * q + 2] = g[2];
    }
  }
#pragma unroll
  for (int k = sur::kUsedOut; k < sur::kRow; ++k) tp[k] = 0.0f;
}

}  // namespace

cudaError_t launch_pair_data(const KConsts& K, const double* soa, int64_t npad, const int32_t* pairs, int64_t P,
                             void* X, float* Bp, float* T, double* F, cudaStream_t st) {
  if (P == 0) return cudaSuccess;
  pair_data<<<(unsigned)((P + 127) / 128), 128, 0, st>>>(K, soa, npad, pairs, P, (__half*)X, Bp, T, F);
  return cudaGetLastError();
}

}  // namespace ddd
