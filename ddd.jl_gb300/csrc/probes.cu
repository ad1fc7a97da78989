// Pipe-peak probes for the roofline denominators of the FP64 / FP32 kernels.
// Each thread runs 8 independent FMA chains for `iters` iterations; the result
// is stored so the chains cannot be removed.  FLOPs = 2 * 8 * iters * threads.
#include <cuda_runtime.h>

#include "ddd_internal.h"

namespace ddd {

__global__ void fp64_peak_probe(double* sink, int iters) {
  double a[8];
  const double m = 1.0000001, c = 1e-9 * threadIdx.x;
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 0.5 + 0.01 * k + 1e-7 * threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void fp32_peak_probe(float* sink, int iters) {
  float a[8];
  const float m = 1.0000001f, c = 1e-9f * threadIdx.x;
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 0.5f + 0.01f * k + 1e-7f * threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t launch_fp64_peak_probe(double* sink, int iters, int blocks, int threads, cudaStream_t st) {
  fp64_peak_probe<<<blocks, threads, 0, st>>>(sink, iters);
  return cudaGetLastError();
}

cudaError_t launch_fp32_peak_probe(float* sink, int iters, int blocks, int threads, cudaStream_t st) {
  fp32_peak_probe<<<blocks, threads, 0, st>>>(sink, iters);
  return cudaGetLastError();
}

}  // namespace ddd
