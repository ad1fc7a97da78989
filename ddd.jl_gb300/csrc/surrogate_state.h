// State of a surrogate object, shared by the training file (surrogate_mlp.cu)
// and the force path (surrogate_force.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace ddd {
struct SurForcePlan;  // surrogate_force.cu
void destroy_force_plan(SurForcePlan* p);
}  // namespace ddd

struct ddd_surrogate {
  int device = 0;
  cudaStream_t own = nullptr;
  // parameters, gradients, Adam moments (FP32, flat layout of surrogate.cuh)
  float *P = nullptr, *G = nullptr, *M1 = nullptr, *M2 = nullptr;
  // FP16 forward weights [out x in] (W1: [W1 | W1], 128 x 16) and BF16
  // transposes [in x out] for the backward pass
  __half *W1 = nullptr, *W2 = nullptr, *W3 = nullptr, *W4 = nullptr;
  __nv_bfloat16 *W2T = nullptr, *W3T = nullptr, *W4T = nullptr;
  int64_t step = 0;
  // activations for the current batch capacity
  int64_t cap = 0;
  float *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr, *Y = nullptr, *dH = nullptr, *dZf = nullptr, *dYf = nullptr;
  __half *H1 = nullptr, *H2 = nullptr, *H3 = nullptr;  // FP16 activations
  __nv_bfloat16 *dY = nullptr, *dZ = nullptr, *AT = nullptr, *BT = nullptr;
  float *gT = nullptr, *colpart = nullptr;
  float* gW1 = nullptr;  // layer-1 weight gradient before folding, 128 x 16
  double *lossPart = nullptr, *loss = nullptr;
  int* err = nullptr;
  ddd::SurForcePlan* plan = nullptr;  // buffers of the force path, per segment count
  std::string lastError;
};
