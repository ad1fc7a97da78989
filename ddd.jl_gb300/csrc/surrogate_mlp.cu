// Training and batched evaluation of the far-field surrogate MLP
// (16 -> 128 -> 128 -> 128 -> 112, GELU, FP16 operands, FP32 accumulation) and
// its Burgers-vector contraction (surrogate.cuh) on the GPU with the project's
// own kernels: every matrix product is the tcgen05 GEMM (tc_gemm.cu);
// activations, the contraction, losses, transposes, bias gradients and the Adam
// update are small elementwise / reduction kernels here.
//
// Forward (batch B; X [B x 16] FP16: hi and lo parts of the 8 geometric
// features; Bp [B x 16] FP32: the 9 Burgers-vector products):
//   Z_1 = X [W_1 | W_1]^T + b_1 (= (X_hi + X_lo) W_1^T + b_1),
//   Z_l = H_{l-1} W_l^T + b_l,  H_l = GELU(Z_l),  Y = H_3 W_4^T + b_4 (112 wide),
//   out[o] = sum_ac Bp[ac] Y[12 ac + o]  (o < 12).
//   Loss = mean over the 12 outputs of (out - T)^2.
// Backward: dout = 2 (out - T) / (12 B);  dY[12 ac + o] = Bp[ac] dout[o];
//   dW_4 = dY^T H_3 (computed as (H_3^T dY)^T),  dH_l = dZ_{l+1} W_{l+1},
//   dZ_l = dH_l * GELU'(Z_l),  dW_l = dZ_l^T H_{l-1},  db_l = column sums of dZ_l;
//   dW_1 = sum of the two 8-column halves of dZ_1^T X.  Forward GEMM operands are
//   FP16 (weights, activations; the GELU is gelu_h2 of surrogate.cuh, as in the
//   inference kernel), backward GEMM operands BF16 (gradients, and BF16 copies
//   of the weights and of the transposed activations); accumulations, bias
//   grads and Adam are FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <random>
#include <vector>

#include "../../include/ddd_gb300.h"
#include "ddd_internal.h"
#include "surrogate.cuh"
#include "surrogate_state.h"

using namespace ddd::sur;

namespace ddd {
namespace {

// Z += bias (FP32, kept for the backward pass); H = gelu_h2(f16(Z)), two
// adjacent columns per thread (cols even).
__global__ void bias_gelu_fwd(float* __restrict__ Z, const float* __restrict__ bias, __half* __restrict__ H,
                              int64_t rows, int cols) {
  const int64_t i = 2 * (blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
  if (i >= rows * cols) return;
  const int c = (int)(i % cols);
  const float z0 = Z[i] + bias[c], z1 = Z[i + 1] + bias[c + 1];
  Z[i] = z0;
  Z[i + 1] = z1;
  *reinterpret_cast<__half2*>(H + i) = gelu_h2(__floats2half2_rn(z0, z1));
}

// Per sample p: y = Y[p] + b4, out[o] = sum_ac Bp[p][ac] y[12 ac + o].  With T:
// the block's loss partial sum, dout = 2 (out - T) / (12 B) and
// dY[p][12 ac + o] = Bp[p][ac] dout[o] (FP32 and BF16; padding columns 0).
// With O: out into O[p] (16 wide, 12 used).
__global__ void contract(const float* __restrict__ Y, const float* __restrict__ b4, const float* __restrict__ Bp,
                         const float* __restrict__ T, int64_t B, float* __restrict__ O, float* __restrict__ dYf,
                         __nv_bfloat16* __restrict__ dY, double* __restrict__ lossPart) {
  __shared__ double red[256];
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double l = 0.0;
  if (p < B) {
    const float* y = Y + p * kOut;
    float bp[kBProd], out[kUsedOut];
#pragma unroll
    for (int ac = 0; ac < kBProd; ++ac) bp[ac] = Bp[p * kRow + ac];
#pragma unroll
    for (int o = 0; o < kUsedOut; ++o) out[o] = 0.0f;
#pragma unroll
    for (int ac = 0; ac < kBProd; ++ac)
#pragma unroll
      for (int o = 0; o < kUsedOut; ++o) out[o] += bp[ac] * (y[kUsedOut * ac + o] + b4[kUsedOut * ac + o]);
    if (O)
#pragma unroll
      for (int o = 0; o < kRow; ++o) O[p * kRow + o] = o < kUsedOut ? out[o] : 0.0f;
    if (T) {
      float g[kUsedOut];
#pragma unroll
      for (int o = 0; o < kUsedOut; ++o) {
        const float d = out[o] - T[p * kRow + o];
        l += (double)d * d;
        g[o] = 2.0f * d / (12.0f * (float)B);
      }
#pragma unroll
      for (int ac = 0; ac < kBProd; ++ac)
#pragma unroll
        for (int o = 0; o < kUsedOut; ++o) {
          const float v = bp[ac] * g[o];
          dYf[p * kOut + kUsedOut * ac + o] = v;
          dY[p * kOut + kUsedOut * ac + o] = __float2bfloat16_rn(v);
        }
      for (int j = kCoef; j < kOut; ++j) {
        dYf[p * kOut + j] = 0.0f;
        dY[p * kOut + j] = __float2bfloat16_rn(0.0f);
      }
    }
  }
  if (!lossPart) return;
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) lossPart[blockIdx.x] = red[0];
}

__global__ void sum_doubles(const double* __restrict__ v, int n, double scale, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += v[i];
    *out += s * scale;
  }
}

__global__ void gelu_bwd(const float* __restrict__ dH, const float* __restrict__ Z, __nv_bfloat16* __restrict__ dZ,
                         float* __restrict__ dZf, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = dH[i] * gelu_grad(Z[i]);
  dZ[i] = __float2bfloat16_rn(g);
  dZf[i] = g;
}

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
template <class T>
__device__ __forceinline__ T from_f(float v);
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// out[C x R] = in[R x C]^T converted to BF16 (BF16 copies exact; FP16 / FP32
// values rounded), 32 x 32 tiles through shared memory.
template <class Tin>
__global__ void transpose_to_bf16(const Tin* __restrict__ in, __nv_bfloat16* __restrict__ out, int64_t R, int C) {
  __shared__ float tile[32][33];
  const int64_t r0 = blockIdx.x * 32;
  const int c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + k;
    const int c = c0 + threadIdx.x;
    if (r < R && c < C) tile[k][threadIdx.x] = to_f(in[r * C + c]);
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k;
    const int64_t r = r0 + threadIdx.x;
    if (r < R && c < C) out[(int64_t)c * R + r] = from_f<__nv_bfloat16>(tile[threadIdx.x][k]);
  }
}

__global__ void f32_to_f16(const float* __restrict__ in, __half* __restrict__ out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2half_rn(in[i]);
}

// [W1 | W1] (128 x 16 FP16) from W1 (128 x 8 FP32): the layer-1 weights of the
// hi / lo feature columns.
__global__ void w1_dup(const float* __restrict__ W1, __half* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kHidden * kGeo) return;
  const int o = i / kGeo, k = i % kGeo;
  const __half w = __float2half_rn(W1[i]);
  out[o * kFeatIn + k] = w;
  out[o * kFeatIn + kGeo + k] = w;
}

// Layer-1 weight gradient: the hi and lo columns' halves of dW1 [128 x 16] summed.
__global__ void w1_fold(const float* __restrict__ g16, float* __restrict__ g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kHidden * kGeo) return;
  const int o = i / kGeo, k = i % kGeo;
  g[i] = g16[o * kFeatIn + k] + g16[o * kFeatIn + kGeo + k];
}

// Column sums of a [rows x cols] FP32 matrix into out[cols], fixed order: block
// b sums rows [b*chunk, (b+1)*chunk) into part[b][cols]; then one pass over b.
__global__ void colsum_part(const float* __restrict__ m, int64_t rows, int cols, int64_t chunk,
                            float* __restrict__ part) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  const int64_t r0 = blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
  float s = 0.0f;
  for (int64_t r = r0; r < r1; ++r) s += m[r * cols + c];
  part[(int64_t)blockIdx.x * cols + c] = s;
}
__global__ void colsum_final(const float* __restrict__ part, int nparts, int cols, float* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  float s = 0.0f;
  for (int b = 0; b < nparts; ++b) s += part[(int64_t)b * cols + c];
  out[c] = s;
}

// grad[out x in] = gT[in x out]^T (FP32), for W4 (computed as H3^T dY).
__global__ void transpose_f32_small(const float* __restrict__ gT, float* __restrict__ g, int inDim, int outDim) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= inDim * outDim) return;
  const int o = i / inDim, k = i % inDim;
  g[i] = gT[k * outDim + o];
}

__global__ void adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                     int n, float lr, float b1, float b2, float eps, float bc1, float bc2, float wd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] + wd * p[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace
}  // namespace ddd

using namespace ddd;

namespace {

template <class T>
cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, n * sizeof(T));
}

cudaError_t ensure_batch(ddd_surrogate* s, int64_t B) {
  if (B <= s->cap) return cudaSuccess;
  for (void* p : {(void*)s->Z1, (void*)s->Z2, (void*)s->Z3, (void*)s->Y, (void*)s->dH, (void*)s->dZf, (void*)s->dYf,
                  (void*)s->H1, (void*)s->H2, (void*)s->H3, (void*)s->dY, (void*)s->dZ, (void*)s->AT, (void*)s->BT,
                  (void*)s->colpart, (void*)s->lossPart})
    if (p) cudaFree(p);
  cudaError_t e = cudaSuccess;
  const size_t h = (size_t)B * kHidden;
  if (e == cudaSuccess) e = dalloc(&s->Z1, h);
  if (e == cudaSuccess) e = dalloc(&s->Z2, h);
  if (e == cudaSuccess) e = dalloc(&s->Z3, h);
  if (e == cudaSuccess) e = dalloc(&s->Y, (size_t)B * kOut);
  if (e == cudaSuccess) e = dalloc(&s->dH, h);
  if (e == cudaSuccess) e = dalloc(&s->dZf, h);
  if (e == cudaSuccess) e = dalloc(&s->dYf, (size_t)B * kOut);
  if (e == cudaSuccess) e = dalloc(&s->H1, h);
  if (e == cudaSuccess) e = dalloc(&s->H2, h);
  if (e == cudaSuccess) e = dalloc(&s->H3, h);
  if (e == cudaSuccess) e = dalloc(&s->dY, (size_t)B * kOut);
  if (e == cudaSuccess) e = dalloc(&s->dZ, h);
  if (e == cudaSuccess) e = dalloc(&s->AT, h);
  if (e == cudaSuccess) e = dalloc(&s->BT, h);
  if (e == cudaSuccess) e = dalloc(&s->colpart, (size_t)(B / 128 + 1) * kHidden);
  if (e == cudaSuccess) e = dalloc(&s->lossPart, (size_t)(B / 256 + 1));
  if (e == cudaSuccess) s->cap = B;
  return e;
}

#define RET(x)                             \
  do {                                     \
    cudaError_t _e = (x);                  \
    if (_e != cudaSuccess) return _e;      \
  } while (0)

template <class Tin>
cudaError_t transpose(const Tin* in, __nv_bfloat16* out, int64_t R, int C, cudaStream_t st) {
  transpose_to_bf16<Tin><<<dim3((unsigned)((R + 31) / 32), (unsigned)((C + 31) / 32)), dim3(32, 8), 0, st>>>(in, out, R,
                                                                                                         C);
  return cudaGetLastError();
}

// BF16 weights and transposes from the FP32 master copy.
cudaError_t refresh_weights(ddd_surrogate* s, cudaStream_t st) {
  w1_dup<<<blocks(kHidden * kGeo), 256, 0, st>>>(s->P + kOffW1, s->W1);
  f32_to_f16<<<blocks(kHidden * kHidden), 256, 0, st>>>(s->P + kOffW2, s->W2, kHidden * kHidden);
  f32_to_f16<<<blocks(kHidden * kHidden), 256, 0, st>>>(s->P + kOffW3, s->W3, kHidden * kHidden);
  f32_to_f16<<<blocks(kOut * kHidden), 256, 0, st>>>(s->P + kOffW4, s->W4, kOut * kHidden);
  // BF16 transposes of the FP32 master weights for the backward pass.
  RET(transpose(s->P + kOffW2, s->W2T, kHidden, kHidden, st));
  RET(transpose(s->P + kOffW3, s->W3T, kHidden, kHidden, st));
  RET(transpose(s->P + kOffW4, s->W4T, kOut, kHidden, st));  // [128 x 112]
  return cudaGetLastError();
}

cudaError_t colsum(ddd_surrogate* s, const float* m, int64_t rows, int cols, float* out, cudaStream_t st) {
  const int64_t chunk = 128;
  const int nparts = (int)((rows + chunk - 1) / chunk);
  colsum_part<<<nparts, cols, 0, st>>>(m, rows, cols, chunk, s->colpart);
  colsum_final<<<1, cols, 0, st>>>(s->colpart, nparts, cols, out);
  return cudaGetLastError();
}

// Forward over a batch of B rows (B % 128 == 0): Z/H buffers and Y filled.
cudaError_t forward(ddd_surrogate* s, const __half* X, int64_t B, cudaStream_t st) {
  RET(launch_tc_gemm_f16((int)B, kHidden, kFeatIn, X, s->W1, s->Z1, s->err, st));
  bias_gelu_fwd<<<blocks(B * kHidden / 2), 256, 0, st>>>(s->Z1, s->P + kOffB1, s->H1, B, kHidden);
  RET(launch_tc_gemm_f16((int)B, kHidden, kHidden, s->H1, s->W2, s->Z2, s->err, st));
  bias_gelu_fwd<<<blocks(B * kHidden / 2), 256, 0, st>>>(s->Z2, s->P + kOffB2, s->H2, B, kHidden);
  RET(launch_tc_gemm_f16((int)B, kHidden, kHidden, s->H2, s->W3, s->Z3, s->err, st));
  bias_gelu_fwd<<<blocks(B * kHidden / 2), 256, 0, st>>>(s->Z3, s->P + kOffB3, s->H3, B, kHidden);
  RET(launch_tc_gemm_f16((int)B, kOut, kHidden, s->H3, s->W4, s->Y, s->err, st));
  return cudaGetLastError();
}

// Loss (added into *s->loss, mean over the batch) and gradients into s->G.
cudaError_t backward(ddd_surrogate* s, const __half* X, const float* Bp, const float* T, int64_t B,
                     cudaStream_t st) {
  const int nLoss = (int)blocks(B);
  contract<<<nLoss, 256, 0, st>>>(s->Y, s->P + kOffB4, Bp, T, B, nullptr, s->dYf, s->dY, s->lossPart);
  sum_doubles<<<1, 32, 0, st>>>(s->lossPart, nLoss, 1.0 / (12.0 * (double)B), s->loss);
  // Layer 4: dW4 = (H3^T dY)^T, db4 = colsum(dY).
  RET(transpose(s->H3, s->AT, B, kHidden, st));   // AT = H3^T [128 x B]
  RET(transpose(s->dY, s->BT, B, kOut, st));      // BT = dY^T [112 x B]
  RET(launch_tc_gemm_bf16(kHidden, kOut, (int)B, s->AT, s->BT, s->gT, s->err, st));  // [128 x 112]
  transpose_f32_small<<<blocks(kOut * kHidden), 256, 0, st>>>(s->gT, s->G + kOffW4, kHidden, kOut);
  RET(colsum(s, s->dYf, B, kOut, s->G + kOffB4, st));
  // Layer 3.
  RET(launch_tc_gemm_bf16((int)B, kHidden, kOut, s->dY, s->W4T, s->dH, s->err, st));  // dH3 = dY W4
  gelu_bwd<<<blocks(B * kHidden), 256, 0, st>>>(s->dH, s->Z3, s->dZ, s->dZf, B * kHidden);
  RET(colsum(s, s->dZf, B, kHidden, s->G + kOffB3, st));
  RET(transpose(s->dZ, s->AT, B, kHidden, st));  // dZ3^T
  RET(transpose(s->H2, s->BT, B, kHidden, st));  // H2^T
  RET(launch_tc_gemm_bf16(kHidden, kHidden, (int)B, s->AT, s->BT, s->G + kOffW3, s->err, st));
  // Layer 2 (dH2 = dZ3 W3).
  RET(launch_tc_gemm_bf16((int)B, kHidden, kHidden, s->dZ, s->W3T, s->dH, s->err, st));
  gelu_bwd<<<blocks(B * kHidden), 256, 0, st>>>(s->dH, s->Z2, s->dZ, s->dZf, B * kHidden);
  RET(colsum(s, s->dZf, B, kHidden, s->G + kOffB2, st));
  RET(transpose(s->dZ, s->AT, B, kHidden, st));
  RET(transpose(s->H1, s->BT, B, kHidden, st));
  RET(launch_tc_gemm_bf16(kHidden, kHidden, (int)B, s->AT, s->BT, s->G + kOffW2, s->err, st));
  // Layer 1 (dH1 = dZ2 W2).
  RET(launch_tc_gemm_bf16((int)B, kHidden, kHidden, s->dZ, s->W2T, s->dH, s->err, st));
  gelu_bwd<<<blocks(B * kHidden), 256, 0, st>>>(s->dH, s->Z1, s->dZ, s->dZf, B * kHidden);
  RET(colsum(s, s->dZf, B, kHidden, s->G + kOffB1, st));
  RET(transpose(s->dZ, s->AT, B, kHidden, st));
  RET(transpose(X, s->BT, B, kFeatIn, st));  // X^T [16 x B]
  RET(launch_tc_gemm_bf16(kHidden, kFeatIn, (int)B, s->AT, s->BT, s->gW1, s->err, st));
  w1_fold<<<blocks(kHidden * kGeo), 256, 0, st>>>(s->gW1, s->G + kOffW1);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

ddd_surrogate* ddd_surrogate_create(ddd_ctx* ctx, uint64_t seed) {
  DDD_NVTX("ddd_surrogate_create");
  if (!ctx) return nullptr;
  ddd_surrogate* s = new ddd_surrogate();
  s->device = ddd::ctx_device(ctx);
  bool ok = cudaSetDevice(s->device) == cudaSuccess &&
            cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && dalloc(&s->P, kNumParams) == cudaSuccess && dalloc(&s->G, kNumParams) == cudaSuccess &&
       dalloc(&s->M1, kNumParams) == cudaSuccess && dalloc(&s->M2, kNumParams) == cudaSuccess;
  ok = ok && dalloc(&s->W1, kHidden * kFeatIn) == cudaSuccess && dalloc(&s->gW1, kHidden * kFeatIn) == cudaSuccess && dalloc(&s->W2, kHidden * kHidden) == cudaSuccess &&
       dalloc(&s->W3, kHidden * kHidden) == cudaSuccess && dalloc(&s->W4, kOut * kHidden) == cudaSuccess &&
       dalloc(&s->W2T, kHidden * kHidden) == cudaSuccess && dalloc(&s->W3T, kHidden * kHidden) == cudaSuccess &&
       dalloc(&s->W4T, kHidden * kOut) == cudaSuccess && dalloc(&s->gT, kHidden * kOut) == cudaSuccess &&
       dalloc(&s->loss, 1) == cudaSuccess && dalloc(&s->err, 1) == cudaSuccess;
  if (!ok) {
    ddd_surrogate_destroy(s);
    return nullptr;
  }
  // Glorot-uniform weights, zero biases (host RNG, then one copy).
  std::vector<float> h(kNumParams, 0.0f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int out, int in, int inUsed) {
    const float a = std::sqrt(6.0f / (float)(inUsed + out));
    std::uniform_real_distribution<float> U(-a, a);
    for (int o = 0; o < out; ++o)
      for (int k = 0; k < in; ++k) h[off + o * in + k] = k < inUsed ? U(rng) : 0.0f;
  };
  fill(kOffW1, kHidden, kGeo, kUsedGeo);
  fill(kOffW2, kHidden, kHidden, kHidden);
  fill(kOffW3, kHidden, kHidden, kHidden);
  fill(kOffW4, kOut, kHidden, kHidden);
  for (int o = kCoef; o < kOut; ++o)
    for (int k = 0; k < kHidden; ++k) h[kOffW4 + o * kHidden + k] = 0.0f;
  ok = cudaMemcpy(s->P, h.data(), kNumParams * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemset(s->M1, 0, kNumParams * sizeof(float)) == cudaSuccess &&
       cudaMemset(s->M2, 0, kNumParams * sizeof(float)) == cudaSuccess &&
       cudaMemset(s->G, 0, kNumParams * sizeof(float)) == cudaSuccess &&
       refresh_weights(s, s->own) == cudaSuccess && cudaStreamSynchronize(s->own) == cudaSuccess;
  if (!ok) {
    ddd_surrogate_destroy(s);
    return nullptr;
  }
  return s;
}

void ddd_surrogate_destroy(ddd_surrogate* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->own) cudaStreamSynchronize(s->own);
  ddd::destroy_force_plan(s->plan);
  for (void* p : {(void*)s->P, (void*)s->G, (void*)s->M1, (void*)s->M2, (void*)s->W1, (void*)s->W2, (void*)s->W3,
                  (void*)s->W4, (void*)s->gW1, (void*)s->W2T, (void*)s->W3T, (void*)s->W4T, (void*)s->Z1, (void*)s->Z2,
                  (void*)s->Z3, (void*)s->Y, (void*)s->dH, (void*)s->dZf, (void*)s->dYf, (void*)s->H1, (void*)s->H2,
                  (void*)s->H3, (void*)s->dY, (void*)s->dZ, (void*)s->AT, (void*)s->BT, (void*)s->gT,
                  (void*)s->colpart, (void*)s->lossPart, (void*)s->loss, (void*)s->err})
    if (p) cudaFree(p);
  if (s->own) cudaStreamDestroy(s->own);
  delete s;
}

int ddd_surrogate_params(ddd_surrogate* s, float* host, int set) {
  if (!s || !host) return DDD_EINVAL;
  cudaSetDevice(s->device);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return DDD_EDEVICE;
  if (set) {
    e = cudaMemcpy(s->P, host, kNumParams * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = refresh_weights(s, s->own);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->own);
  } else {
    e = cudaMemcpy(host, s->P, kNumParams * sizeof(float), cudaMemcpyDeviceToHost);
  }
  return e == cudaSuccess ? DDD_OK : DDD_EDEVICE;
}

int ddd_surrogate_num_params(void) { return kNumParams; }

}  // extern "C"

namespace {

// CRC-32 (IEEE 802.3, reflected, polynomial 0xEDB88320; the zlib checksum).
uint32_t crc32_bytes(const unsigned char* p, size_t n) {
  struct Table {
    uint32_t v[256];
    Table() {
      for (uint32_t i = 0; i < 256; ++i) {
        uint32_t c = i;
        for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        v[i] = c;
      }
    }
  };
  static const Table t;  // initialised once, thread-safe (C++11 static local)
  const uint32_t* table = t.v;
  uint32_t c = 0xFFFFFFFFu;
  for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

// Checkpoint layout (little-endian): "DDDGBSUR", u32 version, u32 parameter
// count, f64 kappa, f64 nu, f64 aSq, f32 parameters, u32 CRC-32 of all that
// precedes it.
constexpr char kMagic[8] = {'D', 'D', 'D', 'G', 'B', 'S', 'U', 'R'};
constexpr uint32_t kVersion = 1;
constexpr size_t kHeader = 8 + 4 + 4 + 3 * 8;

template <class T>
void put(std::vector<unsigned char>& b, size_t off, T v) {
  std::memcpy(b.data() + off, &v, sizeof v);
}
template <class T>
T get(const std::vector<unsigned char>& b, size_t off) {
  T v;
  std::memcpy(&v, b.data() + off, sizeof v);
  return v;
}

}  // namespace

extern "C" {

int ddd_surrogate_save(ddd_surrogate* s, const char* path, double kappa, double nu, double aSq) {
  DDD_NVTX("ddd_surrogate_save");
  if (!s || !path) return DDD_EINVAL;
  std::vector<unsigned char> b(kHeader + (size_t)kNumParams * 4 + 4);
  std::memcpy(b.data(), kMagic, 8);
  put<uint32_t>(b, 8, kVersion);
  put<uint32_t>(b, 12, (uint32_t)kNumParams);
  put<double>(b, 16, kappa);
  put<double>(b, 24, nu);
  put<double>(b, 32, aSq);
  const int rc = ddd_surrogate_params(s, reinterpret_cast<float*>(b.data() + kHeader), 0);
  if (rc) return rc;
  put<uint32_t>(b, b.size() - 4, crc32_bytes(b.data(), b.size() - 4));
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    s->lastError = std::string("cannot open for writing: ") + path;
    return DDD_EINVAL;
  }
  const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
  if (std::fclose(f) != 0 || !ok) {
    s->lastError = std::string("write failed: ") + path;
    return DDD_EINVAL;
  }
  return DDD_OK;
}

int ddd_surrogate_load(ddd_surrogate* s, const char* path, double* kappa, double* nu, double* aSq) {
  DDD_NVTX("ddd_surrogate_load");
  if (!s || !path) return DDD_EINVAL;
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    s->lastError = std::string("cannot open: ") + path;
    return DDD_EINVAL;
  }
  std::vector<unsigned char> b;
  unsigned char chunk[65536];
  size_t n;
  while ((n = std::fread(chunk, 1, sizeof chunk, f)) > 0) b.insert(b.end(), chunk, chunk + n);
  std::fclose(f);
  auto bad = [&](const char* why) {
    s->lastError = std::string(why) + ": " + path;
    return DDD_EINVAL;
  };
  if (b.size() < kHeader + 4 || std::memcmp(b.data(), kMagic, 8) != 0) return bad("not a surrogate checkpoint");
  if (get<uint32_t>(b, 8) != kVersion) return bad("unsupported checkpoint version");
  if (get<uint32_t>(b, 12) != (uint32_t)kNumParams || b.size() != kHeader + (size_t)kNumParams * 4 + 4)
    return bad("checkpoint size does not match this network");
  if (crc32_bytes(b.data(), b.size() - 4) != get<uint32_t>(b, b.size() - 4)) return bad("checkpoint CRC mismatch");
  std::vector<float> params((size_t)kNumParams);
  std::memcpy(params.data(), b.data() + kHeader, params.size() * 4);
  const int rc = ddd_surrogate_params(s, params.data(), 1);
  if (rc) return rc;
  if (kappa) *kappa = get<double>(b, 16);
  if (nu) *nu = get<double>(b, 24);
  if (aSq) *aSq = get<double>(b, 32);
  return DDD_OK;
}

// One forward + backward on B rows (B % 128 == 0), no update: loss and
// gradients (flat FP32 layout) copied to the host.
int ddd_surrogate_grads(ddd_surrogate* s, const void* X, const float* Bp, const float* T, int64_t B, double* loss,
                        float* grads) {
  DDD_NVTX("ddd_surrogate_grads");
  if (!s || !X || !Bp || !T || B <= 0 || B % 128) return DDD_EINVAL;
  cudaSetDevice(s->device);
  if (cudaDeviceSynchronize() != cudaSuccess) return DDD_EDEVICE;  // caller's inputs are ready
  cudaStream_t st = s->own;
  cudaError_t e = ensure_batch(s, B);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->loss, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = forward(s, (const __half*)X, B, st);
  if (e == cudaSuccess) e = backward(s, (const __half*)X, Bp, T, B, st);
  int flag = 0;
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, s->loss, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && grads)
    e = cudaMemcpyAsync(grads, s->G, kNumParams * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, s->err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return DDD_EDEVICE;
  return flag ? DDD_ETIMEOUT : DDD_OK;
}

// Adam training over P samples (X [P x 16] BF16, Bp and T [P x 16] FP32,
// device), in batches of B (P % B == 0, B % 128 == 0), `epochs` passes in a
// fixed order; the mean loss of each epoch goes to lossHistory (host, may be NULL).
int ddd_surrogate_train(ddd_surrogate* s, const void* X, const float* Bp, const float* T, int64_t P, int64_t B,
                        int epochs, float lr, float weightDecay, double* lossHistory) {
  DDD_NVTX("ddd_surrogate_train");
  if (!s || !X || !Bp || !T || B <= 0 || B % 128 || P < B || P % B || epochs <= 0) return DDD_EINVAL;
  cudaSetDevice(s->device);
  if (cudaDeviceSynchronize() != cudaSuccess) return DDD_EDEVICE;  // caller's inputs are ready
  cudaStream_t st = s->own;
  cudaError_t e = ensure_batch(s, B);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->err, 0, sizeof(int), st);
  const int64_t nb = P / B;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
    e = cudaMemsetAsync(s->loss, 0, sizeof(double), st);
    // Cosine learning-rate schedule over the epochs.
    const float lre = 0.5f * lr * (1.0f + std::cos(3.14159265f * (float)ep / (float)epochs));
    for (int64_t b = 0; b < nb && e == cudaSuccess; ++b) {
      const __half* xb = (const __half*)X + b * B * kFeatIn;
      const float* bpb = Bp + b * B * kRow;
      const float* tb = T + b * B * kRow;
      e = forward(s, xb, B, st);
      if (e == cudaSuccess) e = backward(s, xb, bpb, tb, B, st);
      if (e != cudaSuccess) break;
      ++s->step;
      const float bc1 = 1.0f - std::pow(b1, (float)s->step), bc2 = 1.0f - std::pow(b2, (float)s->step);
      adam<<<blocks(kNumParams), 256, 0, st>>>(s->P, s->G, s->M1, s->M2, kNumParams, lre, b1, b2, eps, bc1, bc2,
                                               weightDecay);
      e = refresh_weights(s, st);
    }
    if (e == cudaSuccess && lossHistory) {
      double l = 0;
      e = cudaMemcpyAsync(&l, s->loss, sizeof(double), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      lossHistory[ep] = l / (double)nb;
    }
  }
  int flag = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, s->err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return DDD_EDEVICE;
  return flag ? DDD_ETIMEOUT : DDD_OK;
}

// Batched evaluation (P % 128 == 0): O [P x 16] FP32 (device, 12 used) = the
// contracted scaled node forces of the rows of X and Bp.
int ddd_surrogate_forward(ddd_surrogate* s, const void* X, const float* Bp, int64_t P, float* O) {
  DDD_NVTX("ddd_surrogate_forward");
  if (!s || !X || !Bp || !O || P <= 0 || P % 128) return DDD_EINVAL;
  cudaSetDevice(s->device);
  if (cudaDeviceSynchronize() != cudaSuccess) return DDD_EDEVICE;  // caller's inputs are ready
  cudaStream_t st = s->own;
  const int64_t B = P < 65536 ? P : 65536;
  cudaError_t e = ensure_batch(s, B);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->err, 0, sizeof(int), st);
  for (int64_t off = 0; off < P && e == cudaSuccess; off += B) {
    const int64_t b = (P - off) < B ? (P - off) : B;
    e = forward(s, (const __half*)X + off * kFeatIn, b, st);
    if (e != cudaSuccess) break;
    contract<<<blocks(b), 256, 0, st>>>(s->Y, s->P + kOffB4, Bp + off * kRow, nullptr, b, O + off * kRow, nullptr,
                                        nullptr, nullptr);
    e = cudaGetLastError();
  }
  int flag = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, s->err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return DDD_EDEVICE;
  return flag ? DDD_ETIMEOUT : DDD_OK;
}

}  // extern "C"
