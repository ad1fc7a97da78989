// Learned far-field surrogate: pair features, output frame and the bilinear
// Burgers-vector contraction.
//
// A far pair (midpoint separation R well above the segment lengths) is
// described in its own frame: e3 along the midpoint separation r = m_j - m_i,
// e1 along the part of t_i perpendicular to e3, e2 = e3 x e1.
//
// The pair force is exactly bilinear in the two Burgers vectors (the stress of
// segment j is linear in b_j, the Peach-Koehler force on segment i linear in
// b_i), so the network only sees the geometry and the Burgers vectors enter
// through an exact contraction:
//   geometric features (7 used of 8):  t_i.e1, t_i.e3, t_j.e1, t_j.e2, t_j.e3,
//                                      10 L_i / R, 10 L_j / R;
//   network outputs: 108 coefficients C[ac][o] (ac = 3 a + c, o = 0..11);
//   scaled node forces: out[o] = sum_ac (b_i.e_a)(b_j.e_c) C[ac][o].
// out holds the four node forces (Fnode1, Fnode2 on segment i, Fnode3, Fnode4
// on segment j) in the (e1, e2, e3) frame divided by the far-field scale
// mu4pi L_i L_j / R^2.  Rotation equivariance and the Burgers-vector linearity
// are built in; the network learns the angular and L/R dependence.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

namespace ddd {
namespace sur {

constexpr int kGeo = 8;      // geometric features (7 used, padded)
constexpr int kUsedGeo = 7;
// Layer-1 input: each feature as two FP16 numbers, hi = f16(f) and
// lo = f16(f - hi) (columns 0-7 and 8-15), against the weights [W1 | W1]:
// the product sees the features to ~22 significant bits instead of FP16's 11.
// The forward pass runs in FP16 operands (weights and activations) with FP32
// accumulation; the GELU epilogue computes two activations per instruction.
constexpr int kFeatIn = 2 * kGeo;  // 16
constexpr int kHidden = 128;
constexpr int kUsedOut = 12;       // node-force components (4 nodes x 3)
constexpr int kBProd = 9;          // (b_i.e_a)(b_j.e_c)
constexpr int kCoef = kBProd * kUsedOut;  // 108 network outputs used
constexpr int kOut = 112;          // layer-4 width (108 padded to a multiple of 16)
constexpr int kRow = 16;           // padded per-sample row of the b-product and target buffers

struct Frame {
  float e1[3], e2[3], e3[3];
  float scale;
};

// r: midpoint separation (already in FP32), ti/tj: unit directions, bi/bj:
// Burgers vectors, Li/Lj: lengths, mu4pi: mu / (4 pi).  f: the 8 geometric
// features; bp: the 9 Burgers-vector products; fr: the frame and scale.
__host__ __device__ __forceinline__ void pair_features(const float r[3], const float ti[3], const float tj[3],
                                                       const float bi[3], const float bj[3], float Li, float Lj,
                                                       float mu4pi, float* f, float* bp, Frame& fr) {
  const float R2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const float invR = 1.0f / sqrtf(R2);
  float e3[3] = {r[0] * invR, r[1] * invR, r[2] * invR};
  const float a = ti[0] * e3[0] + ti[1] * e3[1] + ti[2] * e3[2];
  float e1[3] = {ti[0] - a * e3[0], ti[1] - a * e3[1], ti[2] - a * e3[2]};
  float n1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  if (n1 < 1e-10f) {
    // t_i along e3: any direction perpendicular to e3.
    const float ax = fabsf(e3[0]) < 0.9f ? 1.0f : 0.0f, ay = 1.0f - ax;
    e1[0] = ay * e3[2];
    e1[1] = -ax * e3[2];
    e1[2] = ax * e3[1] - ay * e3[0];
    n1 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  }
  const float in1 = 1.0f / sqrtf(n1);
  e1[0] *= in1;
  e1[1] *= in1;
  e1[2] *= in1;
  float e2[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
  auto d = [](const float* u, const float* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
  f[0] = d(ti, e1);
  f[1] = a;
  f[2] = d(tj, e1);
  f[3] = d(tj, e2);
  f[4] = d(tj, e3);
  f[5] = 10.0f * Li * invR;
  f[6] = 10.0f * Lj * invR;
  f[7] = 0.0f;
  const float bl[3] = {d(bi, e1), d(bi, e2), d(bi, e3)};
  const float br[3] = {d(bj, e1), d(bj, e2), d(bj, e3)};
  for (int p = 0; p < 3; ++p)
    for (int q = 0; q < 3; ++q) bp[3 * p + q] = bl[p] * br[q];
  for (int k = 0; k < 3; ++k) {
    fr.e1[k] = e1[k];
    fr.e2[k] = e2[k];
    fr.e3[k] = e3[k];
  }
  fr.scale = mu4pi * Li * Lj * invR * invR;
}

// The features of one pair as the layer-1 operand row: hi parts, then lo parts
// (FP32 values that round exactly or to the nearest FP16 when stored).
__device__ __forceinline__ void split_features(const float* f, float* row) {
#pragma unroll
  for (int k = 0; k < kGeo; ++k) {
    const float hi = __half2float(__float2half_rn(f[k]));
    row[k] = hi;
    row[kGeo + k] = f[k] - hi;
  }
}

__device__ __forceinline__ uint32_t h2_bits(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }
__device__ __forceinline__ __half2 bits_h2(uint32_t u) { return *reinterpret_cast<__half2*>(&u); }

// GELU (tanh form) of two FP16 values per instruction: x (x p(x^2)) with
// p = sqrt(2/pi) (1 + 0.044715 x^2), h = 0.5 x (1 + tanh(x p)), the hardware
// FP16 tanh approximation.  Errors are a few FP16 ulps (~1e-3 relative), below
// the rounding of an FP16 activation times the fan-in's averaging; overflow of
// x^2 for |x| > 256 gives tanh = +-1, i.e. h = x or 0, as the exact function.
// The training forward pass and the inference kernel both use this function.
__device__ __forceinline__ __half2 gelu_h2(__half2 x) {
  const __half2 c1 = __float2half2_rn(0.7978845608f);
  const __half2 c2 = __float2half2_rn(0.7978845608f * 0.044715f);
  const __half2 hf = __float2half2_rn(0.5f);
  const __half2 p = __hfma2(c2, __hmul2(x, x), c1);
  uint32_t th;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(th) : "r"(h2_bits(__hmul2(x, p))));
  const __half2 hx = __hmul2(hf, x);
  return __hfma2(hx, bits_h2(th), hx);
}

// 2 GELU(x) = x (1 + tanh(.)) for the inference kernel, whose next-layer
// weights are staged halved: exactly twice gelu_h2's result (the same
// operations on x instead of x / 2), one multiplication fewer.
__device__ __forceinline__ __half2 gelu2_h2(__half2 x) {
  const __half2 c1 = __float2half2_rn(0.7978845608f);
  const __half2 c2 = __float2half2_rn(0.7978845608f * 0.044715f);
  const __half2 p = __hfma2(c2, __hmul2(x, x), c1);
  uint32_t th;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(th) : "r"(h2_bits(__hmul2(x, p))));
  return __hfma2(x, bits_h2(th), x);
}

// Global-frame force from a scaled local output triple.
__host__ __device__ __forceinline__ void to_global(const Frame& fr, const float* y, double* F) {
  for (int k = 0; k < 3; ++k)
    F[k] = (double)fr.scale * ((double)y[0] * fr.e1[k] + (double)y[1] * fr.e2[k] + (double)y[2] * fr.e3[k]);
}

// Scaled local output triple from a global-frame force.
__host__ __device__ __forceinline__ void to_local(const Frame& fr, const double* F, float* y) {
  const double s = 1.0 / (double)fr.scale;
  y[0] = (float)(s * (F[0] * fr.e1[0] + F[1] * fr.e1[1] + F[2] * fr.e1[2]));
  y[1] = (float)(s * (F[0] * fr.e2[0] + F[1] * fr.e2[1] + F[2] * fr.e2[2]));
  y[2] = (float)(s * (F[0] * fr.e3[0] + F[1] * fr.e3[1] + F[2] * fr.e3[2]));
}

// tanh: the hardware approximation on the GPU (max relative error ~2^-11,
// below the BF16 rounding of the activations), libm on a CPU.
__host__ __device__ __forceinline__ float tanh_fast(float x) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
#else
  return tanhf(x);
#endif
}

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
__host__ __device__ __forceinline__ float gelu(float x) {
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  return 0.5f * x * (1.0f + tanh_fast(u));
}
__host__ __device__ __forceinline__ float gelu_grad(float x) {
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  const float th = tanh_fast(u);
  const float du = 0.7978845608028654f * (1.0f + 3.0f * 0.044715f * x * x);
  return 0.5f * (1.0f + th) + 0.5f * x * (1.0f - th * th) * du;
}

// Per-segment data of the force path (10 rows of npad floats, sorted order):
// midpoint xyz, direction xyz, length (0 for an external or padding segment),
// Burgers vector xyz.
constexpr int kMsRows = 10;
constexpr int kMsM = 0, kMsT = 3, kMsL = 6, kMsB = 7;

// Trust region of the surrogate: a pair is evaluated by the network when both
// segments are active and its midpoint separation R satisfies
// R^2 >= kappa^2 max(L_i, L_j)^2.  Every kernel that classifies pairs calls this
// function on the same FP32 data; the explicit round-to-nearest intrinsics keep
// the result identical whatever the contraction flags of the translation unit,
// so each pair is counted by exactly one of the network and the exact pass.
__device__ __forceinline__ bool pair_is_far(float mix, float miy, float miz, float Li, float mjx, float mjy,
                                            float mjz, float Lj, float kappa2, float& dx, float& dy, float& dz,
                                            float& R2, float& Lm2) {
  dx = __fsub_rn(mjx, mix);
  dy = __fsub_rn(mjy, miy);
  dz = __fsub_rn(mjz, miz);
  R2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  const float Lm = fmaxf(Li, Lj);
  Lm2 = __fmul_rn(Lm, Lm);
  return Li > 0.0f && Lj > 0.0f && R2 >= __fmul_rn(kappa2, Lm2);
}
__device__ __forceinline__ bool pair_is_far(float mix, float miy, float miz, float Li, float mjx, float mjy,
                                            float mjz, float Lj, float kappa2, float& dx, float& dy, float& dz) {
  float R2, Lm2;
  return pair_is_far(mix, miy, miz, Li, mjx, mjy, mjz, Lj, kappa2, dx, dy, dz, R2, Lm2);
}

// Flat parameter layout (FP32 master copy): W1 [128 x 8], b1 [128],
// W2 [128 x 128], b2, W3 [128 x 128], b3, W4 [112 x 128], b4 [112]; every W is
// [out x in] (row-major, input contiguous); output row 12 ac + o of W4 / b4 is
// coefficient C[ac][o] (rows 108-111 are padding).
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHidden * kGeo;
constexpr int kOffW2 = kOffB1 + kHidden;
constexpr int kOffB2 = kOffW2 + kHidden * kHidden;
constexpr int kOffW3 = kOffB2 + kHidden;
constexpr int kOffB3 = kOffW3 + kHidden * kHidden;
constexpr int kOffW4 = kOffB3 + kHidden;
constexpr int kOffB4 = kOffW4 + kOut * kHidden;
constexpr int kNumParams = kOffB4 + kOut;

}  // namespace sur
}  // namespace ddd
