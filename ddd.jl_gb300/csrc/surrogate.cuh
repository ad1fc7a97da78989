// Learned far-field surrogate: pair features and output frame.
//
// A far pair (midpoint separation R well above the segment lengths) is
// described in its own frame: e3 along the midpoint separation r = m_j - m_i,
// e1 along the part of t_i perpendicular to e3, e2 = e3 x e1.  Features
// (dimensionless, 13 used of 16):
//   t_i.e1, t_i.e3, t_j.e1, t_j.e2, t_j.e3, b_i.(e1,e2,e3), b_j.(e1,e2,e3),
//   10 L_i/R, 10 L_j/R (scaled to O(0.1-1) like the others).
// Outputs: the four node forces (Fnode1, Fnode2 on segment i, Fnode3, Fnode4 on
// segment j) in the (e1, e2, e3) frame divided by the far-field scale
// mu4pi * L_i * L_j / R^2 (the order of the force between two segments at
// distance R for unit Burgers vectors).  Equivariance under rotations is built
// in; the network only learns the angular and L/R dependence.
#pragma once

namespace ddd {
namespace sur {

constexpr int kFeat = 16;  // padded feature count (K of layer 1)
constexpr int kUsedFeat = 13;
constexpr int kHidden = 128;
constexpr int kOut = 16;  // padded output count (N of layer 4)
constexpr int kUsedOut = 12;

struct Frame {
  float e1[3], e2[3], e3[3];
  float scale;
};

// r: midpoint separation (already in FP32), ti/tj: unit directions, bi/bj:
// Burgers vectors, Li/Lj: lengths, mu4pi: mu / (4 pi).
__host__ __device__ __forceinline__ void pair_features(const float r[3], const float ti[3], const float tj[3],
                                                       const float bi[3], const float bj[3], float Li, float Lj,
                                                       float mu4pi, float* f, Frame& fr) {
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
  f[5] = d(bi, e1);
  f[6] = d(bi, e2);
  f[7] = d(bi, e3);
  f[8] = d(bj, e1);
  f[9] = d(bj, e2);
  f[10] = d(bj, e3);
  f[11] = 10.0f * Li * invR;
  f[12] = 10.0f * Lj * invR;
  f[13] = f[14] = f[15] = 0.0f;
  for (int k = 0; k < 3; ++k) {
    fr.e1[k] = e1[k];
    fr.e2[k] = e2[k];
    fr.e3[k] = e3[k];
  }
  fr.scale = mu4pi * Li * Lj * invR * invR;
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
                                            float mjz, float Lj, float kappa2, float& dx, float& dy, float& dz) {
  dx = __fsub_rn(mjx, mix);
  dy = __fsub_rn(mjy, miy);
  dz = __fsub_rn(mjz, miz);
  const float R2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  const float Lm = fmaxf(Li, Lj);
  return Li > 0.0f && Lj > 0.0f && R2 >= __fmul_rn(kappa2, __fmul_rn(Lm, Lm));
}

// Flat parameter layout (FP32 master copy): W1 [128 x 16], b1 [128],
// W2 [128 x 128], b2, W3 [128 x 128], b3, W4 [16 x 128], b4 [16]; every W is
// [out x in] (row-major, input contiguous).
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHidden * kFeat;
constexpr int kOffW2 = kOffB1 + kHidden;
constexpr int kOffB2 = kOffW2 + kHidden * kHidden;
constexpr int kOffW3 = kOffB2 + kHidden;
constexpr int kOffB3 = kOffW3 + kHidden * kHidden;
constexpr int kOffW4 = kOffB3 + kHidden;
constexpr int kOffB4 = kOffW4 + kOut * kHidden;
constexpr int kNumParams = kOffB4 + kOut;

}  // namespace sur
}  // namespace ddd
