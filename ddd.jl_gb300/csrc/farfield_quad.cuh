// Far-field pair force by Gauss-Legendre quadrature on both segments, in FP32.
//
// The force on segment f (nodes n1f, n2f, Burgers b_f, l_f = n2f - n1f) from
// the stress of segment o is the line integral
//   F_k = int_0^1 N_k(xi) (sigma_o(x(xi)) b_f) x l_f dxi,  x(xi) = n1f + xi l_f,
// N_1 = 1 - xi, N_2 = xi (DislocationForces.jl:292-300 for the force density).
// sigma_o is the non-singular stress of segment o (DislocationFEM.jl:135-299):
// with R = x - n1o, s1 = -R.t_o, nd = R - (R.t_o) t_o, A = a^2 + |nd|^2 and
// endpoint functions of s (Ra = sqrt(A + s^2))
//   s03 = s/(Ra A), s13 = -1/Ra, s05 = (2 s03 + s/Ra^3)/A, s15 = -1/Ra^3,
//   s25 = s03 - s/Ra^3,
// sigma = sum_term I_term [s_term(s1 + L_o) - s_term(s1)], the I_term tensors
// built from t_o, nd and b_o.  Each endpoint difference is the integral of
// the s-derivative, and those are free of cancellation:
//   s03' = 1/Ra^3, s13' = s/Ra^3, s05' = 3/Ra^5, s15' = 3s/Ra^5, s25' = 3s^2/Ra^5,
// so for a far pair both integrals go to Gauss-Legendre rules in plain FP32
// (the analytic four-corner form and the endpoint differences cancel as the
// pair separates, which is what the df64 forms pay for).  The I_term tensors
// are contracted with b_f first:
//   V03 = c b_f + mu4pinu (nd (txb.b_f) + txb (nd.b_f)) - mu4pi (t (dxb.b_f) + dxb (t.b_f))
//   V13 = -nu mu4pinu (t (txb.b_f) + txb (t.b_f))
//   V05 = c (a^2 b_f + nd (nd.b_f)) - a^2 mu8pi (t (dxb.b_f) + dxb (t.b_f))
//   V15 = a^2 mu8pi (t (txb.b_f) + txb (t.b_f)) - c (t (nd.b_f) + nd (t.b_f))
//   V25 = c t (t.b_f)
// with t = t_o, txb = t_o x b_o, dxb = nd x b_o, c = mu4pinu (dxb.t_o); then
// sigma b_f = L_o sum_h w_h sum_term s_term'(s1 + L_o xi_h) V_term.
//
// Accuracy (measured against the long-double analytic force, 3-point rules):
// median 1.5e-10 / max 2e-9 relative at R/L = 30, ~1e-8 at R/L = 1000, where
// the analytic FP64 formula itself is off by ~3e-5; the FP32 arithmetic adds
// ~1e-7.  The caller keeps this form to pairs R >= kappa max(L_f, L_o).
//
// Device functions under nvcc; plain inline C++ under a host compiler.
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define QF_HD __host__ __device__ __forceinline__
#else
#define QF_HD inline
#endif

namespace ddd {
namespace qf {

struct QConst {
  float a2, mu4pi, mu4pinu, nuMu4pinu, a2mu8pi;
};

// Gauss-Legendre points and weights on [0, 1].
template <int NQ>
struct Rule;
template <>
struct Rule<2> {
  static QF_HD float x(int i) { return i == 0 ? 0.21132486540518712f : 0.78867513459481288f; }
  static QF_HD float w(int) { return 0.5f; }
};
template <>
struct Rule<3> {
  static QF_HD float x(int i) { return i == 0 ? 0.11270166537925831f : (i == 1 ? 0.5f : 0.88729833462074169f); }
  static QF_HD float w(int i) { return i == 1 ? 0.44444444444444444f : 0.27777777777777778f; }
};

QF_HD float rsqrt_(float v) {
#if defined(__CUDA_ARCH__)
  const float y = rsqrtf(v);
#else
  const float y = 1.0f / std::sqrt(v);
#endif
  return y * (1.5f - 0.5f * v * y * y);  // one Newton step
}

struct V3f {
  float x, y, z;
};
QF_HD V3f operator+(V3f a, V3f b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
QF_HD V3f operator-(V3f a, V3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
QF_HD V3f operator*(float s, V3f a) { return {s * a.x, s * a.y, s * a.z}; }
QF_HD float dot(V3f a, V3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
QF_HD V3f cross(V3f a, V3f b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// Forces on the field segment's two nodes (Fa on n1f, Fb on n2f) from the
// source segment o.  dm = m_f - m_o (midpoint difference, FP32 to ~1e-7
// relative), lf = n2f - n1f, bf its Burgers vector; to, Lo, bo of the source.
template <int NQ>
QF_HD void side(const QConst& K, V3f dm, V3f lf, V3f bf, V3f to, float Lo, V3f bo, V3f& Fa, V3f& Fb) {
  const V3f txb = cross(to, bo);
  const float tb = dot(to, bf), txbb = dot(txb, bf);
  const V3f V13 = (-K.nuMu4pinu) * (txbb * to + tb * txb);
  const V3f T15 = K.a2mu8pi * (txbb * to + tb * txb);  // the t-only part of V15
  const V3f R0 = dm + (0.5f * Lo) * to;              // x - n1o at xi = 1/2
  Fa = {0.f, 0.f, 0.f};
  Fb = {0.f, 0.f, 0.f};
#pragma unroll
  for (int g = 0; g < NQ; ++g) {
    const float xi = Rule<NQ>::x(g);
    const V3f R = R0 + (xi - 0.5f) * lf;
    const float Rdt = dot(R, to);
    const V3f nd = R - Rdt * to;
    const float A = K.a2 + dot(nd, nd);
    const float s1 = -Rdt;
    const V3f dxb = cross(nd, bo);
    const float c = K.mu4pinu * dot(dxb, to);
    const float ndb = dot(nd, bf), dxbb = dot(dxb, bf);
    const V3f tdx = dxbb * to + tb * dxb;
    const V3f V03 = c * bf + K.mu4pinu * (txbb * nd + ndb * txb) - K.mu4pi * tdx;
    const V3f V05 = c * (K.a2 * bf + ndb * nd) - K.a2mu8pi * tdx;
    const V3f V15 = T15 - c * (ndb * to + tb * nd);
    const V3f V25 = (c * tb) * to;
    float S03 = 0.f, S13 = 0.f, S05 = 0.f, S15 = 0.f, S25 = 0.f;
#pragma unroll
    for (int h = 0; h < NQ; ++h) {
      const float s = s1 + Lo * Rule<NQ>::x(h);
      const float ri = rsqrt_(A + s * s);
      const float w3 = Rule<NQ>::w(h) * ri * ri * ri;
      const float w5 = 3.0f * w3 * ri * ri;
      S03 += w3;
      S13 += w3 * s;
      S05 += w5;
      S15 += w5 * s;
      S25 += w5 * s * s;
    }
    const V3f sb = Lo * (S03 * V03 + S13 * V13 + S05 * V05 + S15 * V15 + S25 * V25);
    const V3f f = cross(sb, lf);
    const float w = Rule<NQ>::w(g);
    Fa = Fa + (w * (1.0f - xi)) * f;
    Fb = Fb + (w * xi) * f;
  }
}

}  // namespace qf
}  // namespace ddd
