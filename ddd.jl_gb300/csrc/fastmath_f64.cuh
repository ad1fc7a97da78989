// Table-driven FP64 logarithm and arctangent for the fast FP64 pair kernel,
// written in plain IEEE arithmetic (explicit fused multiply-adds, one IEEE
// division in the arctangent) so that a host compiler reproduces the GPU's
// results bit for bit.  Both aim at ~1 ulp, the accuracy the pair formula
// needs: its own rounding noise comes from cancellation across the four
// corners, far above an ulp of one logarithm.
//
// Methods (published, restated):
//   log: P. T. P. Tang, "Table-driven implementation of the logarithm function
//        in IEEE floating-point arithmetic", ACM TOMS 16 (1990): v = 2^k m,
//        m reduced by a table point c_j = 1 + j/256 to r = (m - c_j)/c_j with
//        |r| <= 2^-9, log v = k ln2 + ln c_j + log1p(r), log1p by its Taylor
//        series to r^6 (truncation < 2^-56 relative).  m is kept in
//        [sqrt(1/2), sqrt(2)) (the table then holds ln(c_j / 2) for the upper
//        half) so that k ln2 and ln c_j never cancel near v = 1.  The part of
//        (m - c_j)/c_j lost by rounding r is recovered with one FMA
//        (remainder m - c_j - c_j r) and added to the tail.
//   atan: |z| > 1 by atan z = pi/2 - atan(1/z); the argument (z or 1/z) is
//        reduced by a table point c_j = j/64 through the addition formula
//        atan w = atan c_j + atan((w - c_j)/(1 + w c_j)), written for the
//        |z| > 1 case as (1 - |z| c_j)/(|z| + c_j) so that one division serves
//        both; |u| <= 1/128 and the odd Taylor series to u^7 (truncation
//        < 2^-59 relative).  The table index comes from an FP32 estimate: any
//        nearby index is exact algebra, only |u| depends on it.
// Out-of-range arguments (log of a non-positive, subnormal, infinite or NaN
// value; atan of an infinity or NaN) go to the standard functions.
//
// Device functions under nvcc; plain inline C++ under a host compiler.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define FM_HD __device__ __forceinline__
#define FM_TABLE_QUAL __device__
#else
#include <cmath>
#define FM_HD inline
#define FM_TABLE_QUAL
#endif

namespace ddd {
namespace fm {

struct fm_d2 {
  double hi, lo;
};
struct fm_d3 {
  double c, hi, lo;
};

#include "f64_tables.h"

FM_HD double fma_(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
FM_HD long long as_ll(double v) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(v);
#else
  long long r;
  std::memcpy(&r, &v, sizeof r);
  return r;
#endif
}
FM_HD double as_d(long long v) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(v);
#else
  double r;
  std::memcpy(&r, &v, sizeof r);
  return r;
#endif
}
template <class T>
FM_HD T ld(const T* p) {
#if defined(__CUDA_ARCH__)
  T r;
  if constexpr (sizeof(T) == 8) {
    r = __ldg(reinterpret_cast<const double*>(p));
  } else {
    const double* q = reinterpret_cast<const double*>(p);
    double* s = reinterpret_cast<double*>(&r);
    for (unsigned k = 0; k < sizeof(T) / 8; ++k) s[k] = __ldg(q + k);
  }
  return r;
#else
  return *p;
#endif
}
FM_HD double std_log(double v) { return ::log(v); }
FM_HD double std_atan(double v) { return ::atan(v); }

FM_HD double log(double v) {
  const long long bits = as_ll(v);
  const int hi = (int)(bits >> 32);
  if (hi < 0x00100000 || hi >= 0x7ff00000) return std_log(v);  // <= 0, subnormal, inf, NaN
  const int mh = hi & 0x000FFFFF;
  const int j = (mh + 0x800) >> 12;        // c_j = 1 + j/256 nearest to m = 1 + f
  const bool half = mh >= 0x6A09E;          // m >= sqrt(2): log(m/2) + (k + 1) ln2
  const int k = (hi >> 20) - 1023 + (half ? 1 : 0);
  const double m = as_d((bits & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  const double c = as_d(0x3FF0000000000000LL + ((long long)j << 44));
  const double ic = ld(&kLogInvC[j]);
  const double mc = m - c;                  // exact (Sterbenz)
  const double r = mc * ic;
  const double rl = fma_(-c, r, mc) * ic;   // (m - c - c r) / c
  const fm_d2 T = half ? ld(&kLogHalfC[j]) : ld(&kLogC[j]);
  const double kd = (double)k;
  const double hiP = fma_(kd, FM_LN2_HI, T.hi);  // k * LN2_HI exact
  const double loP = fma_(kd, FM_LN2_LO, T.lo);
  double q = -1.0 / 6.0;
  q = fma_(q, r, 1.0 / 5.0);
  q = fma_(q, r, -0.25);
  q = fma_(q, r, 1.0 / 3.0);
  q = fma_(q, r, -0.5);
  const double tail = fma_(r * r, q, loP + rl);
  return hiP + (r + tail);
}

FM_HD float as_f(int v) {
#if defined(__CUDA_ARCH__)
  return __int_as_float(v);
#else
  float r;
  std::memcpy(&r, &v, sizeof r);
  return r;
#endif
}

FM_HD double atan(double z) {
  const long long bits = as_ll(z);
  const long long sgn = bits & (long long)0x8000000000000000ULL;
  const long long ab = bits ^ sgn;              // |z|; positive doubles order as integers
  if (ab >= 0x7FF0000000000000LL) return std_atan(z);  // inf, NaN
  const double a = as_d(ab);
  const bool big = ab > 0x3FF0000000000000LL;   // |z| > 1
  // FP32 estimate of |z| from its high word (exponent re-biased, 20 mantissa
  // bits, truncated): 0 below the FP32 normal range, infinity above it.
  const int hi = (int)(ab >> 32);
  const int e = (hi >> 20) - 1023;
  const float af = e < -126 ? 0.0f : (e > 127 ? as_f(0x7F800000) : as_f(((e + 127) << 23) | ((hi & 0xFFFFF) << 3)));
#if defined(__CUDA_ARCH__)
  const float w = big ? __frcp_rn(af) : af;  // correctly rounded: the host's 1.0f / af
#else
  const float w = big ? 1.0f / af : af;
#endif
  const int j = (int)(w * 64.0f + 0.5f);    // 0..64
  const fm_d3 T = big ? ld(&kAtanCompC[j]) : ld(&kAtanC[j]);
  const double num = big ? fma_(-a, T.c, 1.0) : a - T.c;
  const double den = big ? a + T.c : fma_(a, T.c, 1.0);
  const double u = num / den;
  const double u2 = u * u;
  double p = fma_(u2, -1.0 / 7.0, 0.2);
  p = fma_(p, u2, -1.0 / 3.0);
  const double s = fma_(u * u2, p, u);      // atan(u)
  const double r = big ? T.hi + (T.lo - s) : T.hi + (T.lo + s);
  return as_d(as_ll(r) ^ sgn);
}

}  // namespace fm
}  // namespace ddd
