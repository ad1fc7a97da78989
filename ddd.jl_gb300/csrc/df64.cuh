// Double-float ("df64") arithmetic on the FP32 pipes: a value is hi + lo with
// |lo| <= ulp(hi)/2, about 48 significant bits.  On GB300 the FP32 pipes issue
// 64x as many operations per clock as the FP64 pipe, so df64 runs the pair
// arithmetic several times faster than native FP64 at ~2^-47 relative precision.
//
// Algorithms (published methods, restated):
//   TwoSum (Knuth), FastTwoSum (Dekker), TwoProd via FMA;
//   add / mul / div / sqrt as in Hida, Li & Bailey, "Library for double-double
//   and quad-double arithmetic" (2001): the "sloppy" or IEEE-style addition,
//   the FMA product, division by two Newton-style corrections, sqrt by one
//   Newton step on an FP32 root;
//   log: x = 2^e m, m reduced by a 64-entry table to m/c_j in [1 - 2^-7, 1 + 2^-7],
//        log(m/c_j) = 2 atanh(u), u = (m - c_j)/(m + c_j), odd series;
//   atan: |x| > 1 folded by atan(x) = pi/2 - atan(1/x), then x = c_j + reduced
//        argument with c_j = j/32, atan(x) = atan(c_j) + atan((x - c_j)/(1 + x c_j)),
//        odd series.
// Compiled with --fmad=false so the error-free transformations stay exact;
// every fused product is an explicit fmaf.
//
// Device functions under nvcc; plain inline C++ under a host compiler, so that
// the same arithmetic can be checked on a CPU against the oracle.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define DF_HD __device__ __forceinline__
#define DDD_DF_TABLE_QUAL __device__
#else
#define DF_HD inline
#define DDD_DF_TABLE_QUAL
#include <cmath>
#endif

namespace ddd {

struct float2_ {
  float x, y;
};

#include "df64_tables.h"

DF_HD float df_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
DF_HD float df_sqrtf(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
// Approximate quotient for the first step of a df64 division (any error < 2^-20 works).
DF_HD float df_qapprox(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
DF_HD int32_t df_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_int(f);
#else
  int32_t i;
  std::memcpy(&i, &f, 4);
  return i;
#endif
}
DF_HD float df_from_bits(int32_t i) {
#if defined(__CUDA_ARCH__)
  return __int_as_float(i);
#else
  float f;
  std::memcpy(&f, &i, 4);
  return f;
#endif
}

struct df64 {
  float hi, lo;
};

DF_HD df64 two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
DF_HD df64 fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}
DF_HD df64 two_prod(float a, float b) {
  float p = a * b;
  float e = df_fma(a, b, -p);
  return {p, e};
}

DF_HD df64 df(float a) { return {a, 0.0f}; }
DF_HD df64 df_from_double(double d) {
  float hi = (float)d;
  float lo = (float)(d - (double)hi);
  return {hi, lo};
}
DF_HD double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

DF_HD df64 operator-(df64 a) { return {-a.hi, -a.lo}; }

// Addition.  DDD_DF_ACCURATE_ADD selects the IEEE-style form (error relative to
// the result); the default is the "sloppy" form (error <= ~2^-47 (|a| + |b|)),
// which is as accurate as the operands themselves whenever they carry their own
// rounding error of that size — every computed df64 value does.
DF_HD df64 operator+(df64 a, df64 b) {
#ifdef DDD_DF_ACCURATE_ADD
  df64 s = two_sum(a.hi, b.hi);
  df64 t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
#else
  df64 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
#endif
}
DF_HD df64 operator-(df64 a, df64 b) { return a + (-b); }
DF_HD df64 operator+(df64 a, float b) {
  df64 s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}
DF_HD df64 operator-(df64 a, float b) { return a + (-b); }
DF_HD df64 operator+(float a, df64 b) { return b + a; }
DF_HD df64 operator-(float a, df64 b) { return (-b) + a; }

DF_HD df64 operator*(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  p.lo = df_fma(a.hi, b.lo, p.lo);
  p.lo = df_fma(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
DF_HD df64 operator*(df64 a, float b) {
  df64 p = two_prod(a.hi, b);
  p.lo = df_fma(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
DF_HD df64 operator*(float a, df64 b) { return b * a; }
// Exact scaling by a power of two.
DF_HD df64 df_scale(df64 a, float p2) { return {a.hi * p2, a.lo * p2}; }

DF_HD df64 operator/(df64 a, df64 b) {
  float q1 = df_qapprox(a.hi, b.hi);
  df64 r = a - b * q1;
  float q2 = df_qapprox(r.hi, b.hi);
  r = r - b * q2;
  float q3 = df_qapprox(r.hi, b.hi);
  df64 q = fast_two_sum(q1, q2);
  return q + q3;
}
DF_HD df64 df_recip(df64 b) { return df(1.0f) / b; }

DF_HD df64 df_sqrt(df64 a) {
  if (!(a.hi > 0.0f)) return {a.hi == 0.0f ? 0.0f : df_sqrtf(a.hi), 0.0f};
  float s = df_sqrtf(a.hi);
  df64 r = a - two_prod(s, s);
  float corr = df_qapprox(r.hi, 2.0f * s);
  return fast_two_sum(s, corr);
}

DF_HD bool operator>(df64 a, df64 b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
DF_HD bool operator<(df64 a, df64 b) { return b > a; }

// Natural logarithm, a > 0 and normal.
DF_HD df64 df_log(df64 a) {
  const int32_t bits = df_bits(a.hi);
  const int32_t e = ((bits >> 23) & 0xff) - 127;
  const int32_t j = (bits >> 17) & 63;            // top 6 mantissa bits
  const float scale = df_from_bits((127 - e) << 23);  // 2^-e, exact
  const df64 m = {a.hi * scale, a.lo * scale};        // m in [1, 2)
  const float c = 1.0f + ((float)j + 0.5f) * 0.015625f;  // exact
  const df64 u = (m - c) / (m + c);                   // |u| < 2^-8
  const df64 u2 = u * u;
  const float t = u2.hi;
  // log(m/c) = 2u + 2u^3 (1/3 + u^2/5 + u^4/7)
  const float tail = t * (0.2f + t * 0.14285714285714285f);
  const df64 P = df64{kDfThird_HI, kDfThird_LO} + tail;
  const df64 r = df_scale(u + u * u2 * P, 2.0f);
  const float2_ lc = kDfLogC[j];
  const df64 le = df64{kDfLn2_HI, kDfLn2_LO} * (float)e;
  return le + (df64{lc.x, lc.y} + r);
}

// Arctangent.
DF_HD df64 df_atan(df64 x) {
  const bool neg = x.hi < 0.0f;
  df64 z = neg ? -x : x;
  const bool inv = z.hi > 1.0f;
  if (inv) z = df_recip(z);
  int j = (int)(z.hi * 32.0f + 0.5f);
  j = j < 0 ? 0 : (j > 32 ? 32 : j);
  const float c = (float)j * 0.03125f;  // exact
  const df64 u = (z - c) / (df(1.0f) + z * c);  // |u| <= 1/64 (slightly more near the fold)
  const df64 u2 = u * u;
  const float t = u2.hi;
  // atan(u) = u + u^3 (-1/3 + u^2/5 - u^4/7 + u^6/9 - u^8/11)
  const float tail = t * (0.2f + t * (-0.14285714285714285f + t * (0.1111111111111111f - t * 0.09090909090909091f)));
  const df64 Q = df64{-kDfThird_HI, -kDfThird_LO} + tail;
  const df64 au = u + u * u2 * Q;
  const float2_ ac = kDfAtanC[j];
  df64 r = df64{ac.x, ac.y} + au;
  if (inv) r = df64{kDfPiHalf_HI, kDfPiHalf_LO} - r;
  return neg ? -r : r;
}

}  // namespace ddd
