// FP64 logarithm and arctangent evaluated on the integer pipes, in 64- and
// 128-bit fixed point, with one final rounding to the nearest double.
//
// Why: on GB300 the FP64 pipe retires 2 lanes per SM per clock, the integer
// pipes 64 and the FP32 pipe 128.  The pair kernels are bound by FP64 issue,
// and a table-driven FP64 logarithm costs ~16 FP64 instructions (an
// arctangent ~26).  The same functions in integer arithmetic take ~100 integer
// instructions, which run beside the FP64 work instead of in its place, and
// they are more accurate (one rounding at the end, < 0.51 ulp measured).
//
// Methods (published, restated):
//   log: the table reduction of P. T. P. Tang, ACM TOMS 16 (1990), in fixed
//        point.  x = 2^E m, m in [1, 2); the top 8 fraction bits pick C_j
//        (an 11-bit integer, ~1024/m) so that r = m C_j 2^-10 - 1 is exact in
//        64 bits with |r| <= 2^-8 (for m >= 1.414, m/2 and E + 1 are used, so
//        log never cancels next to x = 1).  log x = E ln2 - ln(C_j/1024 or
//        C_j/512) + log1p(r), log1p(r) = r W(r), W = 1 - r/2 + r^2 Q(r) by the
//        Taylor series to r^8 (truncation < 2^-67 relative).  Next to x = 1
//        (E = 0, C_j = 1024 or 512) the result is r W alone, so its relative
//        accuracy holds however small r is; elsewhere |log x| >= 2^-8 and the
//        sum is formed in 128-bit fixed point (2^-116).
//   atan: atan z = pi/2 - atan(1/z) for |z| > 1 and the addition formula
//        atan w = atan(j/64) + atan((w - j/64)/(1 + w j/64)), written for
//        |z| > 1 as (1 - |z| j/64)/(|z| + j/64) so that one division serves
//        both.  The division is a fixed-point reciprocal: FP32 seed, two
//        Newton steps (~2^-60).  atan u = u - u^3 B(u^2) with |u| <= 2^-7 and
//        the series to u^9 (truncation < 2^-80).  For |z| < 1/128 the result
//        is |z| (1 - z^2 B(z^2)), relative; for |z| < 2^-27 it is z.
// Out-of-range arguments (log of a non-positive, subnormal, infinite or NaN
// value; atan of an infinity or NaN) go to the standard functions.
//
// Device functions under nvcc; plain inline C++ under a host compiler, which
// gives the same bits (integer arithmetic, and FP32 only in correctly rounded
// operations).
#pragma once
#include <cstdint>

#include "fastmath_f64.cuh"

#ifdef __CUDACC__
#define IM_TABLE_QUAL __device__
#else
#define IM_TABLE_QUAL
#endif

namespace ddd {
namespace im {

typedef unsigned long long u64;
typedef long long i64;
struct im_u128 {
  u64 lo, hi;
};

#include "int_tables.h"

constexpr u64 kSign = 0x8000000000000000ULL;
constexpr u64 kFrac = 0x000FFFFFFFFFFFFFULL;
constexpr u64 kHidden = 0x0010000000000000ULL;
constexpr i64 kThird64 = 6148914691236517205LL;   // 1/3, 2^-64
constexpr i64 kFifth64 = 3689348814741910323LL;   // 1/5, 2^-64

FM_HD u64 umulhi(u64 a, u64 b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (u64)(((unsigned __int128)a * b) >> 64);
#endif
}
FM_HD i64 smulhi(i64 a, i64 b) {
#if defined(__CUDA_ARCH__)
  return __mul64hi(a, b);
#else
  return (i64)(((__int128)a * b) >> 64);
#endif
}
FM_HD unsigned umulhi32(unsigned a, unsigned b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (unsigned)(((u64)a * b) >> 32);
#endif
}
FM_HD int smulhi32(int a, int b) {
#if defined(__CUDA_ARCH__)
  return __mulhi(a, b);
#else
  return (int)(((i64)a * b) >> 32);
#endif
}
FM_HD int clz64(u64 v) {  // v != 0
#if defined(__CUDA_ARCH__)
  return __clzll((i64)v);
#else
  return __builtin_clzll(v);
#endif
}
FM_HD float rcp_rn(float v) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(v);
#else
  return 1.0f / v;
#endif
}
FM_HD unsigned ld32(const unsigned* p) {
#if defined(__CUDA_ARCH__)
  return __ldg(p);
#else
  return *p;
#endif
}
FM_HD im_u128 ld128(const im_u128* p) {
#if defined(__CUDA_ARCH__)
  const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p));
  return {v.x, v.y};
#else
  return *p;
#endif
}
FM_HD unsigned f32_bits(float v) {
#if defined(__CUDA_ARCH__)
  return (unsigned)__float_as_int(v);
#else
  unsigned r;
  std::memcpy(&r, &v, sizeof r);
  return r;
#endif
}

FM_HD void add128(u64& hi, u64& lo, u64 bh, u64 bl) {
  const u64 l = lo + bl;
  hi = hi + bh + (l < lo ? 1ULL : 0ULL);
  lo = l;
}
FM_HD void neg128(u64& hi, u64& lo) {
  lo = ~lo + 1ULL;
  hi = ~hi + (lo == 0 ? 1ULL : 0ULL);
}

// (hi:lo) 2^-scale rounded to the nearest double (ties to even), for
// 0 < hi:lo < 2^127 and a normal result; `sign` is OR'ed into the bits.
FM_HD double to_double(u64 hi, u64 lo, int scale, u64 sign) {
  u64 h, l;
  int lz;
  if (hi != 0) {
    lz = clz64(hi);
    h = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    l = lo << lz;
  } else {
    lz = 64 + clz64(lo);
    h = lo << (lz - 64);
    l = 0;
  }
  const u64 m = h >> 11;  // 53 bits, the leading one at bit 52
  const u64 rest = h & 0x7FFULL;
  const u64 up = (rest > 0x400ULL || (rest == 0x400ULL && (l != 0 || (m & 1ULL)))) ? 1ULL : 0ULL;
  const u64 e = (u64)(127 - lz - scale + 1022);  // biased exponent - 1; the leading one adds 1
  return fm::as_d((i64)(((e << 52) + m + up) | sign));
}

FM_HD double log(double x) {
  const u64 u = (u64)fm::as_ll(x);
  if (u - kHidden >= 0x7FE0000000000000ULL) return fm::std_log(x);  // <= 0, subnormal, inf, NaN
  const int j = (int)((u >> 44) & 0xFFULL);
  const int half = j >= IM_LOG_HALF_J ? 1 : 0;
  const int E = (int)(u >> 52) - 1023 + half;
  const u64 M = (u & kFrac) | kHidden;
  const i64 r = (i64)(M * (u64)ld32(&kILogC[j]) - (1ULL << 62));  // r, 2^-62, |r| < 2^54
  const u64 ar = r < 0 ? (u64)(-r) : (u64)r;
  const u64 a9 = ar << 9;
  const u64 r2 = umulhi(a9, a9);  // r^2, 2^-78 (< 2^62)
  // Q = 1/3 - r/4 + r^2 V, V = 1/5 - r/6 + r^2/7 - r^3/8 (32-bit, 2^-34).
  const int rho = (int)(r >> 24);             // r, 2^-38
  const unsigned r2s = (unsigned)(r2 >> 44);  // r^2, 2^-34
  const unsigned V = 3435973837u - (unsigned)smulhi32(rho, 44739243) + umulhi32(r2s, 613566757u) -
                     (unsigned)(smulhi32((int)r2s, rho) >> 9);
  const unsigned T = umulhi32((unsigned)(r2 >> 30), V);           // r^2 V, 2^-50
  const i64 Q = kThird64 - r + (i64)((u64)T << 14);               // 2^-64
  const i64 r2Q = smulhi((i64)r2, Q);                              // r^2 Q, 2^-78
  const u64 W = (1ULL << 63) - (u64)r + (u64)(r2Q >> 15);         // W = log1p(r)/r, 2^-63
  u64 ph = umulhi(ar, W), pl = ar * W;                             // |r| W, 2^-125
  if (E == 0 && (j == 0 || j == 255)) {  // next to 1: ln C_j = 0
    if (r == 0) return 0.0;
    return to_double(ph, pl, 125, r < 0 ? kSign : 0ULL);
  }
  u64 sh = ph >> 9, sl = (ph << 55) | (pl >> 9);  // 2^-116
  if (r < 0) neg128(sh, sl);
  const im_u128 L = ld128(&kILogL[j]);
  add128(sh, sl, L.hi, L.lo);
  const u64 aE = (u64)(E < 0 ? -E : E);
  u64 eh = aE * kILn2Hi + umulhi(aE, kILn2Lo), el = aE * kILn2Lo;
  if (E < 0) neg128(eh, el);
  add128(sh, sl, eh, el);
  const u64 sign = sh & kSign;
  if (sign) neg128(sh, sl);
  return to_double(sh, sl, 116, sign);
}

// B(u^2) = 1/3 - u^2/5 + u^4/7 - u^6/9 for |u| <= 2^-7 (u2: u^2, 2^-74), 2^-64.
FM_HD i64 atan_series(i64 u2) {
  const unsigned u2s = (unsigned)((u64)u2 >> 29);                              // u^2, 2^-45
  const unsigned u4 = umulhi32(u2s, u2s);                                       // u^4, 2^-58
  const unsigned inner = 2454267026u - (umulhi32(u2s, 1908874354u) >> 13);      // 1/7 - u^2/9, 2^-34
  const unsigned t = umulhi32(u4, inner);                                       // 2^-60
  return kThird64 - (smulhi(u2 << 2, kFifth64) >> 12) + (i64)((u64)t << 4);
}

FM_HD double atan(double z) {
  const u64 u = (u64)fm::as_ll(z);
  const u64 sign = u & kSign;
  const u64 ab = u ^ sign;
  if (ab >= 0x7FF0000000000000ULL) return fm::std_atan(z);  // inf, NaN
  if (ab < 0x3E40000000000000ULL) return z;                  // |z| < 2^-27: atan z rounds to z
  const int Ea = (int)(ab >> 52) - 1023;
  const u64 Ma = (ab & kFrac) | kHidden;
  const bool big = ab > 0x3FF0000000000000ULL;  // |z| > 1
  int j;
  i64 N;   // numerator, 2^-62
  u64 D;   // denominator, 2^-60, in [1, 3)
  if (!big) {
    if (Ea < -7) {
      j = 0;
    } else {
      const u64 A62 = Ma << (Ea + 10);
      j = (int)((A62 + (1ULL << 55)) >> 56);
    }
    if (j == 0) {  // |z| < 1/128: |z| (1 - z^2 B(z^2)), relative
      const i64 U69 = (i64)(Ea + 17 >= 0 ? Ma << (Ea + 17) : Ma >> -(Ea + 17));
      const i64 u2 = smulhi(U69, U69);                     // z^2, 2^-74
      const i64 zB = smulhi(u2, atan_series(u2)) >> 11;    // z^2 B, 2^-63
      const u64 W = (1ULL << 63) - (u64)zB;
      return to_double(umulhi(Ma, W), Ma * W, 115 - Ea, sign);
    }
    N = (i64)((Ma << (Ea + 10)) - ((u64)j << 56));
    const u64 mj = Ma * (u64)j;
    D = (1ULL << 60) + (Ea + 2 >= 0 ? mj << (Ea + 2) : mj >> -(Ea + 2));
  } else {
    if (Ea >= 7) {
      j = 0;
    } else {  // j = round(64/|z|) from an FP32 reciprocal (any nearby j is exact algebra)
      const float mf = fm::as_f((int)(0x3F800000u | (unsigned)((Ma >> 29) & 0x7FFFFFULL)));
      j = (int)(rcp_rn(mf) * (float)(64 >> Ea) + 0.5f);
    }
    const u64 mj = Ma * (u64)j;
    N = (i64)((Ea <= 62 ? 1ULL << (62 - Ea) : 0ULL) - (mj << 4));
    D = (Ma << 8) + (Ea <= 54 ? (u64)j << (54 - Ea) : 0ULL);
  }
  // Y ~ 1/D: FP32 seed from the top 24 bits of D, two Newton steps (2^-62).
  const int lead = 63 - clz64(D);  // 60 or 61
  const float df = fm::as_f((int)(((unsigned)(127 + lead - 60) << 23) | (unsigned)((D >> (lead - 23)) & 0x7FFFFFULL)));
  const unsigned yb = f32_bits(rcp_rn(df));
  const int ye = (int)(yb >> 23) - 127;  // -2..0
  u64 Y = (u64)((yb & 0x7FFFFFu) | 0x800000u) << (39 + ye);
  const u64 D62 = D << 2;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const i64 e = (i64)((1ULL << 60) - umulhi(D62, Y));  // 1 - D Y, 2^-60
    Y = (u64)((i64)Y + (smulhi((i64)Y, e << 3) << 1));
  }
  const u64 aN = N < 0 ? (u64)(-N) : (u64)N;
  const u64 qh = umulhi(aN, Y), ql = aN * Y;  // |u|, 2^-124
  i64 U69 = (i64)((qh << 9) | (ql >> 55));
  if (N < 0) U69 = -U69;
  const i64 u2 = smulhi(U69, U69);                         // u^2, 2^-74
  const i64 u3 = smulhi(u2, U69);                          // u^3, 2^-79
  const i64 at = U69 - (smulhi(u3, atan_series(u2)) >> 10);  // atan u, 2^-69
  u64 sh = (u64)(at >> 13), sl = (u64)at << 51;            // 2^-120, sign-extended
  if (big) {
    neg128(sh, sl);
    const im_u128 T = ld128(&kIAtanTC[j]);
    add128(sh, sl, T.hi, T.lo);
  } else {
    const im_u128 T = ld128(&kIAtanT[j]);
    add128(sh, sl, T.hi, T.lo);
  }
  return to_double(sh, sl, 120, sign);
}

}  // namespace im
}  // namespace ddd
