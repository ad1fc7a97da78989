// The general branch (1 - c^2 > sqrt(eps)) of the non-singular seg-seg force in
// a reformulated FP64 form that issues fewer FP64 instructions than the
// reference's literal evaluation (pair_f64.cuh), for DDD_MODE_FP64_FAST.
// Same formulas (Arsenlis et al. 2007, App. A.1, as written in DDD.jl
// src/Processing/DislocationForces.jl:879-1165 and :1480-1561); differences:
//   * per corner, one IEEE division instead of four: with R1 = Ra + y + x c,
//     R2 = Ra + x + y c and Q = 1 / (Ra R1 R2), 1/(Ra R1) = Q R2,
//     1/(Ra R2) = Q R1 and 1/Ra = Q (R1 R2); the division by a^2 + d^2(1 - c^2)
//     becomes a product with its reciprocal, taken once per pair;
//   * the logarithms and arctangents are, by the template argument FMATH:
//     the integer-pipe im::log / im::atan (intmath_f64.cuh, kMathInt: they
//     take no FP64 pipe slots and are correctly rounded but for ~1 case in
//     10^3), the FP64 table-driven fm::log / fm::atan (fastmath_f64.cuh,
//     kMathTable) or CUDA's (kMathCuda);
//   * explicit fused multiply-adds (fma_) in the corner terms, the products of
//     unit and Burgers vectors, and the force assembly, which is regrouped on
//     five vectors per side;
//   * the terms whose rounding sets the reference's own error keep its
//     separate rounding: c, 1 - c^2, d, the local coordinates x1, x2, y1, y2
//     (R.t and (lim - c lim) / (1 - c^2)), the argument of Ra, and
//     Ra + y + x c, Ra + x + y c.  Measured on a CPU against long double: with
//     these kept, the node-force error is the reference arithmetic's own
//     (1.00-1.01x); fusing the local coordinates as well makes the result
//     more accurate than the reference (0.6x its error on sparse networks) but
//     moves it ~3e-10 away from the reference's values, past the parity bound.
// Everything else is plain IEEE arithmetic, so the same header compiled for a
// CPU (no contraction) gives the GPU's results bit for bit when FMATH is
// kMathInt or kMathTable.
#pragma once
#include "fastmath_f64.cuh"
#include "intmath_f64.cuh"

namespace ddd {
namespace fx {

struct X3 {
  double x, y, z;
};
FM_HD X3 operator+(X3 a, X3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
FM_HD X3 operator-(X3 a, X3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
FM_HD X3 operator-(X3 a) { return {-a.x, -a.y, -a.z}; }
FM_HD X3 operator*(double s, X3 a) { return {s * a.x, s * a.y, s * a.z}; }
FM_HD X3 operator*(X3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
FM_HD double dot(X3 a, X3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
FM_HD X3 cross(X3 a, X3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// Fused forms: a.b with two FMAs; a x b with one FMA per component.
FM_HD double dotf(X3 a, X3 b) { return fm::fma_(a.z, b.z, fm::fma_(a.y, b.y, a.x * b.x)); }
FM_HD X3 crossf(X3 a, X3 b) {
  return {fm::fma_(a.y, b.z, -(a.z * b.y)), fm::fma_(a.z, b.x, -(a.x * b.z)), fm::fma_(a.x, b.y, -(a.y * b.x))};
}
// s a + v, fused per component.
FM_HD X3 fmv(double s, X3 a, X3 v) { return {fm::fma_(s, a.x, v.x), fm::fma_(s, a.y, v.y), fm::fma_(s, a.z, v.z)}; }
// v with its sign flipped when sm is the sign-bit mask (integer operations).
FM_HD double sgn(double v, long long sm) { return fm::as_d(fm::as_ll(v) ^ sm); }

struct KFast {
  double aSq, mu4pi, mu8pi, mu4pinu, mu8piaSq, mu4pinuaSq;
};

constexpr int kMathCuda = 0, kMathTable = 1, kMathInt = 2;

template <int FMATH>
FM_HD double lg(double v) {
  if (FMATH == kMathInt) return im::log(v);
  if (FMATH == kMathTable) return fm::log(v);
  return fm::std_log(v);
}
template <int FMATH>
FM_HD double at(double v) {
  if (FMATH == kMathInt) return im::atan(v);
  if (FMATH == kMathTable) return fm::atan(v);
  return fm::std_atan(v);
}

// Per-pair constants of the corners: aSq_dSq = a^2 + d^2 (1 - c^2),
// den = 1/sqrt((1 - c^2) aSq_dSq), c2 = 2c, cden = (1 + c) den, m2den = -2 den.
struct CornerK {
  double aSq_dSq, c, cSq, omcSqI, c2, cden, m2den;
};

// SegSegInteg at one corner (DislocationForces.jl:1480-1561), added (sm = 0) or
// subtracted (sm = sign bit) into integ[19]; the first corner (FIRST, sm = 0)
// writes instead of adding to zero.
template <int FMATH, bool FIRST>
FM_HD void corner(const CornerK& P, double x, double y, long long sm, double* integ) {
  const double aSq_dSq = P.aSq_dSq, c = P.c, cSq = P.cSq, omcSqI = P.omcSqI;
  const double xSq = x * x;
  const double ySq = y * y;
  // (x y) (2c) equals the reference's ((2x) y) c bit for bit (scaling by 2 is exact).
  const double Ra = sqrt(aSq_dSq + xSq + ySq + x * y * P.c2);
  const double R1 = Ra + y + x * c;  // Ra_Rd_t1
  const double R2 = Ra + x + y * c;  // Ra_Rd_t2
  const double L1 = lg<FMATH>(R1);
  const double L2 = lg<FMATH>(R2);
  const double R12 = R1 * R2;
  const double Q = 1.0 / (Ra * R12);
  const double RaInv = Q * R12;
  const double S1 = Q * R2;  // RaSq_R_t1_I = 1/(Ra R1)
  const double S2 = Q * R1;  // RaSq_R_t2_I = 1/(Ra R2)
  const double xS1 = x * S1, xxS1 = x * xS1;
  const double yS2 = y * S2, yyS2 = y * yS2;

  const double integ1 = P.m2den * at<FMATH>((Ra + x + y) * P.cden);
  const double c_1 = aSq_dSq * integ1;
  const double c_5_6 = fm::fma_(c, Ra, -c_1) * omcSqI;
  const double integ2 = fm::fma_(c, L2, -L1) * omcSqI;
  const double integ3 = fm::fma_(c, L1, -L2) * omcSqI;
  const double integ4 = fm::fma_(c, c_1, -Ra) * omcSqI;
  const double integ5 = fm::fma_(y, L2, c_5_6);
  const double integ6 = fm::fma_(x, L1, c_5_6);

  const double c_11_12 = fm::fma_(-c, RaInv, integ1);
  const double c_15_18 = fm::fma_(c, xS1, -RaInv);
  const double x_13_14 = x * c_15_18;
  const double c_19 = fm::fma_(c, yS2, -RaInv);
  const double y_13_14 = y * c_19;
  const double c_16 = fm::fma_(-cSq, yyS2, fm::fma_(-(x - c * y), RaInv, L2));
  const double z_15_18 = y * c_16;
  const double c_17_19 = fm::fma_(-cSq, xxS1, fm::fma_(-(y - c * x), RaInv, L1));
  const double c15_18_19 = 2.0 * integ4;

  // integ[6] and integ[7..18] take their numerators: the caller scales the
  // four-corner sums by 1/aSq_dSq and 1/(1 - c^2) once.
  const double v[19] = {integ1,
                        integ2,
                        integ3,
                        integ4,
                        integ5,
                        integ6,
                        integ1 - xS1 - yS2,
                        fm::fma_(-c, S2, S1),
                        fm::fma_(-c, S1, S2),
                        fm::fma_(-c, xS1 + yS2 + integ1, RaInv),
                        fm::fma_(cSq, yS2, xS1 + c_11_12),
                        fm::fma_(cSq, xS1, yS2 + c_11_12),
                        fm::fma_(c, y_13_14 - integ2, integ3 - x_13_14),
                        fm::fma_(c, x_13_14 - integ3, integ2 - y_13_14),
                        fm::fma_(c, fm::fma_(xSq, c_15_18, -c15_18_19), integ5 - z_15_18),
                        fm::fma_(c, c_16, fm::fma_(2.0, integ2, xxS1)),
                        fm::fma_(c, c_17_19, fm::fma_(2.0, integ3, yyS2)),
                        fm::fma_(c, z_15_18 - integ5, fm::fma_(-xSq, c_15_18, c15_18_19)),
                        fm::fma_(c, fm::fma_(x, c_17_19, -integ6), fm::fma_(-ySq, c_19, c15_18_19))};
#pragma unroll
  for (int k = 0; k < 19; ++k) {
    if (FIRST)
      integ[k] = v[k];
    else
      integ[k] += sgn(v[k], sm);
  }
}

// General branch of calcSegSegForce; NEED12 / NEED34 as in pair_f64.cuh.
template <bool NEED12, bool NEED34, int FMATH>
FM_HD void general_pair(const KFast& K, X3 b1, X3 n11, X3 n12, X3 t1, double t1N, X3 b2, X3 n21, X3 n22, X3 t2,
                        double t2N, double c, X3& F1, X3& F2, X3& F3, X3& F4) {
  const double mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, mu8piaSq = K.mu8piaSq, mu4pinuaSq = K.mu4pinuaSq;
  const double cSq = c * c;
  const double omcSq = 1.0 - cSq;
  const double omcSqI = 1.0 / omcSq;

  const X3 t2ct1 = crossf(t2, t1);
  const X3 t1ct2 = -t2ct1;
  const X3 b2ct2 = crossf(b2, t2);
  const X3 b1ct1 = crossf(b1, t1);

  const double t2db2 = dotf(t2, b2);
  const double t2db1 = dotf(t2, b1);
  const double t1db2 = dotf(t1, b2);
  const double t1db1 = dotf(t1, b1);

  const double t2ct1db2 = dotf(t2ct1, b2);
  const double t1ct2db1 = dotf(t1ct2, b1);
  const double b1ct1db2 = dotf(b1ct1, b2);
  const double b2ct2db1 = dotf(b2ct2, b1);

  const X3 t2ct1ct2 = fmv(-c, t2, t1);
  const X3 t1ct2ct1 = fmv(-c, t1, t2);
  const X3 t2cb1ct2 = fmv(-t2db1, t2, b1);
  const X3 t1cb2ct1 = fmv(-t1db2, t1, b2);
  const X3 b1ct1ct2 = fmv(-c, b1, t2db1 * t1);
  const X3 b2ct2ct1 = fmv(-c, b2, t1db2 * t2);

  const double t2ct1cb1dt1 = fm::fma_(-t1db1, c, t2db1);
  const double t1ct2cb2dt2 = fm::fma_(-t2db2, c, t1db2);
  const double t2ct1cb1db2 = fm::fma_(t2db1, t1db2, -(t1db1 * t2db2));

  const X3 R1 = n21 - n11;
  const X3 R2 = n22 - n12;
  const double d = dot(R2, t2ct1) * omcSqI;

  const double mu4pid = mu4pi * d;
  const double mu4pinud = mu4pinu * d;
  const double mu4pinudSq = mu4pinud * d;
  const double mu4pinudCu = mu4pinudSq * d;
  const double mu4pinuaSqd = mu4pinuaSq * d;
  const double mu8piaSqd = mu8piaSq * d;

  const double lim11 = dot(R1, t1);
  const double lim12 = dot(R1, t2);
  const double lim21 = dot(R2, t1);
  const double lim22 = dot(R2, t2);

  const double x1 = (lim12 - c * lim11) * omcSqI;
  const double x2 = (lim22 - c * lim21) * omcSqI;
  const double y1 = (lim11 - c * lim12) * omcSqI;
  const double y2 = (lim21 - c * lim22) * omcSqI;

  double integ[19];
  const double aSq_dSq = K.aSq + d * d * omcSq;
  const double aSq_dSqI = 1.0 / aSq_dSq;
  const double den = 1.0 / sqrt(omcSq * aSq_dSq);
  const CornerK P{aSq_dSq, c, cSq, omcSqI, 2.0 * c, (1.0 + c) * den, -2.0 * den};
  // ((I(x1,y1) - I(x1,y2)) - I(x2,y1)) + I(x2,y2), DislocationForces.jl:948-951.
  corner<FMATH, true>(P, x1, y1, 0LL, integ);
#pragma unroll 1
  for (int q = 1; q < 4; ++q) {
    const double x = (q & 2) ? x2 : x1;
    const double y = (q & 1) ? y2 : y1;
    const long long sm = (q == 1 || q == 2) ? (long long)0x8000000000000000ULL : 0LL;
    corner<FMATH, false>(P, x, y, sm, integ);
  }
  integ[6] *= aSq_dSqI;
#pragma unroll
  for (int k = 7; k < 19; ++k) integ[k] *= omcSqI;

  // Force assembly.  The reference forms 11 vectors V[k] per side and sums
  // V[k] Fi[k] (DislocationForces.jl:953-1145); every V[k] is a combination of
  // five vectors (side 1: A = t2 x t1, B = b1 x t1, C = b2 - (t1.b2) t1,
  // D = (t1.b2) t2 - c b2, E = t2 - c t1; side 2: A, B = b2 x t2,
  // G = (t2.b1) t1 - c b1, H = t1 - c t2, K = b1 - (t2.b1) t2), so each node's
  // force is sum_m e_m (sum_k s_km Fi[k]): the scalar coefficients s_km first,
  // then five vector terms.
  double Fi[11];
  if (NEED12) {
    const X3& A = t2ct1;
    const X3& B = b1ct1;
    const X3& C = t1cb2ct1;
    const X3& D = b2ct2ct1;
    const X3& E = t1ct2ct1;
    const double p1 = fm::fma_(t1db2, t2db1, t2ct1cb1db2);  // V1 = p1 A
    const double p2 = t1ct2cb2dt2;                           // V2 = p2 B
    const double p3a = -b1ct1db2, p3c = -t2db1;              // V3 = p3a A + p3c C
    const double p4 = -t2ct1db2;                             // V4 = p4 B
    const double p5d = t2db1, p5a = b2ct2db1;                // V5 = p5d D + p5a A
    const double r3 = mu4pinudCu * t1ct2cb2dt2 * t1ct2db1;
    const double r4a = mu4pinudSq * t1ct2cb2dt2 * t2db1;
    const double r4b = mu4pinudSq * t1ct2cb2dt2 * t1ct2db1;
    const double r5 = mu4pinudSq * fm::fma_(t2ct1db2, t1ct2db1, t1ct2cb2dt2 * t1db1);
    const double r6a = mu4pinud * fm::fma_(t1ct2cb2dt2, t1db1, t2ct1db2 * t1ct2db1);
    const double r6b = mu4pinud * t2ct1db2 * t2db1;
    const double r7 = mu4pinud * t1ct2cb2dt2 * t2db1;
    const double r8 = mu4pinud * t2ct1db2 * t1db1;
    const double r9 = mu4pinu * t2ct1db2 * t2db1;
    const double r10 = mu4pinu * t2ct1db2 * t1db1;
    // s_km of V[0..10] on A, B, C, D, E.
    const double a0 = mu4pid * p1, a1 = fm::fma_(mu4pi, p5a, -mu4pinu * b2ct2db1), a2 = mu4pi * p3a,
                 a3 = mu8piaSqd * p1, a4 = fm::fma_(mu8piaSq, p5a, r4b), a5 = mu8piaSq * p3a;
    const double b0 = -mu4pinud * p2, b2 = -mu4pinu * p4, b3 = -mu4pinuaSqd * p2, b5 = -mu4pinuaSq * p4;
    const double c2 = mu4pi * p3c, c5 = mu8piaSq * p3c;
    const double d0 = mu4pinud * t1ct2db1, d1 = fm::fma_(mu4pi, p5d, -mu4pinu * t2db1), d2 = -mu4pinu * t1db1,
                 d4 = mu8piaSq * p5d;
    const double e0 = mu4pinud * b2ct2db1;
    auto node = [&](double tN) {
      double al = Fi[0] * a0;
      al = fm::fma_(Fi[1], a1, al);
      al = fm::fma_(Fi[2], a2, al);
      al = fm::fma_(Fi[3], a3, al);
      al = fm::fma_(Fi[4], a4, al);
      al = fm::fma_(Fi[5], a5, al);
      al = fm::fma_(Fi[6], -r6a, al);
      al = fm::fma_(Fi[7], -r7, al);
      al = fm::fma_(Fi[9], r9, al);
      al = fm::fma_(Fi[10], r10, al);
      double be = Fi[0] * b0;
      be = fm::fma_(Fi[2], b2, be);
      be = fm::fma_(Fi[3], b3, be);
      be = fm::fma_(Fi[5], b5, be);
      const double ga = fm::fma_(Fi[2], c2, Fi[5] * c5);
      double de = Fi[0] * d0;
      de = fm::fma_(Fi[1], d1, de);
      de = fm::fma_(Fi[2], d2, de);
      de = fm::fma_(Fi[4], d4, de);
      double ep = Fi[0] * e0;
      ep = fm::fma_(Fi[3], -r3, ep);
      ep = fm::fma_(Fi[4], r4a, ep);
      ep = fm::fma_(Fi[5], r5, ep);
      ep = fm::fma_(Fi[6], -r6b, ep);
      ep = fm::fma_(Fi[8], -r8, ep);
      X3 f = al * A;
      f = fmv(be, B, f);
      f = fmv(ga, C, f);
      f = fmv(de, D, f);
      f = fmv(ep, E, f);
      return f * tN;
    };

    const double y2_ = -y2;
    Fi[0] = fm::fma_(y2_, integ[0], integ[2]);
    Fi[1] = fm::fma_(y2_, integ[1], integ[3]);
    Fi[2] = fm::fma_(y2_, integ[2], integ[5]);
    Fi[3] = fm::fma_(y2_, integ[6], integ[8]);
    Fi[4] = fm::fma_(y2_, integ[7], integ[9]);
    Fi[5] = fm::fma_(y2_, integ[8], integ[11]);
    Fi[6] = fm::fma_(y2_, integ[9], integ[13]);
    Fi[7] = fm::fma_(y2_, integ[10], integ[12]);
    Fi[8] = fm::fma_(y2_, integ[11], integ[16]);
    Fi[9] = fm::fma_(y2_, integ[12], integ[14]);
    Fi[10] = fm::fma_(y2_, integ[13], integ[18]);
    F1 = node(t1N);

    Fi[0] = fm::fma_(y1, integ[0], -integ[2]);
    Fi[1] = fm::fma_(y1, integ[1], -integ[3]);
    Fi[2] = fm::fma_(y1, integ[2], -integ[5]);
    Fi[3] = fm::fma_(y1, integ[6], -integ[8]);
    Fi[4] = fm::fma_(y1, integ[7], -integ[9]);
    Fi[5] = fm::fma_(y1, integ[8], -integ[11]);
    Fi[6] = fm::fma_(y1, integ[9], -integ[13]);
    Fi[7] = fm::fma_(y1, integ[10], -integ[12]);
    Fi[8] = fm::fma_(y1, integ[11], -integ[16]);
    Fi[9] = fm::fma_(y1, integ[12], -integ[14]);
    Fi[10] = fm::fma_(y1, integ[13], -integ[18]);
    F2 = node(t1N);
  }
  if (NEED34) {
    const X3& A = t2ct1;
    const X3& B = b2ct2;
    const X3& G = b1ct1ct2;
    const X3& H = t2ct1ct2;
    const X3& Kv = t2cb1ct2;
    const double p1 = -fm::fma_(t2db1, t1db2, t2ct1cb1db2);  // V1 = p1 A
    const double p2 = t2ct1cb1dt1;                            // V2 = p2 B
    const double p3a = b1ct1db2, p3g = -t1db2;                // V3 = p3a A + p3g G
    const double p5k = t1db2, p5a = -b2ct2db1;                // V5 = p5k K + p5a A
    const double p6 = t1ct2db1;                               // V6 = p6 B
    const double r3 = mu4pinudCu * t2ct1cb1dt1 * t2ct1db2;
    const double r4 = mu4pinudSq * fm::fma_(t1ct2db1, t2ct1db2, t2ct1cb1dt1 * t2db2);
    const double r5a = mu4pinudSq * t2ct1cb1dt1 * t1db2;
    const double r5b = mu4pinudSq * t2ct1cb1dt1 * t2ct1db2;
    const double r6a = mu4pinud * fm::fma_(t2ct1cb1dt1, t2db2, t1ct2db1 * t2ct1db2);
    const double r6b = mu4pinud * t1ct2db1 * t1db2;
    const double r7 = mu4pinud * t1ct2db1 * t2db2;
    const double r8 = mu4pinud * t2ct1cb1dt1 * t1db2;
    const double r9 = mu4pinu * t1ct2db1 * t2db2;
    const double r10 = mu4pinu * t1ct2db1 * t1db2;
    // s_km of V[0..10] on A, B, G, H, K.
    const double a0 = mu4pid * p1, a1 = mu4pi * p5a, a2 = fm::fma_(mu4pi, p3a, -mu4pinu * b1ct1db2),
                 a3 = mu8piaSqd * p1, a4 = mu8piaSq * p5a, a5 = fm::fma_(mu8piaSq, p3a, r5b);
    const double b0 = -mu4pinud * p2, b1 = -mu4pinu * p6, b3 = -mu4pinuaSqd * p2, b4 = -mu4pinuaSq * p6;
    const double g0 = mu4pinud * t2ct1db2, g1 = mu4pinu * t2db2, g2 = fm::fma_(mu4pi, p3g, mu4pinu * t1db2),
                 g5 = mu8piaSq * p3g;
    const double h0 = mu4pinud * b1ct1db2;
    const double k1 = mu4pi * p5k, k4 = mu8piaSq * p5k;
    auto node = [&](double tN) {
      double al = Fi[0] * a0;
      al = fm::fma_(Fi[1], a1, al);
      al = fm::fma_(Fi[2], a2, al);
      al = fm::fma_(Fi[3], a3, al);
      al = fm::fma_(Fi[4], a4, al);
      al = fm::fma_(Fi[5], a5, al);
      al = fm::fma_(Fi[6], r6a, al);
      al = fm::fma_(Fi[8], r8, al);
      al = fm::fma_(Fi[9], r9, al);
      al = fm::fma_(Fi[10], r10, al);
      double be = Fi[0] * b0;
      be = fm::fma_(Fi[1], b1, be);
      be = fm::fma_(Fi[3], b3, be);
      be = fm::fma_(Fi[4], b4, be);
      double ge = Fi[0] * g0;
      ge = fm::fma_(Fi[1], g1, ge);
      ge = fm::fma_(Fi[2], g2, ge);
      ge = fm::fma_(Fi[5], g5, ge);
      double he = Fi[0] * h0;
      he = fm::fma_(Fi[3], -r3, he);
      he = fm::fma_(Fi[4], -r4, he);
      he = fm::fma_(Fi[5], -r5a, he);
      he = fm::fma_(Fi[6], -r6b, he);
      he = fm::fma_(Fi[7], -r7, he);
      const double ka = fm::fma_(Fi[1], k1, Fi[4] * k4);
      X3 f = al * A;
      f = fmv(be, B, f);
      f = fmv(ge, G, f);
      f = fmv(he, H, f);
      f = fmv(ka, Kv, f);
      return f * tN;
    };

    Fi[0] = fm::fma_(x2, integ[0], -integ[1]);
    Fi[1] = fm::fma_(x2, integ[1], -integ[4]);
    Fi[2] = fm::fma_(x2, integ[2], -integ[3]);
    Fi[3] = fm::fma_(x2, integ[6], -integ[7]);
    Fi[4] = fm::fma_(x2, integ[7], -integ[10]);
    Fi[5] = fm::fma_(x2, integ[8], -integ[9]);
    Fi[6] = fm::fma_(x2, integ[9], -integ[12]);
    Fi[7] = fm::fma_(x2, integ[10], -integ[15]);
    Fi[8] = fm::fma_(x2, integ[11], -integ[13]);
    Fi[9] = fm::fma_(x2, integ[12], -integ[17]);
    Fi[10] = fm::fma_(x2, integ[13], -integ[14]);
    F3 = node(t2N);

    const double x1_ = -x1;
    Fi[0] = fm::fma_(x1_, integ[0], integ[1]);
    Fi[1] = fm::fma_(x1_, integ[1], integ[4]);
    Fi[2] = fm::fma_(x1_, integ[2], integ[3]);
    Fi[3] = fm::fma_(x1_, integ[6], integ[7]);
    Fi[4] = fm::fma_(x1_, integ[7], integ[10]);
    Fi[5] = fm::fma_(x1_, integ[8], integ[9]);
    Fi[6] = fm::fma_(x1_, integ[9], integ[12]);
    Fi[7] = fm::fma_(x1_, integ[10], integ[15]);
    Fi[8] = fm::fma_(x1_, integ[11], integ[13]);
    Fi[9] = fm::fma_(x1_, integ[12], integ[17]);
    Fi[10] = fm::fma_(x1_, integ[13], integ[14]);
    F4 = node(t2N);
  }
}

}  // namespace fx
}  // namespace ddd
