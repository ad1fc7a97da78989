// General branch of the non-singular segment-segment force in df64 arithmetic
// (double-float on the FP32 pipes).  Same formulas and evaluation order as the
// FP64 kernel (pair_f64.cuh), i.e. as DislocationForces.jl:879-1165 and
// SegSegInteg :1480-1561, with every scalar a df64.
#pragma once
#include "df64.cuh"

namespace ddd {

struct DV3 {
  df64 x, y, z;
};
DF_HD DV3 operator+(DV3 a, DV3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
DF_HD DV3 operator-(DV3 a, DV3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
DF_HD DV3 operator-(DV3 a) { return {-a.x, -a.y, -a.z}; }
DF_HD DV3 operator*(df64 s, DV3 a) { return {s * a.x, s * a.y, s * a.z}; }
DF_HD DV3 operator*(DV3 a, df64 s) { return {a.x * s, a.y * s, a.z * s}; }
DF_HD df64 dot(DV3 a, DV3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DF_HD DV3 cross(DV3 a, DV3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

struct KConstsDF {
  df64 aSq, mu4pi, mu4pinu, mu8piaSq, mu4pinuaSq;
};

// SegSegInteg at one corner in df64, added or subtracted (neg) into integ[19].
// aSq_dSq = aSq + d^2 (1 - c^2), its inverse, and den = 1 / sqrt((1 - c^2) aSq_dSq)
// are computed once per pair by the caller.
DF_HD void seg_seg_integ_df(df64 aSq_dSq, df64 aSq_dSqI, df64 den, df64 c, df64 cSq, df64 omcSqI, df64 x, df64 y,
                            bool neg, df64* integ) {
  df64 xSq = x * x;
  df64 ySq = y * y;
  df64 Ra = df_sqrt(aSq_dSq + xSq + ySq + df_scale(x, 2.0f) * y * c);
  df64 RaInv = df_recip(Ra);

  df64 Ra_Rd_t1 = Ra + y + x * c;
  df64 Ra_Rd_t2 = Ra + x + y * c;

  df64 log_Ra_Rd_t1 = df_log(Ra_Rd_t1);
  df64 xlog_Ra_Rd_t1 = x * log_Ra_Rd_t1;
  df64 log_Ra_Rd_t2 = df_log(Ra_Rd_t2);
  df64 ylog_Ra_Rd_t2 = y * log_Ra_Rd_t2;

  df64 RaSq_R_t1_I = RaInv / Ra_Rd_t1;
  df64 xRaSq_R_t1_I = x * RaSq_R_t1_I;
  df64 xSqRaSq_R_t1_I = x * xRaSq_R_t1_I;

  df64 RaSq_R_t2_I = RaInv / Ra_Rd_t2;
  df64 yRaSq_R_t2_I = y * RaSq_R_t2_I;
  df64 ySqRaSq_R_t2_I = y * yRaSq_R_t2_I;

  df64 integ1 = df_scale(-den, 2.0f) * df_atan((df(1.0f) + c) * (Ra + x + y) * den);

  df64 c_1 = aSq_dSq * integ1;
  df64 c_5_6 = (c * Ra - c_1) * omcSqI;

  df64 integ2 = (c * log_Ra_Rd_t2 - log_Ra_Rd_t1) * omcSqI;
  df64 integ3 = (c * log_Ra_Rd_t1 - log_Ra_Rd_t2) * omcSqI;
  df64 integ4 = (c * c_1 - Ra) * omcSqI;
  df64 integ5 = ylog_Ra_Rd_t2 + c_5_6;
  df64 integ6 = xlog_Ra_Rd_t1 + c_5_6;

  df64 c_11_12 = integ1 - c * RaInv;
  df64 c_15_18 = c * xRaSq_R_t1_I - RaInv;
  df64 x_13_14 = x * c_15_18;
  df64 c_19 = c * yRaSq_R_t2_I - RaInv;
  df64 y_13_14 = y * c_19;
  df64 c_16 = log_Ra_Rd_t2 - (x - c * y) * RaInv - cSq * ySqRaSq_R_t2_I;
  df64 z_15_18 = y * c_16;
  df64 c_17_19 = log_Ra_Rd_t1 - (y - c * x) * RaInv - cSq * xSqRaSq_R_t1_I;

  df64 c15_18_19 = df_scale(integ4, 2.0f);

  df64 v[19];
  v[0] = integ1;
  v[1] = integ2;
  v[2] = integ3;
  v[3] = integ4;
  v[4] = integ5;
  v[5] = integ6;
  v[6] = (integ1 - xRaSq_R_t1_I - yRaSq_R_t2_I) * aSq_dSqI;
  v[7] = (RaSq_R_t1_I - c * RaSq_R_t2_I) * omcSqI;
  v[8] = (RaSq_R_t2_I - c * RaSq_R_t1_I) * omcSqI;
  v[9] = (RaInv - c * (xRaSq_R_t1_I + yRaSq_R_t2_I + integ1)) * omcSqI;
  v[10] = (xRaSq_R_t1_I + cSq * yRaSq_R_t2_I + c_11_12) * omcSqI;
  v[11] = (yRaSq_R_t2_I + cSq * xRaSq_R_t1_I + c_11_12) * omcSqI;
  v[12] = (integ3 - x_13_14 + c * (y_13_14 - integ2)) * omcSqI;
  v[13] = (integ2 - y_13_14 + c * (x_13_14 - integ3)) * omcSqI;
  v[14] = (integ5 - z_15_18 + c * (xSq * c_15_18 - c15_18_19)) * omcSqI;
  v[15] = (xSqRaSq_R_t1_I + c * c_16 + df_scale(integ2, 2.0f)) * omcSqI;
  v[16] = (ySqRaSq_R_t2_I + c * c_17_19 + df_scale(integ3, 2.0f)) * omcSqI;
  v[17] = (c15_18_19 - xSq * c_15_18 + c * (z_15_18 - integ5)) * omcSqI;
  v[18] = (c15_18_19 - ySq * c_19 + c * (x * c_17_19 - integ6)) * omcSqI;
#pragma unroll
  for (int k = 0; k < 19; ++k) integ[k] = integ[k] + (neg ? -v[k] : v[k]);
}

DF_HD DV3 fsum11_df(const DV3* V, const df64* F) {
  DV3 s = V[0] * F[0] + V[1] * F[1];
#pragma unroll
  for (int k = 2; k < 11; ++k) s = s + V[k] * F[k];
  return s;
}

// General branch of calcSegSegForce in df64 (forces on seg 1 if NEED12, seg 2 if NEED34).
template <bool NEED12, bool NEED34>
DF_HD void general_pair_df(const KConstsDF& K, DV3 b1, DV3 n11, DV3 n12, DV3 t1, df64 t1N, DV3 b2, DV3 n21, DV3 n22,
                           DV3 t2, df64 t2N, df64 c, DV3& F1, DV3& F2, DV3& F3, DV3& F4) {
  const df64 mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, mu8piaSq = K.mu8piaSq, mu4pinuaSq = K.mu4pinuaSq;
  df64 cSq = c * c;
  df64 omcSq = df(1.0f) - cSq;
  df64 omcSqI = df_recip(omcSq);

  DV3 t2ct1 = cross(t2, t1);
  DV3 t1ct2 = -t2ct1;
  DV3 b2ct2 = cross(b2, t2);
  DV3 b1ct1 = cross(b1, t1);

  df64 t2db2 = dot(t2, b2);
  df64 t2db1 = dot(t2, b1);
  df64 t1db2 = dot(t1, b2);
  df64 t1db1 = dot(t1, b1);

  df64 t2ct1db2 = dot(t2ct1, b2);
  df64 t1ct2db1 = dot(t1ct2, b1);
  df64 b1ct1db2 = dot(b1ct1, b2);
  df64 b2ct2db1 = dot(b2ct2, b1);

  DV3 t2ct1ct2 = t1 - c * t2;
  DV3 t1ct2ct1 = t2 - c * t1;
  DV3 t2cb1ct2 = b1 - t2db1 * t2;
  DV3 t1cb2ct1 = b2 - t1db2 * t1;
  DV3 b1ct1ct2 = t2db1 * t1 - c * b1;
  DV3 b2ct2ct1 = t1db2 * t2 - c * b2;

  df64 t2ct1cb1dt1 = t2db1 - t1db1 * c;
  df64 t1ct2cb2dt2 = t1db2 - t2db2 * c;
  df64 t2ct1cb1db2 = t2db1 * t1db2 - t1db1 * t2db2;

  DV3 R1 = n21 - n11;
  DV3 R2 = n22 - n12;
  df64 d = dot(R2, t2ct1) * omcSqI;

  df64 mu4pid = mu4pi * d;
  df64 mu4pinud = mu4pinu * d;
  df64 mu4pinudSq = mu4pinud * d;
  df64 mu4pinudCu = mu4pinudSq * d;
  df64 mu4pinuaSqd = mu4pinuaSq * d;
  df64 mu8piaSqd = mu8piaSq * d;

  df64 lim11 = dot(R1, t1);
  df64 lim12 = dot(R1, t2);
  df64 lim21 = dot(R2, t1);
  df64 lim22 = dot(R2, t2);

  df64 x1 = (lim12 - c * lim11) * omcSqI;
  df64 x2 = (lim22 - c * lim21) * omcSqI;
  df64 y1 = (lim11 - c * lim12) * omcSqI;
  df64 y2 = (lim21 - c * lim22) * omcSqI;

  df64 integ[19];
#pragma unroll
  for (int k = 0; k < 19; ++k) integ[k] = df(0.0f);
  const df64 aSq_dSq = K.aSq + d * d * omcSq;
  const df64 aSq_dSqI = df_recip(aSq_dSq);
  const df64 den = df_recip(df_sqrt(omcSq * aSq_dSq));
#ifdef __CUDACC__
#pragma unroll 1
#endif
  for (int q = 0; q < 4; ++q) {
    df64 x = (q & 2) ? x2 : x1;
    df64 y = (q & 1) ? y2 : y1;
    seg_seg_integ_df(aSq_dSq, aSq_dSqI, den, c, cSq, omcSqI, x, y, q == 1 || q == 2, integ);
  }

  DV3 V[11];
  df64 Fi[11];
  df64 tmp1, tmp2;
  if (NEED12) {
    tmp1 = t1db2 * t2db1 + t2ct1cb1db2;
    DV3 V1 = tmp1 * t2ct1;
    DV3 V2 = b1ct1 * t1ct2cb2dt2;
    DV3 V3 = t1ct2 * b1ct1db2 - t1cb2ct1 * t2db1;
    DV3 V4 = -b1ct1 * t2ct1db2;
    DV3 V5 = b2ct2ct1 * t2db1 - t1ct2 * b2ct2db1;

    tmp1 = mu4pinud * t1ct2db1;
    tmp2 = mu4pinud * b2ct2db1;
    V[0] = mu4pid * V1 - mu4pinud * V2 + tmp1 * b2ct2ct1 + tmp2 * t1ct2ct1;
    tmp1 = mu4pinu * t2db1;
    tmp2 = mu4pinu * b2ct2db1;
    V[1] = mu4pi * V5 - tmp1 * b2ct2ct1 + tmp2 * t1ct2;
    tmp1 = mu4pinu * t1db1;
    V[2] = -tmp1 * b2ct2ct1 + mu4pi * V3 - mu4pinu * V4;
    tmp1 = mu4pinudCu * t1ct2cb2dt2 * t1ct2db1;
    V[3] = mu8piaSqd * V1 - mu4pinuaSqd * V2 - tmp1 * t1ct2ct1;
    tmp1 = mu4pinudSq * t1ct2cb2dt2 * t2db1;
    tmp2 = mu4pinudSq * t1ct2cb2dt2 * t1ct2db1;
    V[4] = mu8piaSq * V5 + tmp1 * t1ct2ct1 - tmp2 * t1ct2;
    tmp1 = mu4pinudSq * (t2ct1db2 * t1ct2db1 + t1ct2cb2dt2 * t1db1);
    V[5] = mu8piaSq * V3 - mu4pinuaSq * V4 + tmp1 * t1ct2ct1;
    tmp1 = mu4pinud * (t1ct2cb2dt2 * t1db1 + t2ct1db2 * t1ct2db1);
    tmp2 = mu4pinud * t2ct1db2 * t2db1;
    V[6] = tmp1 * t1ct2 - tmp2 * t1ct2ct1;
    tmp1 = mu4pinud * t1ct2cb2dt2 * t2db1;
    V[7] = tmp1 * t1ct2;
    tmp1 = mu4pinud * t2ct1db2 * t1db1;
    V[8] = -tmp1 * t1ct2ct1;
    DV3 tv = mu4pinu * t2ct1db2 * t1ct2;
    V[9] = -tv * t2db1;
    V[10] = -tv * t1db1;

    Fi[0] = integ[2] - y2 * integ[0];
    Fi[1] = integ[3] - y2 * integ[1];
    Fi[2] = integ[5] - y2 * integ[2];
    Fi[3] = integ[8] - y2 * integ[6];
    Fi[4] = integ[9] - y2 * integ[7];
    Fi[5] = integ[11] - y2 * integ[8];
    Fi[6] = integ[13] - y2 * integ[9];
    Fi[7] = integ[12] - y2 * integ[10];
    Fi[8] = integ[16] - y2 * integ[11];
    Fi[9] = integ[14] - y2 * integ[12];
    Fi[10] = integ[18] - y2 * integ[13];
    F1 = fsum11_df(V, Fi) * t1N;

    Fi[0] = y1 * integ[0] - integ[2];
    Fi[1] = y1 * integ[1] - integ[3];
    Fi[2] = y1 * integ[2] - integ[5];
    Fi[3] = y1 * integ[6] - integ[8];
    Fi[4] = y1 * integ[7] - integ[9];
    Fi[5] = y1 * integ[8] - integ[11];
    Fi[6] = y1 * integ[9] - integ[13];
    Fi[7] = y1 * integ[10] - integ[12];
    Fi[8] = y1 * integ[11] - integ[16];
    Fi[9] = y1 * integ[12] - integ[14];
    Fi[10] = y1 * integ[13] - integ[18];
    F2 = fsum11_df(V, Fi) * t1N;
  }
  if (NEED34) {
    tmp1 = t2db1 * t1db2 + t2ct1cb1db2;
    DV3 V1 = tmp1 * t1ct2;
    DV3 V2 = b2ct2 * t2ct1cb1dt1;
    DV3 V3 = t2ct1 * b1ct1db2 - b1ct1ct2 * t1db2;
    DV3 V5 = t2cb1ct2 * t1db2 - t2ct1 * b2ct2db1;
    DV3 V6 = b2ct2 * t1ct2db1;

    tmp1 = mu4pinud * t2ct1db2;
    tmp2 = mu4pinud * b1ct1db2;
    V[0] = mu4pid * V1 - mu4pinud * V2 + tmp1 * b1ct1ct2 + tmp2 * t2ct1ct2;
    tmp1 = mu4pinu * t2db2;
    V[1] = tmp1 * b1ct1ct2 + mu4pi * V5 - mu4pinu * V6;
    tmp1 = mu4pinu * t1db2;
    tmp2 = mu4pinu * b1ct1db2;
    V[2] = mu4pi * V3 + tmp1 * b1ct1ct2 - tmp2 * t2ct1;
    tmp1 = mu4pinudCu * t2ct1cb1dt1 * t2ct1db2;
    V[3] = mu8piaSqd * V1 - mu4pinuaSqd * V2 - tmp1 * t2ct1ct2;
    tmp1 = mu4pinudSq * (t1ct2db1 * t2ct1db2 + t2ct1cb1dt1 * t2db2);
    V[4] = mu8piaSq * V5 - mu4pinuaSq * V6 - tmp1 * t2ct1ct2;
    tmp1 = mu4pinudSq * t2ct1cb1dt1 * t1db2;
    tmp2 = mu4pinudSq * t2ct1cb1dt1 * t2ct1db2;
    V[5] = mu8piaSq * V3 - tmp1 * t2ct1ct2 + tmp2 * t2ct1;
    tmp1 = mu4pinud * (t2ct1cb1dt1 * t2db2 + t1ct2db1 * t2ct1db2);
    tmp2 = mu4pinud * t1ct2db1 * t1db2;
    V[6] = tmp1 * t2ct1 - tmp2 * t2ct1ct2;
    tmp1 = mu4pinud * t1ct2db1 * t2db2;
    V[7] = -tmp1 * t2ct1ct2;
    tmp1 = mu4pinud * t2ct1cb1dt1 * t1db2;
    V[8] = tmp1 * t2ct1;
    DV3 tv = mu4pinu * t1ct2db1 * t2ct1;
    V[9] = tv * t2db2;
    V[10] = tv * t1db2;

    Fi[0] = x2 * integ[0] - integ[1];
    Fi[1] = x2 * integ[1] - integ[4];
    Fi[2] = x2 * integ[2] - integ[3];
    Fi[3] = x2 * integ[6] - integ[7];
    Fi[4] = x2 * integ[7] - integ[10];
    Fi[5] = x2 * integ[8] - integ[9];
    Fi[6] = x2 * integ[9] - integ[12];
    Fi[7] = x2 * integ[10] - integ[15];
    Fi[8] = x2 * integ[11] - integ[13];
    Fi[9] = x2 * integ[12] - integ[17];
    Fi[10] = x2 * integ[13] - integ[14];
    F3 = fsum11_df(V, Fi) * t2N;

    Fi[0] = integ[1] - x1 * integ[0];
    Fi[1] = integ[4] - x1 * integ[1];
    Fi[2] = integ[3] - x1 * integ[2];
    Fi[3] = integ[7] - x1 * integ[6];
    Fi[4] = integ[10] - x1 * integ[7];
    Fi[5] = integ[9] - x1 * integ[8];
    Fi[6] = integ[12] - x1 * integ[9];
    Fi[7] = integ[15] - x1 * integ[10];
    Fi[8] = integ[13] - x1 * integ[11];
    Fi[9] = integ[17] - x1 * integ[12];
    Fi[10] = integ[14] - x1 * integ[13];
    F4 = fsum11_df(V, Fi) * t2N;
  }
}

}  // namespace ddd

namespace ddd {

struct F3 {
  float x, y, z;
};
DF_HD F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
DF_HD F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
DF_HD F3 operator-(F3 a) { return {-a.x, -a.y, -a.z}; }
DF_HD F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
DF_HD F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
DF_HD float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DF_HD F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
DF_HD F3 f3(DV3 v) { return {v.x.hi, v.y.hi, v.z.hi}; }

struct KConstsF {
  float mu4pi, mu4pinu, mu8piaSq, mu4pinuaSq;
};

// Mixed form of the general branch: the integration-domain geometry (c, d,
// x1..y2), the four corner antiderivatives and their first moments (Fint) in
// df64 — the cancellation-prone part, whose terms cancel by up to (R/L)^3 for
// a pair at distance R — and the V-vector assembly (products of unit vectors,
// Burgers vectors and powers of d, no cancellation of that order) in FP32.
// The 11-term node sums are taken in df64 from FP32 V and df64 Fint.
template <bool NEED12, bool NEED34, bool SUM32 = false>
DF_HD void general_pair_mixed(const KConstsDF& K, const KConstsF& KF, F3 b1, DV3 n11, DV3 n12, DV3 t1, float t1N,
                              F3 b2, DV3 n21, DV3 n22, DV3 t2, float t2N, df64 c, DV3& F1, DV3& F2, DV3& F3_,
                              DV3& F4) {
  df64 cSq = c * c;
  df64 omcSq = df(1.0f) - cSq;
  df64 omcSqI = df_recip(omcSq);

  DV3 t2ct1d = cross(t2, t1);
  DV3 R1 = n21 - n11;
  DV3 R2 = n22 - n12;
  df64 d = dot(R2, t2ct1d) * omcSqI;
  df64 lim11 = dot(R1, t1);
  df64 lim12 = dot(R1, t2);
  df64 lim21 = dot(R2, t1);
  df64 lim22 = dot(R2, t2);
  df64 x1 = (lim12 - c * lim11) * omcSqI;
  df64 x2 = (lim22 - c * lim21) * omcSqI;
  df64 y1 = (lim11 - c * lim12) * omcSqI;
  df64 y2 = (lim21 - c * lim22) * omcSqI;

  df64 integ[19];
#pragma unroll
  for (int k = 0; k < 19; ++k) integ[k] = df(0.0f);
  const df64 aSq_dSq = K.aSq + d * d * omcSq;
  const df64 aSq_dSqI = df_recip(aSq_dSq);
  const df64 den = df_recip(df_sqrt(omcSq * aSq_dSq));
#ifdef __CUDACC__
#pragma unroll 1
#endif
  for (int q = 0; q < 4; ++q) {
    df64 x = (q & 2) ? x2 : x1;
    df64 y = (q & 1) ? y2 : y1;
    seg_seg_integ_df(aSq_dSq, aSq_dSqI, den, c, cSq, omcSqI, x, y, q == 1 || q == 2, integ);
  }

  // FP32 geometry of the V vectors.
  const float mu4pi = KF.mu4pi, mu4pinu = KF.mu4pinu, mu8piaSq = KF.mu8piaSq, mu4pinuaSq = KF.mu4pinuaSq;
  const F3 ft1 = f3(t1), ft2 = f3(t2);
  const float cf = c.hi;
  const float dfl = d.hi;
  F3 t2ct1 = cross(ft2, ft1);
  F3 t1ct2 = -t2ct1;
  F3 b2ct2 = cross(b2, ft2);
  F3 b1ct1 = cross(b1, ft1);
  float t2db2 = dot(ft2, b2), t2db1 = dot(ft2, b1), t1db2 = dot(ft1, b2), t1db1 = dot(ft1, b1);
  float t2ct1db2 = dot(t2ct1, b2), t1ct2db1 = dot(t1ct2, b1), b1ct1db2 = dot(b1ct1, b2), b2ct2db1 = dot(b2ct2, b1);
  F3 t2ct1ct2 = ft1 - cf * ft2;
  F3 t1ct2ct1 = ft2 - cf * ft1;
  F3 t2cb1ct2 = b1 - t2db1 * ft2;
  F3 t1cb2ct1 = b2 - t1db2 * ft1;
  F3 b1ct1ct2 = t2db1 * ft1 - cf * b1;
  F3 b2ct2ct1 = t1db2 * ft2 - cf * b2;
  float t2ct1cb1dt1 = t2db1 - t1db1 * cf;
  float t1ct2cb2dt2 = t1db2 - t2db2 * cf;
  float t2ct1cb1db2 = t2db1 * t1db2 - t1db1 * t2db2;
  float mu4pid = mu4pi * dfl;
  float mu4pinud = mu4pinu * dfl;
  float mu4pinudSq = mu4pinud * dfl;
  float mu4pinudCu = mu4pinudSq * dfl;
  float mu4pinuaSqd = mu4pinuaSq * dfl;
  float mu8piaSqd = mu8piaSq * dfl;

  F3 V[11];
  df64 Fi[11];
  float tmp1, tmp2;
  auto nodesum = [&](float tN) {
    if (SUM32) {
      F3 s = {0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 11; ++k) s = s + V[k] * (Fi[k].hi + Fi[k].lo);
      return DV3{df(s.x * tN), df(s.y * tN), df(s.z * tN)};
    }
    DV3 s = {df(0.f), df(0.f), df(0.f)};
#pragma unroll
    for (int k = 0; k < 11; ++k) {
      s.x = s.x + Fi[k] * V[k].x;
      s.y = s.y + Fi[k] * V[k].y;
      s.z = s.z + Fi[k] * V[k].z;
    }
    return DV3{s.x * tN, s.y * tN, s.z * tN};
  };
  if (NEED12) {
    tmp1 = t1db2 * t2db1 + t2ct1cb1db2;
    F3 V1 = tmp1 * t2ct1;
    F3 V2 = b1ct1 * t1ct2cb2dt2;
    F3 V3 = t1ct2 * b1ct1db2 - t1cb2ct1 * t2db1;
    F3 V4 = -b1ct1 * t2ct1db2;
    F3 V5 = b2ct2ct1 * t2db1 - t1ct2 * b2ct2db1;
    tmp1 = mu4pinud * t1ct2db1;
    tmp2 = mu4pinud * b2ct2db1;
    V[0] = mu4pid * V1 - mu4pinud * V2 + tmp1 * b2ct2ct1 + tmp2 * t1ct2ct1;
    tmp1 = mu4pinu * t2db1;
    tmp2 = mu4pinu * b2ct2db1;
    V[1] = mu4pi * V5 - tmp1 * b2ct2ct1 + tmp2 * t1ct2;
    tmp1 = mu4pinu * t1db1;
    V[2] = -tmp1 * b2ct2ct1 + mu4pi * V3 - mu4pinu * V4;
    tmp1 = mu4pinudCu * t1ct2cb2dt2 * t1ct2db1;
    V[3] = mu8piaSqd * V1 - mu4pinuaSqd * V2 - tmp1 * t1ct2ct1;
    tmp1 = mu4pinudSq * t1ct2cb2dt2 * t2db1;
    tmp2 = mu4pinudSq * t1ct2cb2dt2 * t1ct2db1;
    V[4] = mu8piaSq * V5 + tmp1 * t1ct2ct1 - tmp2 * t1ct2;
    tmp1 = mu4pinudSq * (t2ct1db2 * t1ct2db1 + t1ct2cb2dt2 * t1db1);
    V[5] = mu8piaSq * V3 - mu4pinuaSq * V4 + tmp1 * t1ct2ct1;
    tmp1 = mu4pinud * (t1ct2cb2dt2 * t1db1 + t2ct1db2 * t1ct2db1);
    tmp2 = mu4pinud * t2ct1db2 * t2db1;
    V[6] = tmp1 * t1ct2 - tmp2 * t1ct2ct1;
    tmp1 = mu4pinud * t1ct2cb2dt2 * t2db1;
    V[7] = tmp1 * t1ct2;
    tmp1 = mu4pinud * t2ct1db2 * t1db1;
    V[8] = -tmp1 * t1ct2ct1;
    F3 tv = mu4pinu * t2ct1db2 * t1ct2;
    V[9] = -tv * t2db1;
    V[10] = -tv * t1db1;

    Fi[0] = integ[2] - y2 * integ[0];
    Fi[1] = integ[3] - y2 * integ[1];
    Fi[2] = integ[5] - y2 * integ[2];
    Fi[3] = integ[8] - y2 * integ[6];
    Fi[4] = integ[9] - y2 * integ[7];
    Fi[5] = integ[11] - y2 * integ[8];
    Fi[6] = integ[13] - y2 * integ[9];
    Fi[7] = integ[12] - y2 * integ[10];
    Fi[8] = integ[16] - y2 * integ[11];
    Fi[9] = integ[14] - y2 * integ[12];
    Fi[10] = integ[18] - y2 * integ[13];
    F1 = nodesum(t1N);
    Fi[0] = y1 * integ[0] - integ[2];
    Fi[1] = y1 * integ[1] - integ[3];
    Fi[2] = y1 * integ[2] - integ[5];
    Fi[3] = y1 * integ[6] - integ[8];
    Fi[4] = y1 * integ[7] - integ[9];
    Fi[5] = y1 * integ[8] - integ[11];
    Fi[6] = y1 * integ[9] - integ[13];
    Fi[7] = y1 * integ[10] - integ[12];
    Fi[8] = y1 * integ[11] - integ[16];
    Fi[9] = y1 * integ[12] - integ[14];
    Fi[10] = y1 * integ[13] - integ[18];
    F2 = nodesum(t1N);
  }
  if (NEED34) {
    tmp1 = t2db1 * t1db2 + t2ct1cb1db2;
    F3 V1 = tmp1 * t1ct2;
    F3 V2 = b2ct2 * t2ct1cb1dt1;
    F3 V3 = t2ct1 * b1ct1db2 - b1ct1ct2 * t1db2;
    F3 V5 = t2cb1ct2 * t1db2 - t2ct1 * b2ct2db1;
    F3 V6 = b2ct2 * t1ct2db1;
    tmp1 = mu4pinud * t2ct1db2;
    tmp2 = mu4pinud * b1ct1db2;
    V[0] = mu4pid * V1 - mu4pinud * V2 + tmp1 * b1ct1ct2 + tmp2 * t2ct1ct2;
    tmp1 = mu4pinu * t2db2;
    V[1] = tmp1 * b1ct1ct2 + mu4pi * V5 - mu4pinu * V6;
    tmp1 = mu4pinu * t1db2;
    tmp2 = mu4pinu * b1ct1db2;
    V[2] = mu4pi * V3 + tmp1 * b1ct1ct2 - tmp2 * t2ct1;
    tmp1 = mu4pinudCu * t2ct1cb1dt1 * t2ct1db2;
    V[3] = mu8piaSqd * V1 - mu4pinuaSqd * V2 - tmp1 * t2ct1ct2;
    tmp1 = mu4pinudSq * (t1ct2db1 * t2ct1db2 + t2ct1cb1dt1 * t2db2);
    V[4] = mu8piaSq * V5 - mu4pinuaSq * V6 - tmp1 * t2ct1ct2;
    tmp1 = mu4pinudSq * t2ct1cb1dt1 * t1db2;
    tmp2 = mu4pinudSq * t2ct1cb1dt1 * t2ct1db2;
    V[5] = mu8piaSq * V3 - tmp1 * t2ct1ct2 + tmp2 * t2ct1;
    tmp1 = mu4pinud * (t2ct1cb1dt1 * t2db2 + t1ct2db1 * t2ct1db2);
    tmp2 = mu4pinud * t1ct2db1 * t1db2;
    V[6] = tmp1 * t2ct1 - tmp2 * t2ct1ct2;
    tmp1 = mu4pinud * t1ct2db1 * t2db2;
    V[7] = -tmp1 * t2ct1ct2;
    tmp1 = mu4pinud * t2ct1cb1dt1 * t1db2;
    V[8] = tmp1 * t2ct1;
    F3 tv = mu4pinu * t1ct2db1 * t2ct1;
    V[9] = tv * t2db2;
    V[10] = tv * t1db2;

    Fi[0] = x2 * integ[0] - integ[1];
    Fi[1] = x2 * integ[1] - integ[4];
    Fi[2] = x2 * integ[2] - integ[3];
    Fi[3] = x2 * integ[6] - integ[7];
    Fi[4] = x2 * integ[7] - integ[10];
    Fi[5] = x2 * integ[8] - integ[9];
    Fi[6] = x2 * integ[9] - integ[12];
    Fi[7] = x2 * integ[10] - integ[15];
    Fi[8] = x2 * integ[11] - integ[13];
    Fi[9] = x2 * integ[12] - integ[17];
    Fi[10] = x2 * integ[13] - integ[14];
    F3_ = nodesum(t2N);
    Fi[0] = integ[1] - x1 * integ[0];
    Fi[1] = integ[4] - x1 * integ[1];
    Fi[2] = integ[3] - x1 * integ[2];
    Fi[3] = integ[7] - x1 * integ[6];
    Fi[4] = integ[10] - x1 * integ[7];
    Fi[5] = integ[9] - x1 * integ[8];
    Fi[6] = integ[12] - x1 * integ[9];
    Fi[7] = integ[15] - x1 * integ[10];
    Fi[8] = integ[13] - x1 * integ[11];
    Fi[9] = integ[17] - x1 * integ[12];
    Fi[10] = integ[14] - x1 * integ[13];
    F4 = nodesum(t2N);
  }
}

// Constants of the mixed σ̃ form.
struct KConstsSig {
  df64 aSq;
  float mu4pi, mu4pinu, nuMu4pinu, aSq32, aSqMu8pi;
};

// σ̃ contribution of one segment (n1, n2, unit direction t, Burgers vector b)
// at the point x, added into six df64 accumulators (xx, yy, zz, xy, xz, yz):
// the reference's formulas (DislocationFEM.jl:135-299, sigma_point in
// pair_f64.cuh), with the geometry (R, d, s1, s2), the endpoint terms and their
// differences s_03 ... s_25 in df64 — where the two endpoints cancel — and the
// coefficient assembly (t, d, t x b, d x b products) and the five-term sum in
// FP32.
DF_HD void sigma_point_mixed(const KConstsSig& K, F3 b, DV3 n1, DV3 n2, DV3 t, DV3 x, df64* sig) {
  const DV3 R = x - n1;
  const df64 Rdt = dot(R, t);
  const DV3 nd = R - Rdt * t;
  const df64 d2 = dot(nd, nd);
  const df64 s1 = -Rdt;
  const df64 s2 = -dot(x - n2, t);
  const df64 a2_d2 = K.aSq + d2;
  const df64 a2d2inv = df_recip(a2_d2);
  df64 S[5];
  {
    df64 Ra = df_sqrt(a2_d2 + s1 * s1);
    df64 Rainv = df_recip(Ra);
    df64 Ra3inv = Rainv * Rainv * Rainv;
    df64 sRa3inv = s1 * Ra3inv;
    const df64 s_03a = s1 * Rainv * a2d2inv;
    const df64 s_13a = -Rainv;
    const df64 s_05a = (df_scale(s_03a, 2.0f) + sRa3inv) * a2d2inv;
    const df64 s_15a = -Ra3inv;
    const df64 s_25a = s_03a - sRa3inv;
    Ra = df_sqrt(a2_d2 + s2 * s2);
    Rainv = df_recip(Ra);
    Ra3inv = Rainv * Rainv * Rainv;
    sRa3inv = s2 * Ra3inv;
    const df64 s_03b = s2 * Rainv * a2d2inv;
    const df64 s_13b = -Rainv;
    const df64 s_05b = (df_scale(s_03b, 2.0f) + sRa3inv) * a2d2inv;
    const df64 s_15b = -Ra3inv;
    const df64 s_25b = s_03b - sRa3inv;
    S[0] = s_03b - s_03a;
    S[1] = s_13b - s_13a;
    S[2] = s_05b - s_05a;
    S[3] = s_15b - s_15a;
    S[4] = s_25b - s_25a;
  }
  float Sf[5];
  for (int i = 0; i < 5; ++i) Sf[i] = S[i].hi + S[i].lo;
  const F3 tf = f3(t), dv = f3(nd);
  const F3 txb = cross(tf, b), dxb = cross(dv, b);
  const float common = K.mu4pinu * dot(dxb, tf);
  const float tt[3] = {tf.x, tf.y, tf.z}, dd[3] = {dv.x, dv.y, dv.z};
  const float tb_[3] = {txb.x, txb.y, txb.z}, db_[3] = {dxb.x, dxb.y, dxb.z};
  for (int c = 0; c < 6; ++c) {
    const int p = (c < 3) ? c : (c == 3 ? 0 : (c == 4 ? 0 : 1));
    const int q = (c < 3) ? c : (c == 3 ? 1 : 2);
    float dmd, tmt, tmd, tmtxb, dmtxb, tmdxb;
    if (c < 3) {
      dmd = dd[p] * dd[p];
      tmt = tt[p] * tt[p];
      tmd = 2.0f * tt[p] * dd[p];
      tmtxb = 2.0f * tt[p] * tb_[p];
      dmtxb = 2.0f * dd[p] * tb_[p];
      tmdxb = 2.0f * tt[p] * db_[p];
    } else {
      dmd = dd[p] * dd[q];
      tmt = tt[p] * tt[q];
      tmd = tt[p] * dd[q] + tt[q] * dd[p];
      tmtxb = tt[p] * tb_[q] + tt[q] * tb_[p];
      dmtxb = dd[p] * tb_[q] + dd[q] * tb_[p];
      tmdxb = tt[p] * db_[q] + tt[q] * db_[p];
    }
    const float I03 = (c < 3) ? (common + K.mu4pinu * dmtxb - K.mu4pi * tmdxb) : (K.mu4pinu * dmtxb - K.mu4pi * tmdxb);
    const float I13 = -K.nuMu4pinu * tmtxb;
    const float I05 = (c < 3) ? (common * (K.aSq32 + dmd) - K.aSqMu8pi * tmdxb) : (common * dmd - K.aSqMu8pi * tmdxb);
    const float I15 = K.aSqMu8pi * tmtxb - common * tmd;
    const float I25 = common * tmt;
    sig[c] = sig[c] + (I03 * Sf[0] + I13 * Sf[1] + I05 * Sf[2] + I15 * Sf[3] + I25 * Sf[4]);
  }
}

}  // namespace ddd
