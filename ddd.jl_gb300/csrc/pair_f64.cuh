// FP64 device arithmetic of the non-singular segment–segment force and the
// field-point stress.  The formulas and their evaluation order follow the
// reference (Arsenlis et al. 2007, App. A.1, as written in DDD.jl):
//   src/Processing/DislocationForces.jl:879-1165   calcSegSegForce (general branch)
//   src/Processing/DislocationForces.jl:1167-1442  calcParSegSegForce (near-parallel branch)
//   src/Processing/DislocationForces.jl:1444-1561  ParSegSegInteg / SegSegInteg
//   src/Processing/DislocationFEM.jl:135-299       σ̃ of one segment at one point
// Differences from a literal transcription, all below 1e-13 relative:
//   * t = (n2 - n1)/|n2 - n1| and 1/|n2 - n1| are computed once per segment
//     (same operations the reference repeats per pair);
//   * nvcc contracts a*b + c into FMA in the FMA build (the strict build keeps
//     every multiply and add separate);
//   * log and atan are the integer-pipe functions of intmath_f64.cuh: within
//     0.51 ulp (correctly rounded but for ~1 case in 10^3, like the C library
//     the reference calls), and they take no FP64 pipe time;
//   * the core-correction calls of the near-parallel branch evaluate the general
//     branch directly: their segments make 1 - c^2 = 1.01 sqrt(eps) with the
//     other segment by construction (DislocationForces.jl:1194), so the
//     reference's own branch test always takes the general branch there.
#pragma once
#include <cstdint>

#include "intmath_f64.cuh"

namespace ddd {

struct KConsts {
  double aSq, mu4pi, mu8pi, mu4pinu, nuMu4pinu, mu8piaSq, mu4pinuaSq;
};

// sqrt(eps(Float64)) = 2^-26 (DislocationForces.jl:892,1284,1400) and
// hCotanθc = sqrt((1 - 1.01 sqrt(eps)) / (1.01 sqrt(eps))) / 2 (:1194).
constexpr double kSqrtEps = 1.4901161193847656e-08;
constexpr double kHCotanThetac = 4075.672300430329;

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator-(D3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(D3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// One segment as the pair kernels see it.
struct SegF64 {
  D3 b, n1, n2, t;
  double tN;  // 1 / |n2 - n1|
};

__device__ __forceinline__ void seg_direction(D3 n1, D3 n2, D3& t, double& tN) {
  t = n2 - n1;
  tN = 1.0 / norm(t);
  t = t * tN;
}

// v with its sign flipped when sm is the sign-bit mask (integer pipe, exact).
__device__ __forceinline__ double sgn(double v, unsigned long long sm) {
  return __longlong_as_double(__double_as_longlong(v) ^ (long long)sm);
}

// SegSegInteg at one corner, added (sm = 0) or subtracted (sm = sign bit) into integ[19].
// aSq_dSq = aSq + d^2 (1 - c^2) and den = 1 / sqrt((1 - c^2) aSq_dSq) do not depend
// on the corner; the caller computes them once per pair with the same operations.
__device__ __forceinline__ void seg_seg_integ_acc(double aSq_dSq, double den, double c, double cSq, double omcSqI,
                                                  double x, double y, unsigned long long sm, double* integ) {
  double xSq = x * x;
  double ySq = y * y;
  double Ra = sqrt(aSq_dSq + xSq + ySq + 2.0 * x * y * c);
  double RaInv = 1.0 / Ra;

  double Ra_Rd_t1 = Ra + y + x * c;
  double Ra_Rd_t2 = Ra + x + y * c;

  double log_Ra_Rd_t1 = im::log(Ra_Rd_t1);
  double xlog_Ra_Rd_t1 = x * log_Ra_Rd_t1;
  double log_Ra_Rd_t2 = im::log(Ra_Rd_t2);
  double ylog_Ra_Rd_t2 = y * log_Ra_Rd_t2;

  double RaSq_R_t1_I = RaInv / Ra_Rd_t1;
  double xRaSq_R_t1_I = x * RaSq_R_t1_I;
  double xSqRaSq_R_t1_I = x * xRaSq_R_t1_I;

  double RaSq_R_t2_I = RaInv / Ra_Rd_t2;
  double yRaSq_R_t2_I = y * RaSq_R_t2_I;
  double ySqRaSq_R_t2_I = y * yRaSq_R_t2_I;

  double integ1 = -2.0 * den * im::atan((1.0 + c) * (Ra + x + y) * den);

  double c_1 = aSq_dSq * integ1;
  double c_5_6 = (c * Ra - c_1) * omcSqI;

  double integ2 = (c * log_Ra_Rd_t2 - log_Ra_Rd_t1) * omcSqI;
  double integ3 = (c * log_Ra_Rd_t1 - log_Ra_Rd_t2) * omcSqI;
  double integ4 = (c * c_1 - Ra) * omcSqI;
  double integ5 = ylog_Ra_Rd_t2 + c_5_6;
  double integ6 = xlog_Ra_Rd_t1 + c_5_6;

  double c_11_12 = integ1 - c * RaInv;
  double c_15_18 = c * xRaSq_R_t1_I - RaInv;
  double x_13_14 = x * c_15_18;
  double c_19 = c * yRaSq_R_t2_I - RaInv;
  double y_13_14 = y * c_19;
  double c_16 = log_Ra_Rd_t2 - (x - c * y) * RaInv - cSq * ySqRaSq_R_t2_I;
  double z_15_18 = y * c_16;
  double c_17_19 = log_Ra_Rd_t1 - (y - c * x) * RaInv - cSq * xSqRaSq_R_t1_I;

  double c15_18_19 = 2.0 * integ4;

  integ[0] += sgn(integ1, sm);
  integ[1] += sgn(integ2, sm);
  integ[2] += sgn(integ3, sm);
  integ[3] += sgn(integ4, sm);
  integ[4] += sgn(integ5, sm);
  integ[5] += sgn(integ6, sm);
  integ[6] += sgn(((integ1 - xRaSq_R_t1_I - yRaSq_R_t2_I) / (aSq_dSq)), sm);
  integ[7] += sgn(((RaSq_R_t1_I - c * RaSq_R_t2_I) * omcSqI), sm);
  integ[8] += sgn(((RaSq_R_t2_I - c * RaSq_R_t1_I) * omcSqI), sm);
  integ[9] += sgn(((RaInv - c * (xRaSq_R_t1_I + yRaSq_R_t2_I + integ1)) * omcSqI), sm);
  integ[10] += sgn(((xRaSq_R_t1_I + cSq * yRaSq_R_t2_I + c_11_12) * omcSqI), sm);
  integ[11] += sgn(((yRaSq_R_t2_I + cSq * xRaSq_R_t1_I + c_11_12) * omcSqI), sm);
  integ[12] += sgn(((integ3 - x_13_14 + c * (y_13_14 - integ2)) * omcSqI), sm);
  integ[13] += sgn(((integ2 - y_13_14 + c * (x_13_14 - integ3)) * omcSqI), sm);
  integ[14] += sgn(((integ5 - z_15_18 + c * (xSq * c_15_18 - c15_18_19)) * omcSqI), sm);
  integ[15] += sgn(((xSqRaSq_R_t1_I + c * c_16 + 2.0 * integ2) * omcSqI), sm);
  integ[16] += sgn(((ySqRaSq_R_t2_I + c * c_17_19 + 2.0 * integ3) * omcSqI), sm);
  integ[17] += sgn(((c15_18_19 - xSq * c_15_18 + c * (z_15_18 - integ5)) * omcSqI), sm);
  integ[18] += sgn(((c15_18_19 - ySq * c_19 + c * (x * c_17_19 - integ6)) * omcSqI), sm);
}

__device__ __forceinline__ D3 fsum11(const D3* V, const double* F) {
  D3 s = V[0] * F[0] + V[1] * F[1];
#pragma unroll
  for (int k = 2; k < 11; ++k) s = s + V[k] * F[k];
  return s;
}

// General branch (1 - c^2 > sqrt(eps)) of calcSegSegForce.  NEED12 / NEED34 drop
// the work of the forces on segment 1 / segment 2 when the caller discards them.
template <bool NEED12, bool NEED34>
__device__ __forceinline__ void general_pair(const KConsts& K, D3 b1, D3 n11, D3 n12, D3 t1, double t1N, D3 b2, D3 n21,
                                             D3 n22, D3 t2, double t2N, double c, D3& F1, D3& F2, D3& F3, D3& F4) {
  const double mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, mu8piaSq = K.mu8piaSq, mu4pinuaSq = K.mu4pinuaSq;
  double cSq = c * c;
  double omcSq = 1.0 - cSq;
  double omcSqI = 1.0 / omcSq;

  D3 t2ct1 = cross(t2, t1);
  D3 t1ct2 = -t2ct1;
  D3 b2ct2 = cross(b2, t2);
  D3 b1ct1 = cross(b1, t1);

  double t2db2 = dot(t2, b2);
  double t2db1 = dot(t2, b1);
  double t1db2 = dot(t1, b2);
  double t1db1 = dot(t1, b1);

  double t2ct1db2 = dot(t2ct1, b2);
  double t1ct2db1 = dot(t1ct2, b1);
  double b1ct1db2 = dot(b1ct1, b2);
  double b2ct2db1 = dot(b2ct2, b1);

  D3 t2ct1ct2 = t1 - c * t2;
  D3 t1ct2ct1 = t2 - c * t1;
  D3 t2cb1ct2 = b1 - t2db1 * t2;
  D3 t1cb2ct1 = b2 - t1db2 * t1;
  D3 b1ct1ct2 = t2db1 * t1 - c * b1;
  D3 b2ct2ct1 = t1db2 * t2 - c * b2;

  double t2ct1cb1dt1 = t2db1 - t1db1 * c;
  double t1ct2cb2dt2 = t1db2 - t2db2 * c;
  double t2ct1cb1db2 = t2db1 * t1db2 - t1db1 * t2db2;

  D3 R1 = n21 - n11;
  D3 R2 = n22 - n12;
  double d = dot(R2, t2ct1) * omcSqI;

  double mu4pid = mu4pi * d;
  double mu4pinud = mu4pinu * d;
  double mu4pinudSq = mu4pinud * d;
  double mu4pinudCu = mu4pinudSq * d;
  double mu4pinuaSqd = mu4pinuaSq * d;
  double mu8piaSqd = mu8piaSq * d;

  double lim11 = dot(R1, t1);
  double lim12 = dot(R1, t2);
  double lim21 = dot(R2, t1);
  double lim22 = dot(R2, t2);

  double x1 = (lim12 - c * lim11) * omcSqI;
  double x2 = (lim22 - c * lim21) * omcSqI;
  double y1 = (lim11 - c * lim12) * omcSqI;
  double y2 = (lim21 - c * lim22) * omcSqI;

  double integ[19];
#pragma unroll
  for (int k = 0; k < 19; ++k) integ[k] = 0.0;
  const double aSq_dSq = K.aSq + d * d * omcSq;
  const double den = 1.0 / sqrt(omcSq * aSq_dSq);
  // ((I(x1,y1) - I(x1,y2)) - I(x2,y1)) + I(x2,y2), DislocationForces.jl:948-951.
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    double x = (q & 2) ? x2 : x1;
    double y = (q & 1) ? y2 : y1;
    unsigned long long sm = (q == 1 || q == 2) ? 0x8000000000000000ull : 0ull;
    seg_seg_integ_acc(aSq_dSq, den, c, cSq, omcSqI, x, y, sm, integ);
  }

  D3 V[11];
  double Fi[11];
  double tmp1, tmp2;
  if (NEED12) {
    tmp1 = t1db2 * t2db1 + t2ct1cb1db2;
    D3 V1 = tmp1 * t2ct1;
    D3 V2 = b1ct1 * t1ct2cb2dt2;
    D3 V3 = t1ct2 * b1ct1db2 - t1cb2ct1 * t2db1;
    D3 V4 = -b1ct1 * t2ct1db2;
    D3 V5 = b2ct2ct1 * t2db1 - t1ct2 * b2ct2db1;

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
    D3 tv = mu4pinu * t2ct1db2 * t1ct2;
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
    F1 = fsum11(V, Fi) * t1N;

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
    F2 = fsum11(V, Fi) * t1N;
  }
  if (NEED34) {
    tmp1 = t2db1 * t1db2 + t2ct1cb1db2;
    D3 V1 = tmp1 * t1ct2;
    D3 V2 = b2ct2 * t2ct1cb1dt1;
    D3 V3 = t2ct1 * b1ct1db2 - b1ct1ct2 * t1db2;
    D3 V5 = t2cb1ct2 * t1db2 - t2ct1 * b2ct2db1;
    D3 V6 = b2ct2 * t1ct2db1;

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
    D3 tv = mu4pinu * t1ct2db1 * t2ct1;
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
    F3 = fsum11(V, Fi) * t2N;

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
    F4 = fsum11(V, Fi) * t2N;
  }
}

// ParSegSegInteg at one corner, added or subtracted (sm) into integ[12].
__device__ __forceinline__ void par_seg_seg_integ_acc(double aSq_dSq, double aSq_dSqI, double x, double y,
                                                      unsigned long long sm, double* integ) {
  double xpy = x + y;
  double xmy = x - y;
  double Ra = sqrt(aSq_dSq + xpy * xpy);
  double RaInv = 1.0 / Ra;
  double Log_Ra_ypz = im::log(Ra + xpy);
  double tmp = xmy * Ra * aSq_dSqI;
  double i10 = -aSq_dSqI * xpy * RaInv;
  integ[0] += sgn((Ra * aSq_dSqI), sm);
  integ[1] += sgn((-0.5 * (Log_Ra_ypz - tmp)), sm);
  integ[2] += sgn((-0.5 * (Log_Ra_ypz + tmp)), sm);
  integ[3] += sgn((-Log_Ra_ypz), sm);
  integ[4] += sgn((y * Log_Ra_ypz - Ra), sm);
  integ[5] += sgn((x * Log_Ra_ypz - Ra), sm);
  integ[6] += sgn((aSq_dSqI * (2.0 * aSq_dSqI * Ra - RaInv)), sm);
  integ[7] += sgn((aSq_dSqI * (tmp - x * RaInv)), sm);
  integ[8] += sgn((-aSq_dSqI * (tmp + y * RaInv)), sm);
  integ[9] += sgn(i10, sm);
  integ[10] += sgn((RaInv - y * i10), sm);
  integ[11] += sgn((RaInv - x * i10), sm);
}

// One side of calcParSegSegForce: the analytic parallel part on segment "a"
// (nodes na1 -> na2, direction ta, inverse length taN, Burgers ba) due to the
// segment "b" (nb1 -> nb2, Burgers bb), projected onto a's line and rotated by
// θc, plus the two core-correction evaluations.  SIDE 1 is DislocationForces.jl
// :1204-1317 (returns Fnode1, Fnode2); SIDE 2 is :1319-1433 (Fnode3, Fnode4),
// whose projection roles and integration-variable roles are mirrored.
// Returns 1 when the core corrections were applied, else 0.
template <int SIDE>
__device__ __forceinline__ int par_side(const KConsts& K, D3 na1, D3 na2, D3 ta, double taN, D3 ba, D3 nb1, D3 nb2,
                                        D3 tb, double tbN, D3 bb, D3& Fa1, D3& Fa2) {
  const double mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, mu8piaSq = K.mu8piaSq, mu4pinuaSq = K.mu4pinuaSq;
  // Project segment b onto segment a's line: nbm1/nbm2 are b's nodes moved onto
  // a's line and pulled apart by the critical angle.
  double tmp = dot(nb2 - nb1, ta);
  D3 nbm2 = nb1 + tmp * ta;
  D3 diff = nb2 - nbm2;
  double magDiff = norm(diff);
  D3 tv1 = 0.5 * diff;
  D3 tv2 = kHCotanThetac * magDiff * ta;
  D3 nbm1 = nb1 + tv1 + tv2;
  nbm2 = nbm2 + tv1 - tv2;

  D3 R, nd;
  double x1, x2, y1, y2;
  if (SIDE == 1) {
    R = nbm1 - na1;
    double Rdt = dot(R, ta);
    nd = R - Rdt * ta;
    x1 = dot(nbm1, ta);
    x2 = dot(nbm2, ta);
    y1 = -dot(na1, ta);
    y2 = -dot(na2, ta);
  } else {
    R = na1 - nbm1;
    double Rdt = dot(R, ta);
    nd = R - Rdt * ta;
    x1 = dot(na1, ta);
    x2 = dot(na2, ta);
    y1 = -dot(nbm1, ta);
    y2 = -dot(nbm2, ta);
  }
  double dSq = dot(nd, nd);
  double aSq_dSq = K.aSq + dSq;
  double aSq_dSqI = 1.0 / aSq_dSq;

  double tadbb = dot(ta, bb);
  double tadba = dot(ta, ba);
  double nddba = dot(nd, ba);
  D3 bbcta = cross(bb, ta);
  D3 bacta = cross(ba, ta);
  D3 ndcta = cross(nd, ta);
  double bbctadba = dot(bbcta, ba);
  double bbctadnd = dot(bbcta, nd);
  D3 bbctacta = tadbb * ta - bb;

  double integ[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) integ[k] = 0.0;
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    double x = (q & 2) ? x2 : x1;
    double y = (q & 1) ? y2 : y1;
    unsigned long long sm = (q == 1 || q == 2) ? 0x8000000000000000ull : 0ull;
    par_seg_seg_integ_acc(aSq_dSq, aSq_dSqI, x, y, sm, integ);
  }

  tmp = tadba * tadbb;
  D3 w1 = tmp * nd;
  D3 w2 = bbctadnd * bacta;
  D3 V1 = mu4pinu * (nddba * bbctacta + bbctadba * ndcta - w2) - mu4pi * w1;
  tmp = (mu4pinu - mu4pi) * tadba;
  D3 V2 = tmp * bbctacta;
  tmp = mu4pinu * bbctadnd * nddba;
  D3 V3 = -mu8piaSq * w1 - mu4pinuaSq * w2 - tmp * ndcta;
  tmp = mu8piaSq * tadba;
  double tmp2 = mu4pinu * bbctadnd * tadba;
  D3 V4 = -tmp * bbctacta - tmp2 * ndcta;

  double Fint1, Fint2, Fint3, Fint4;
  if (SIDE == 1) {
    Fint1 = integ[2] - y1 * integ[0];
    Fint2 = integ[5] - y1 * integ[3];
    Fint3 = integ[8] - y1 * integ[6];
    Fint4 = integ[11] - y1 * integ[9];
    Fa2 = (V1 * Fint1 + V2 * Fint2 + V3 * Fint3 + V4 * Fint4) * taN;
    Fint1 = y2 * integ[0] - integ[2];
    Fint2 = y2 * integ[3] - integ[5];
    Fint3 = y2 * integ[6] - integ[8];
    Fint4 = y2 * integ[9] - integ[11];
    Fa1 = (V1 * Fint1 + V2 * Fint2 + V3 * Fint3 + V4 * Fint4) * taN;
  } else {
    Fint1 = integ[1] - x1 * integ[0];
    Fint2 = integ[4] - x1 * integ[3];
    Fint3 = integ[7] - x1 * integ[6];
    Fint4 = integ[10] - x1 * integ[9];
    Fa2 = (V1 * Fint1 + V2 * Fint2 + V3 * Fint3 + V4 * Fint4) * taN;
    Fint1 = x2 * integ[0] - integ[1];
    Fint2 = x2 * integ[3] - integ[4];
    Fint3 = x2 * integ[6] - integ[7];
    Fint4 = x2 * integ[9] - integ[10];
    Fa1 = (V1 * Fint1 + V2 * Fint2 + V3 * Fint3 + V4 * Fint4) * taN;
  }

  // Core corrections (DislocationForces.jl:1280-1317, :1396-1433): the two
  // connector segments nb1 -> nbm1 and nbm2 -> nb2 acting on segment a.
  double magDiffSq = (SIDE == 1) ? dot(diff, diff) : magDiff * magDiff;
  double m1 = dot(nbm1, nbm1);
  double m2 = dot(nbm2, nbm2);
  if (magDiffSq > kSqrtEps * (m1 + m2)) {
    D3 F1, F2, F3, F4, tc;
    double tcN, c;
    seg_direction(nb1, nbm1, tc, tcN);
    c = dot(tc, ta);
    general_pair<false, true>(K, bb, nb1, nbm1, tc, tcN, ba, na1, na2, ta, taN, c, F1, F2, F3, F4);
    Fa1 = Fa1 + F3;
    Fa2 = Fa2 + F4;
    seg_direction(nbm2, nb2, tc, tcN);
    c = dot(tc, ta);
    general_pair<false, true>(K, bb, nbm2, nb2, tc, tcN, ba, na1, na2, ta, taN, c, F1, F2, F3, F4);
    Fa1 = Fa1 + F3;
    Fa2 = Fa2 + F4;
    (void)tb;
    (void)tbN;
    return 1;
  }
  return 0;
}

// calcParSegSegForce (DislocationForces.jl:1167-1442).  NEED34 = false skips
// the second side (the index-list form discards it).  Returns the number of
// sides (0-2) that needed the two core-correction evaluations.
template <bool NEED34>
__device__ __forceinline__ int parallel_pair(const KConsts& K, D3 b1, D3 n11, D3 n12, D3 t1, double t1N, D3 b2,
                                              D3 n21, D3 n22, D3 t2, double t2N, double c, D3& F1, D3& F2, D3& F3,
                                              D3& F4) {
  bool flip = c < 0.0;
  if (flip) {
    D3 tmp = n11;
    n11 = n12;
    n12 = tmp;
    t1 = -t1;
    b1 = -b1;
  }
  int cores = par_side<1>(K, n11, n12, t1, t1N, b1, n21, n22, t2, t2N, b2, F1, F2);
  if (NEED34) cores += par_side<2>(K, n21, n22, t2, t2N, b2, n11, n12, t1, t1N, b1, F3, F4);
  if (flip) {
    D3 tmp = F1;
    F1 = F2;
    F2 = tmp;
  }
  return cores;
}

// σ̃ of one segment at one point, added into sig[6] (xx, yy, zz, xy, xz, yz).
// txb = t x b depends on the segment only: the caller computes it once per
// segment with the same operations (the same bits as computing it here).
__device__ __forceinline__ void sigma_point(const KConsts& K, D3 b, D3 n1, D3 n2, D3 t, D3 txb, D3 x, double* sig) {
  const double mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, nuMu4pinu = K.nuMu4pinu, a2 = K.aSq;
  const double a2mu8pi = a2 * K.mu8pi;
  D3 R = x - n1;
  double Rdt = dot(R, t);
  D3 nd = R - Rdt * t;
  double d2 = dot(nd, nd);
  double s1 = -Rdt;
  double s2 = -dot(x - n2, t);
  double a2_d2 = a2 + d2;
  double a2d2inv = 1.0 / a2_d2;

  double Ra = sqrt(a2_d2 + s1 * s1);
  double Rainv = 1.0 / Ra;
  double Ra3inv = Rainv * Rainv * Rainv;
  double sRa3inv = s1 * Ra3inv;
  double s_03a = s1 * Rainv * a2d2inv;
  double s_13a = -Rainv;
  double s_05a = (2.0 * s_03a + sRa3inv) * a2d2inv;
  double s_15a = -Ra3inv;
  double s_25a = s_03a - sRa3inv;

  Ra = sqrt(a2_d2 + s2 * s2);
  Rainv = 1.0 / Ra;
  Ra3inv = Rainv * Rainv * Rainv;
  sRa3inv = s2 * Ra3inv;
  double s_03b = s2 * Rainv * a2d2inv;
  double s_13b = -Rainv;
  double s_05b = (2.0 * s_03b + sRa3inv) * a2d2inv;
  double s_15b = -Ra3inv;
  double s_25b = s_03b - sRa3inv;

  double s_03 = s_03b - s_03a;
  double s_13 = s_13b - s_13a;
  double s_05 = s_05b - s_05a;
  double s_15 = s_15b - s_15a;
  double s_25 = s_25b - s_25a;

  D3 dxb = cross(nd, b);
  double dxbdt = dot(dxb, t);
  double common = mu4pinu * dxbdt;

  // Component tables: (xx, yy, zz, xy, xz, yz) index pairs.
  const double tt[3] = {t.x, t.y, t.z};
  const double dd[3] = {nd.x, nd.y, nd.z};
  const double tb_[3] = {txb.x, txb.y, txb.z};
  const double db_[3] = {dxb.x, dxb.y, dxb.z};
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const int p = (c < 3) ? c : (c == 3 ? 0 : (c == 4 ? 0 : 1));
    const int q = (c < 3) ? c : (c == 3 ? 1 : 2);
    double dmd, tmt, tmd, tmtxb, dmtxb, tmdxb;
    if (c < 3) {
      dmd = dd[p] * dd[p];
      tmt = tt[p] * tt[p];
      tmd = 2.0 * tt[p] * dd[p];
      tmtxb = 2.0 * tt[p] * tb_[p];
      dmtxb = 2.0 * dd[p] * tb_[p];
      tmdxb = 2.0 * tt[p] * db_[p];
    } else {
      dmd = dd[p] * dd[q];
      tmt = tt[p] * tt[q];
      tmd = tt[p] * dd[q] + tt[q] * dd[p];
      tmtxb = tt[p] * tb_[q] + tt[q] * tb_[p];
      dmtxb = dd[p] * tb_[q] + dd[q] * tb_[p];
      tmdxb = tt[p] * db_[q] + tt[q] * db_[p];
    }
    double I03 = (c < 3) ? (common + mu4pinu * dmtxb - mu4pi * tmdxb) : (mu4pinu * dmtxb - mu4pi * tmdxb);
    double I13 = -nuMu4pinu * tmtxb;
    double I05 = (c < 3) ? (common * (a2 + dmd) - a2mu8pi * tmdxb) : (common * dmd - a2mu8pi * tmdxb);
    double I15 = a2mu8pi * tmtxb - common * tmd;
    double I25 = common * tmt;
    sig[c] += I03 * s_03 + I13 * s_13 + I05 * s_05 + I15 * s_15 + I25 * s_25;
  }
}

}  // namespace ddd
