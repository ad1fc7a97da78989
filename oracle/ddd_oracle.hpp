// CPU ORACLE — test infrastructure only.
//
// A scalar-type-templated C++ restatement of the reference DDD.jl arithmetic for
// the segment–segment force and field-point stress hot path.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this code; the
// product library (libddd_gb300.so) never links or calls it.
//
// Every function keeps the reference's operation order (Julia evaluates
// `a + b + c` as `(a + b) + c`, `s * t * v` as `(s * t) * v`, and never fuses a
// multiply-add unless asked), so the library built from this header with
// -ffp-contract=off reproduces the reference's Float64 rounding up to the
// last-ulp differences of libm's log/atan/sqrt versus Julia's own.
//
// Parity pin: tests/test_oracle_golden.py checks this oracle against every
// golden vector of the reference tests for this path
// (test/SegmentForcesTest.jl:281-443, test/DislocationFEMTest.jl:5-155).
//
// Reference files restated (paths within the DDD.jl project):
//   src/Processing/DislocationForces.jl:670-877   drivers (unroll, Par, Ser, Idx)
//   src/Processing/DislocationForces.jl:879-1165  pair kernel calcSegSegForce
//   src/Processing/DislocationForces.jl:1167-1442 near-parallel branch calcParSegSegForce
//   src/Processing/DislocationForces.jl:1444-1478 ParSegSegInteg
//   src/Processing/DislocationForces.jl:1480-1561 SegSegInteg
//   src/Processing/DislocationFEM.jl:86-303       _calc_σTilde!
//   src/Misc/Misc.jl:314-367                      minimumDistance
//   src/Processing/DislocationTopologyCollision.jl:1-221  detectCollision
//   src/Processing/DislocationFEM.jl:355-707      calc_uTilde, Barnett triangles
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>
#include <utility>
#include <vector>
#include <algorithm>

namespace ddd_oracle {

// ---------------------------------------------------------------------------
// 3-vectors with the StaticArrays semantics used by the reference.
// dot = (x1*y1 + x2*y2) + x3*y3, cross = (a2b3-a3b2, a3b1-a1b3, a1b2-a2b1),
// norm = sqrt((x1^2 + x2^2) + x3^2).
template <class T> struct V3 {
  T x, y, z;
};
template <class T> inline V3<T> operator+(const V3<T>& a, const V3<T>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(const V3<T>& a, const V3<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(const V3<T>& a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(const T& s, const V3<T>& a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator*(const V3<T>& a, const T& s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline T dot(const V3<T>& a, const V3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(const V3<T>& a, const V3<T>& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T norm(const V3<T>& a) {
  using std::sqrt;
  return sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
}

// sqrt(eps(Float64)) = 2^-26, the near-parallel threshold of
// DislocationForces.jl:892,1284,1400.  The threshold is always the Float64 one,
// whatever scalar type instantiates the templates, so that reduced-precision
// studies classify pairs exactly as the reference does.
constexpr double kSqrtEps = 1.4901161193847656e-08;
// Half the cotangent of the critical angle, sqrt((1 - 1.01 sqrt(eps)) / (1.01 sqrt(eps))) / 2
// (DislocationForces.jl:1194), evaluated in Float64.
inline double kHCotanThetac() { return std::sqrt((1.0 - kSqrtEps * 1.01) / (kSqrtEps * 1.01)) / 2.0; }

// Material and core constants (MaterialConstructor.jl:73-82,
// DislocationConstructor.jl:83, DislocationForces.jl:676-682, DislocationFEM.jl:95-100).
template <class T> struct Consts {
  T aSq;      // dlnParams.coreRadSq
  T mu4pi;    // μ / (4π)
  T mu8pi;    // μ4π / 2
  T mu4pinu;  // μ4π / (1 - ν)
  T nuMu4pinu;  // ν μ4πν
  T mu8piaSq;   // aSq * μ8π   (DislocationForces.jl:681)
  T mu4pinuaSq; // aSq * μ4πν  (DislocationForces.jl:682)
};

// ---------------------------------------------------------------------------
// SegSegInteg — DislocationForces.jl:1480-1561.  19 antiderivative terms at one
// (x, y) corner of the integration domain.
template <class T>
inline void seg_seg_integ(T aSq, T d, T c, T cSq, T omcSq, T omcSqI, T x, T y, T* I) {
  using std::atan;
  using std::log;
  using std::sqrt;
  T aSq_dSq = aSq + d * d * omcSq;
  T xSq = x * x;
  T ySq = y * y;
  T Ra = sqrt(aSq_dSq + xSq + ySq + T(2) * x * y * c);
  T RaInv = T(1) / Ra;

  T Ra_Rd_t1 = Ra + y + x * c;
  T Ra_Rd_t2 = Ra + x + y * c;

  T log_Ra_Rd_t1 = log(Ra_Rd_t1);
  T xlog_Ra_Rd_t1 = x * log_Ra_Rd_t1;

  T log_Ra_Rd_t2 = log(Ra_Rd_t2);
  T ylog_Ra_Rd_t2 = y * log_Ra_Rd_t2;

  T RaSq_R_t1_I = RaInv / Ra_Rd_t1;
  T xRaSq_R_t1_I = x * RaSq_R_t1_I;
  T xSqRaSq_R_t1_I = x * xRaSq_R_t1_I;

  T RaSq_R_t2_I = RaInv / Ra_Rd_t2;
  T yRaSq_R_t2_I = y * RaSq_R_t2_I;
  T ySqRaSq_R_t2_I = y * yRaSq_R_t2_I;

  T den = T(1) / sqrt(omcSq * aSq_dSq);

  T integ1 = T(-2) * den * atan((T(1) + c) * (Ra + x + y) * den);

  T c_1 = aSq_dSq * integ1;
  T c_5_6 = (c * Ra - c_1) * omcSqI;

  T integ2 = (c * log_Ra_Rd_t2 - log_Ra_Rd_t1) * omcSqI;
  T integ3 = (c * log_Ra_Rd_t1 - log_Ra_Rd_t2) * omcSqI;
  T integ4 = (c * c_1 - Ra) * omcSqI;
  T integ5 = ylog_Ra_Rd_t2 + c_5_6;
  T integ6 = xlog_Ra_Rd_t1 + c_5_6;

  T c_11_12 = integ1 - c * RaInv;
  T c_15_18 = c * xRaSq_R_t1_I - RaInv;
  T x_13_14 = x * c_15_18;
  T c_19 = c * yRaSq_R_t2_I - RaInv;
  T y_13_14 = y * c_19;
  T c_16 = log_Ra_Rd_t2 - (x - c * y) * RaInv - cSq * ySqRaSq_R_t2_I;
  T z_15_18 = y * c_16;
  T c_17_19 = log_Ra_Rd_t1 - (y - c * x) * RaInv - cSq * xSqRaSq_R_t1_I;

  T c15_18_19 = T(2) * integ4;

  I[0] = integ1;
  I[1] = integ2;
  I[2] = integ3;
  I[3] = integ4;
  I[4] = integ5;
  I[5] = integ6;
  I[6] = (integ1 - xRaSq_R_t1_I - yRaSq_R_t2_I) / (aSq_dSq);
  I[7] = (RaSq_R_t1_I - c * RaSq_R_t2_I) * omcSqI;
  I[8] = (RaSq_R_t2_I - c * RaSq_R_t1_I) * omcSqI;
  I[9] = (RaInv - c * (xRaSq_R_t1_I + yRaSq_R_t2_I + integ1)) * omcSqI;
  I[10] = (xRaSq_R_t1_I + cSq * yRaSq_R_t2_I + c_11_12) * omcSqI;
  I[11] = (yRaSq_R_t2_I + cSq * xRaSq_R_t1_I + c_11_12) * omcSqI;
  I[12] = (integ3 - x_13_14 + c * (y_13_14 - integ2)) * omcSqI;
  I[13] = (integ2 - y_13_14 + c * (x_13_14 - integ3)) * omcSqI;
  I[14] = (integ5 - z_15_18 + c * (xSq * c_15_18 - c15_18_19)) * omcSqI;
  I[15] = (xSqRaSq_R_t1_I + c * c_16 + T(2) * integ2) * omcSqI;
  I[16] = (ySqRaSq_R_t2_I + c * c_17_19 + T(2) * integ3) * omcSqI;
  I[17] = (c15_18_19 - xSq * c_15_18 + c * (z_15_18 - integ5)) * omcSqI;
  I[18] = (c15_18_19 - ySq * c_19 + c * (x * c_17_19 - integ6)) * omcSqI;
}

// ParSegSegInteg — DislocationForces.jl:1444-1478.  12 terms for parallel segments.
template <class T> inline void par_seg_seg_integ(T aSq_dSq, T aSq_dSqI, T x, T y, T* I) {
  using std::log;
  using std::sqrt;
  T xpy = x + y;
  T xmy = x - y;
  T Ra = sqrt(aSq_dSq + xpy * xpy);
  T RaInv = T(1) / Ra;
  T Log_Ra_ypz = log(Ra + xpy);

  T tmp = xmy * Ra * aSq_dSqI;

  I[0] = Ra * aSq_dSqI;
  I[1] = T(-0.5) * (Log_Ra_ypz - tmp);
  I[2] = T(-0.5) * (Log_Ra_ypz + tmp);
  I[3] = -Log_Ra_ypz;
  I[4] = y * Log_Ra_ypz - Ra;
  I[5] = x * Log_Ra_ypz - Ra;
  I[6] = aSq_dSqI * (T(2) * aSq_dSqI * Ra - RaInv);
  I[7] = aSq_dSqI * (tmp - x * RaInv);
  I[8] = -aSq_dSqI * (tmp + y * RaInv);
  I[9] = -aSq_dSqI * xpy * RaInv;
  I[10] = RaInv - y * I[9];
  I[11] = RaInv - x * I[9];
}

// Corner combination I(x1,y1) - I(x1,y2) - I(x2,y1) + I(x2,y2) evaluated
// left to right as the reference's broadcasts do (DislocationForces.jl:948-951).
template <class T>
inline void seg_seg_integ_corners(T aSq, T d, T c, T cSq, T omcSq, T omcSqI, T x1, T x2, T y1, T y2, T* integ) {
  T tmp[19];
  seg_seg_integ(aSq, d, c, cSq, omcSq, omcSqI, x1, y1, integ);
  seg_seg_integ(aSq, d, c, cSq, omcSq, omcSqI, x1, y2, tmp);
  for (int k = 0; k < 19; ++k) integ[k] = integ[k] - tmp[k];
  seg_seg_integ(aSq, d, c, cSq, omcSq, omcSqI, x2, y1, tmp);
  for (int k = 0; k < 19; ++k) integ[k] = integ[k] - tmp[k];
  seg_seg_integ(aSq, d, c, cSq, omcSq, omcSqI, x2, y2, tmp);
  for (int k = 0; k < 19; ++k) integ[k] = integ[k] + tmp[k];
}

template <class T>
inline V3<T> sum11(const V3<T>* V, const T* F) {
  // (V7*F1 + V8*F2 + ... + V17*F11), left fold.
  V3<T> s = V[0] * F[0] + V[1] * F[1];
  for (int k = 2; k < 11; ++k) s = s + V[k] * F[k];
  return s;
}

template <class T>
void par_seg_seg_force(const Consts<T>& K, V3<T> b1, V3<T> n11, V3<T> n12, V3<T> b2, V3<T> n21, V3<T> n22,
                       V3<T>* F);

// calcSegSegForce(aSq, μ4π, μ8π, μ8πaSq, μ4πν, μ4πνaSq, b1, n11, n12, b2, n21, n22)
// — DislocationForces.jl:879-1165.  F[0..3] = Fnode1..Fnode4 (forces on n11, n12, n21, n22).
template <class T>
void seg_seg_force(const Consts<T>& K, V3<T> b1, V3<T> n11, V3<T> n12, V3<T> b2, V3<T> n21, V3<T> n22, V3<T>* F) {
  const T aSq = K.aSq, mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, mu8piaSq = K.mu8piaSq, mu4pinuaSq = K.mu4pinuaSq;
  V3<T> t2 = n22 - n21;
  T t2N = T(1) / norm(t2);
  t2 = t2 * t2N;

  V3<T> t1 = n12 - n11;
  T t1N = T(1) / norm(t1);
  t1 = t1 * t1N;

  T c = dot(t1, t2);
  T cSq = c * c;
  T omcSq = T(1) - cSq;

  if (omcSq > T(kSqrtEps)) {
    T omcSqI = T(1) / omcSq;

    V3<T> t2ct1 = cross(t2, t1);
    V3<T> t1ct2 = -t2ct1;
    V3<T> b2ct2 = cross(b2, t2);
    V3<T> b1ct1 = cross(b1, t1);

    T t2db2 = dot(t2, b2);
    T t2db1 = dot(t2, b1);
    T t1db2 = dot(t1, b2);
    T t1db1 = dot(t1, b1);

    T t2ct1db2 = dot(t2ct1, b2);
    T t1ct2db1 = dot(t1ct2, b1);
    T b1ct1db2 = dot(b1ct1, b2);
    T b2ct2db1 = dot(b2ct2, b1);

    V3<T> t2ct1ct2 = t1 - c * t2;
    V3<T> t1ct2ct1 = t2 - c * t1;
    V3<T> t2cb1ct2 = b1 - t2db1 * t2;
    V3<T> t1cb2ct1 = b2 - t1db2 * t1;
    V3<T> b1ct1ct2 = t2db1 * t1 - c * b1;
    V3<T> b2ct2ct1 = t1db2 * t2 - c * b2;

    T t2ct1cb1dt1 = t2db1 - t1db1 * c;
    T t1ct2cb2dt2 = t1db2 - t2db2 * c;
    T t2ct1cb1db2 = t2db1 * t1db2 - t1db1 * t2db2;

    V3<T> R1 = n21 - n11;
    V3<T> R2 = n22 - n12;
    T d = dot(R2, t2ct1) * omcSqI;

    T mu4pid = mu4pi * d;
    T mu4pinud = mu4pinu * d;
    T mu4pinudSq = mu4pinud * d;
    T mu4pinudCu = mu4pinudSq * d;
    T mu4pinuaSqd = mu4pinuaSq * d;
    T mu8piaSqd = mu8piaSq * d;

    T lim11 = dot(R1, t1);
    T lim12 = dot(R1, t2);
    T lim21 = dot(R2, t1);
    T lim22 = dot(R2, t2);

    T x1 = (lim12 - c * lim11) * omcSqI;
    T x2 = (lim22 - c * lim21) * omcSqI;
    T y1 = (lim11 - c * lim12) * omcSqI;
    T y2 = (lim21 - c * lim22) * omcSqI;

    T integ[19];
    seg_seg_integ_corners(aSq, d, c, cSq, omcSq, omcSqI, x1, x2, y1, y2, integ);

    V3<T> V[11];
    T Fi[11];
    T tmp1, tmp2;
    // Seg 1, nodes 2-1 (DislocationForces.jl:953-1048).
    {
      tmp1 = t1db2 * t2db1 + t2ct1cb1db2;
      V3<T> V1 = tmp1 * t2ct1;
      V3<T> V2 = b1ct1 * t1ct2cb2dt2;
      V3<T> V3_ = t1ct2 * b1ct1db2 - t1cb2ct1 * t2db1;
      V3<T> V4 = -b1ct1 * t2ct1db2;
      V3<T> V5 = b2ct2ct1 * t2db1 - t1ct2 * b2ct2db1;

      tmp1 = mu4pinud * t1ct2db1;
      tmp2 = mu4pinud * b2ct2db1;
      V[0] = mu4pid * V1 - mu4pinud * V2 + tmp1 * b2ct2ct1 + tmp2 * t1ct2ct1;  // V7

      tmp1 = mu4pinu * t2db1;
      tmp2 = mu4pinu * b2ct2db1;
      V[1] = mu4pi * V5 - tmp1 * b2ct2ct1 + tmp2 * t1ct2;  // V8

      tmp1 = mu4pinu * t1db1;
      V[2] = -tmp1 * b2ct2ct1 + mu4pi * V3_ - mu4pinu * V4;  // V9

      tmp1 = mu4pinudCu * t1ct2cb2dt2 * t1ct2db1;
      V[3] = mu8piaSqd * V1 - mu4pinuaSqd * V2 - tmp1 * t1ct2ct1;  // V10

      tmp1 = mu4pinudSq * t1ct2cb2dt2 * t2db1;
      tmp2 = mu4pinudSq * t1ct2cb2dt2 * t1ct2db1;
      V[4] = mu8piaSq * V5 + tmp1 * t1ct2ct1 - tmp2 * t1ct2;  // V11

      tmp1 = mu4pinudSq * (t2ct1db2 * t1ct2db1 + t1ct2cb2dt2 * t1db1);
      V[5] = mu8piaSq * V3_ - mu4pinuaSq * V4 + tmp1 * t1ct2ct1;  // V12

      tmp1 = mu4pinud * (t1ct2cb2dt2 * t1db1 + t2ct1db2 * t1ct2db1);
      tmp2 = mu4pinud * t2ct1db2 * t2db1;
      V[6] = tmp1 * t1ct2 - tmp2 * t1ct2ct1;  // V13

      tmp1 = mu4pinud * t1ct2cb2dt2 * t2db1;
      V[7] = tmp1 * t1ct2;  // V14

      tmp1 = mu4pinud * t2ct1db2 * t1db1;
      V[8] = -tmp1 * t1ct2ct1;  // V15

      V3<T> tmpVec1 = mu4pinu * t2ct1db2 * t1ct2;
      V[9] = -tmpVec1 * t2db1;   // V16
      V[10] = -tmpVec1 * t1db1;  // V17

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
      F[0] = sum11(V, Fi) * t1N;

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
      F[1] = sum11(V, Fi) * t1N;
    }
    // Seg 2, nodes 4-3 (DislocationForces.jl:1050-1145).
    {
      tmp1 = t2db1 * t1db2 + t2ct1cb1db2;
      V3<T> V1 = tmp1 * t1ct2;
      V3<T> V2 = b2ct2 * t2ct1cb1dt1;
      V3<T> V3_ = t2ct1 * b1ct1db2 - b1ct1ct2 * t1db2;
      V3<T> V5 = t2cb1ct2 * t1db2 - t2ct1 * b2ct2db1;
      V3<T> V6 = b2ct2 * t1ct2db1;

      tmp1 = mu4pinud * t2ct1db2;
      tmp2 = mu4pinud * b1ct1db2;
      V[0] = mu4pid * V1 - mu4pinud * V2 + tmp1 * b1ct1ct2 + tmp2 * t2ct1ct2;  // V7

      tmp1 = mu4pinu * t2db2;
      V[1] = tmp1 * b1ct1ct2 + mu4pi * V5 - mu4pinu * V6;  // V8

      tmp1 = mu4pinu * t1db2;
      tmp2 = mu4pinu * b1ct1db2;
      V[2] = mu4pi * V3_ + tmp1 * b1ct1ct2 - tmp2 * t2ct1;  // V9

      tmp1 = mu4pinudCu * t2ct1cb1dt1 * t2ct1db2;
      V[3] = mu8piaSqd * V1 - mu4pinuaSqd * V2 - tmp1 * t2ct1ct2;  // V10

      tmp1 = mu4pinudSq * (t1ct2db1 * t2ct1db2 + t2ct1cb1dt1 * t2db2);
      V[4] = mu8piaSq * V5 - mu4pinuaSq * V6 - tmp1 * t2ct1ct2;  // V11

      tmp1 = mu4pinudSq * t2ct1cb1dt1 * t1db2;
      tmp2 = mu4pinudSq * t2ct1cb1dt1 * t2ct1db2;
      V[5] = mu8piaSq * V3_ - tmp1 * t2ct1ct2 + tmp2 * t2ct1;  // V12

      tmp1 = mu4pinud * (t2ct1cb1dt1 * t2db2 + t1ct2db1 * t2ct1db2);
      tmp2 = mu4pinud * t1ct2db1 * t1db2;
      V[6] = tmp1 * t2ct1 - tmp2 * t2ct1ct2;  // V13

      tmp1 = mu4pinud * t1ct2db1 * t2db2;
      V[7] = -tmp1 * t2ct1ct2;  // V14

      tmp1 = mu4pinud * t2ct1cb1dt1 * t1db2;
      V[8] = tmp1 * t2ct1;  // V15

      V3<T> tmpVec1 = mu4pinu * t1ct2db1 * t2ct1;
      V[9] = tmpVec1 * t2db2;   // V16
      V[10] = tmpVec1 * t1db2;  // V17

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
      F[2] = sum11(V, Fi) * t2N;

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
      F[3] = sum11(V, Fi) * t2N;
    }
  } else {
    par_seg_seg_force(K, b1, n11, n12, b2, n21, n22, F);
  }
}

// One side of calcParSegSegForce's analytic part (DislocationForces.jl:1215-1281
// for seg 1, :1319-1397 for seg 2) is written out twice below to keep the exact
// statement order of each side.
//
// calcParSegSegForce — DislocationForces.jl:1167-1442.
template <class T>
void par_seg_seg_force(const Consts<T>& K, V3<T> b1, V3<T> n11, V3<T> n12, V3<T> b2, V3<T> n21, V3<T> n22,
                       V3<T>* F) {
  const T aSq = K.aSq, mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, mu8piaSq = K.mu8piaSq, mu4pinuaSq = K.mu4pinuaSq;
  bool flip = false;

  V3<T> t2 = n22 - n21;
  T t2N = T(1) / norm(t2);
  t2 = t2 * t2N;

  V3<T> t1 = n12 - n11;
  T t1N = T(1) / norm(t1);
  t1 = t1 * t1N;

  T c = dot(t2, t1);

  // hCotanθc of DislocationForces.jl:1194, a constant that Julia folds at compile time.
  const T hCotanThetac = T(kHCotanThetac());

  if (c < T(0)) {
    flip = true;
    V3<T> tmpn = n11;
    n11 = n12;
    n12 = tmpn;
    t1 = -t1;
    b1 = -b1;
  }

  V3<T> Fnode1, Fnode2, Fnode3, Fnode4;
  // ---- Segment 1 ----
  {
    T tmp = dot(n22 - n21, t1);
    V3<T> n22m = n21 + tmp * t1;
    V3<T> diff = n22 - n22m;
    T magDiff = norm(diff);

    V3<T> tmpVec1 = T(0.5) * diff;
    V3<T> tmpVec2 = hCotanThetac * magDiff * t1;
    V3<T> n21m = n21 + tmpVec1 + tmpVec2;
    n22m = n22m + tmpVec1 - tmpVec2;

    V3<T> R = n21m - n11;
    T Rdt1 = dot(R, t1);

    V3<T> nd = R - Rdt1 * t1;
    T ndb1 = dot(nd, b1);
    (void)ndb1;
    T dSq = dot(nd, nd);
    T aSq_dSq = aSq + dSq;
    T aSq_dSqI = T(1) / aSq_dSq;

    T x1 = dot(n21m, t1);
    T x2 = dot(n22m, t1);
    T y1 = -dot(n11, t1);
    T y2 = -dot(n12, t1);

    T t1db2 = dot(t1, b2);
    T t1db1 = dot(t1, b1);
    T nddb1 = dot(nd, b1);

    V3<T> b2ct1 = cross(b2, t1);
    V3<T> b1ct1 = cross(b1, t1);
    V3<T> ndct1 = cross(nd, t1);

    T b2ct1db1 = dot(b2ct1, b1);
    T b2ct1dnd = dot(b2ct1, nd);

    V3<T> b2ct1ct1 = t1db2 * t1 - b2;

    T integ[12], tmpI[12];
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x1, y1, integ);
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x1, y2, tmpI);
    for (int k = 0; k < 12; ++k) integ[k] = integ[k] - tmpI[k];
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x2, y1, tmpI);
    for (int k = 0; k < 12; ++k) integ[k] = integ[k] - tmpI[k];
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x2, y2, tmpI);
    for (int k = 0; k < 12; ++k) integ[k] = integ[k] + tmpI[k];

    tmp = t1db1 * t1db2;
    V3<T> tv1 = tmp * nd;
    V3<T> tv2 = b2ct1dnd * b1ct1;
    V3<T> V1 = mu4pinu * (nddb1 * b2ct1ct1 + b2ct1db1 * ndct1 - tv2) - mu4pi * tv1;

    tmp = (mu4pinu - mu4pi) * t1db1;
    V3<T> V2 = tmp * b2ct1ct1;

    tmp = mu4pinu * b2ct1dnd * nddb1;
    V3<T> V3_ = -mu8piaSq * tv1 - mu4pinuaSq * tv2 - tmp * ndct1;

    tmp = mu8piaSq * t1db1;
    T tmp2 = mu4pinu * b2ct1dnd * t1db1;
    V3<T> V4 = -tmp * b2ct1ct1 - tmp2 * ndct1;

    T Fint1 = integ[2] - y1 * integ[0];
    T Fint2 = integ[5] - y1 * integ[3];
    T Fint3 = integ[8] - y1 * integ[6];
    T Fint4 = integ[11] - y1 * integ[9];
    Fnode2 = (V1 * Fint1 + V2 * Fint2 + V3_ * Fint3 + V4 * Fint4) * t1N;

    Fint1 = y2 * integ[0] - integ[2];
    Fint2 = y2 * integ[3] - integ[5];
    Fint3 = y2 * integ[6] - integ[8];
    Fint4 = y2 * integ[9] - integ[11];
    Fnode1 = (V1 * Fint1 + V2 * Fint2 + V3_ * Fint3 + V4 * Fint4) * t1N;

    T magDiffSq = dot(diff, diff);
    T magn21mSq = dot(n21m, n21m);
    T magn22mSq = dot(n22m, n22m);

    if (magDiffSq > T(kSqrtEps) * (magn21mSq + magn22mSq)) {
      V3<T> Fc[4];
      seg_seg_force(K, b2, n21, n21m, b1, n11, n12, Fc);
      Fnode1 = Fnode1 + Fc[2];
      Fnode2 = Fnode2 + Fc[3];
      seg_seg_force(K, b2, n22m, n22, b1, n11, n12, Fc);
      Fnode1 = Fnode1 + Fc[2];
      Fnode2 = Fnode2 + Fc[3];
    }
  }
  // ---- Segment 2 ----
  {
    T tmp = dot(n12 - n11, t2);
    V3<T> n12m = n11 + tmp * t2;
    V3<T> diff = n12 - n12m;
    T magDiff = norm(diff);

    V3<T> tmpVec1 = T(0.5) * diff;
    V3<T> tmpVec2 = hCotanThetac * magDiff * t2;
    V3<T> n11m = n11 + tmpVec1 + tmpVec2;
    n12m = n12m + tmpVec1 - tmpVec2;

    V3<T> R = n21 - n11m;
    T Rdt2 = dot(R, t2);

    V3<T> nd = R - Rdt2 * t2;
    T dSq = dot(nd, nd);
    T aSq_dSq = aSq + dSq;
    T aSq_dSqI = T(1) / aSq_dSq;

    T x1 = dot(n21, t2);
    T x2 = dot(n22, t2);
    T y1 = -dot(n11m, t2);
    T y2 = -dot(n12m, t2);

    T t2db2 = dot(t2, b2);
    T t2db1 = dot(t2, b1);
    T nddb2 = dot(nd, b2);

    V3<T> b2ct2 = cross(b2, t2);
    V3<T> b1ct2 = cross(b1, t2);
    V3<T> ndct2 = cross(nd, t2);

    T b1ct2db2 = dot(b1ct2, b2);
    T b1ct2dnd = dot(b1ct2, nd);

    V3<T> b1ct2ct2 = t2db1 * t2 - b1;

    T integ[12], tmpI[12];
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x1, y1, integ);
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x1, y2, tmpI);
    for (int k = 0; k < 12; ++k) integ[k] = integ[k] - tmpI[k];
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x2, y1, tmpI);
    for (int k = 0; k < 12; ++k) integ[k] = integ[k] - tmpI[k];
    par_seg_seg_integ(aSq_dSq, aSq_dSqI, x2, y2, tmpI);
    for (int k = 0; k < 12; ++k) integ[k] = integ[k] + tmpI[k];

    tmp = t2db2 * t2db1;
    V3<T> tv1 = tmp * nd;
    V3<T> tv2 = b1ct2dnd * b2ct2;
    V3<T> V1 = mu4pinu * (nddb2 * b1ct2ct2 + b1ct2db2 * ndct2 - tv2) - mu4pi * tv1;

    tmp = (mu4pinu - mu4pi) * t2db2;
    V3<T> V2 = tmp * b1ct2ct2;

    tmp = mu4pinu * b1ct2dnd * nddb2;
    V3<T> V3_ = -mu8piaSq * tv1 - mu4pinuaSq * tv2 - tmp * ndct2;

    tmp = mu8piaSq * t2db2;
    T tmp2 = mu4pinu * b1ct2dnd * t2db2;
    V3<T> V4 = -tmp * b1ct2ct2 - tmp2 * ndct2;

    T Fint1 = integ[1] - x1 * integ[0];
    T Fint2 = integ[4] - x1 * integ[3];
    T Fint3 = integ[7] - x1 * integ[6];
    T Fint4 = integ[10] - x1 * integ[9];
    Fnode4 = (V1 * Fint1 + V2 * Fint2 + V3_ * Fint3 + V4 * Fint4) * t2N;

    Fint1 = x2 * integ[0] - integ[1];
    Fint2 = x2 * integ[3] - integ[4];
    Fint3 = x2 * integ[6] - integ[7];
    Fint4 = x2 * integ[9] - integ[10];
    Fnode3 = (V1 * Fint1 + V2 * Fint2 + V3_ * Fint3 + V4 * Fint4) * t2N;

    T magDiffSq = magDiff * magDiff;
    T magn11mSq = dot(n11m, n11m);
    T magn12mSq = dot(n12m, n12m);

    if (magDiffSq > T(kSqrtEps) * (magn11mSq + magn12mSq)) {
      V3<T> Fc[4];
      seg_seg_force(K, b1, n11, n11m, b2, n21, n22, Fc);
      Fnode3 = Fnode3 + Fc[2];
      Fnode4 = Fnode4 + Fc[3];
      seg_seg_force(K, b1, n12m, n12, b2, n21, n22, Fc);
      Fnode3 = Fnode3 + Fc[2];
      Fnode4 = Fnode4 + Fc[3];
    }
  }
  if (flip) {
    V3<T> tmpF = Fnode1;
    Fnode1 = Fnode2;
    Fnode2 = tmpF;
  }
  F[0] = Fnode1;
  F[1] = Fnode2;
  F[2] = Fnode3;
  F[3] = Fnode4;
}

// ---------------------------------------------------------------------------
// Self force of one segment — _calcSelfForce (DislocationForces.jl:414-455):
// the force on node 2 (node 1 gets its negative).  tVec = n2 - n1 (not
// normalised), b the Burgers vector.  Constants: a = coreRad, aSq = coreRad²,
// μ4π, νomνInv = ν/(1-ν), omνInv = 1/(1-ν) (MaterialConstructor.jl:73-82),
// Ec = coreEnergy.
template <class T> struct SelfConsts {
  T a, aSq, mu4pi, nuOmNuInv, omNuInv, Ec;
};

template <class T>
inline V3<T> self_force_node2(const SelfConsts<T>& K, const V3<T>& tVec, const V3<T>& b) {
  using std::log;
  using std::sqrt;
  const T tVecSq = dot(tVec, tVec);
  const T L = sqrt(tVecSq);
  const T Linv = T(1) / L;
  const V3<T> t = tVec * Linv;  // tVecI *= Linv
  const T La = sqrt(tVecSq + K.aSq);
  const T bScrew = dot(t, b);
  const V3<T> bEdge = b - bScrew * t;
  const T bEdgeSq = dot(bEdge, bEdge);
  const T LaMa = La - K.a;
  const T tor = K.mu4pi * bScrew *
                (K.nuOmNuInv * (log((La + L) / K.a) - T(2) * LaMa * Linv) - LaMa * LaMa / (T(2) * La * L));
  const T torCore = T(2) * K.Ec * K.nuOmNuInv * bScrew;
  const T torTot = tor + torCore;
  const T lonCore = (bScrew * bScrew + bEdgeSq * K.omNuInv) * K.Ec;
  return torTot * bEdge - lonCore * t;
}

// PK force of one segment — _calcPKForce (DislocationForces.jl:292-300) for a
// given stress at the midpoint: (σ̂ b) × t, t = n2 - n1 (not normalised),
// sig = (xx, yy, zz, xy, xz, yz).
template <class T> inline V3<T> pk_force(const T* sig, const V3<T>& b, const V3<T>& t) {
  const V3<T> sb = {sig[0] * b.x + sig[3] * b.y + sig[4] * b.z, sig[3] * b.x + sig[1] * b.y + sig[5] * b.z,
                    sig[4] * b.x + sig[5] * b.y + sig[2] * b.z};
  return cross(sb, t);
}

// ---------------------------------------------------------------------------
// BCC mobility of one node — the loop body of dlnMobility
// (DislocationMobility.jl:16-178, the ! form :186-341 is the same per node).
// links: 2 × nLinks (1-based nodes), conn: ldConn × nodes (1-based links and
// columns, _makeConnect! layout), segForce: 3 × 2 × nLinks.  node1 is 0-based.
// Outer products follow ⊗(x, y) = x y' (Misc.jl:215) with the scalar applied to
// the left vector first, as Julia's left-to-right `s * t ⊗ t` does.  The
// velocity solves totalDrag v = f by Cramer's rule (det and adjugate).
struct MobParams {
  double sigmaPN, edge, screw, climb, line;
};

template <class T> struct M33 {
  T a[3][3];
};

template <class T> inline void add_outer(M33<T>& M, T s, const V3<T>& x, const V3<T>& y, T scale, T diag) {
  // M += scale * (diag I + (s x) y')
  const T sx[3] = {s * x.x, s * x.y, s * x.z};
  const T yy[3] = {y.x, y.y, y.z};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M.a[i][j] = M.a[i][j] + scale * ((i == j ? diag : T(0)) + sx[i] * yy[j]);
}

template <class T> inline V3<T> solve3(const M33<T>& M, const V3<T>& f) {
  const T(&a)[3][3] = M.a;
  const T c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  const T c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
  const T c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  const T det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
  const T x0 = (c00 * f.x + (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * f.y + (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * f.z) / det;
  const T x1 = (c01 * f.x + (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * f.y + (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * f.z) / det;
  const T x2 = (c02 * f.x + (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * f.y + (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * f.z) / det;
  return {x0, x1, x2};
}

template <class T>
inline void mobility_bcc_node(const MobParams& P, const T* coord, const T* bVec, const int64_t* links,
                              const int64_t* conn, int64_t ldConn, const T* segForce, int64_t node1, V3<T>& force,
                              V3<T>& vel) {
  using std::abs;
  using std::sqrt;
  const T eps = std::numeric_limits<T>::epsilon();
  const T sqrtBType = sqrt(eps);
  M33<T> drag = {};
  force = {T(0), T(0), T(0)};
  const int64_t numConnect = conn[ldConn * node1];
  const V3<T> x1 = {coord[3 * node1], coord[3 * node1 + 1], coord[3 * node1 + 2]};
  for (int64_t c = 1; c <= numConnect; ++c) {
    const int64_t link = conn[ldConn * node1 + 2 * c - 1] - 1;
    const int64_t colLink = conn[ldConn * node1 + 2 * c];
    const int64_t node2 = links[2 * link + (3 - colLink) - 1] - 1;
    V3<T> t = V3<T>{coord[3 * node2], coord[3 * node2 + 1], coord[3 * node2 + 2]} - x1;
    const T nT = sqrt(dot(t, t));
    if (nT < eps) continue;
    const T tN = T(1) / nT;
    t = t * tN;
    V3<T> f = {segForce[6 * link + 3 * (colLink - 1)], segForce[6 * link + 3 * (colLink - 1) + 1],
               segForce[6 * link + 3 * (colLink - 1) + 2]};
    if (sqrt(dot(f, f)) * tN < T(P.sigmaPN)) f = {T(0), T(0), T(0)};
    force = force + f;
    V3<T> b = {bVec[3 * link], bVec[3 * link + 1], bVec[3 * link + 2]};
    const T nB = sqrt(dot(b, b));
    const T ab[3] = {abs(b.x), abs(b.y), abs(b.z)};
    const T mn = std::min(std::min(ab[0], ab[1]), ab[2]);
    int type1 = 0, type2 = 0, type3 = 0;
    for (int k = 0; k < 3; ++k) {
      const T r = ab[k] / mn;
      type1 += abs(T(1) - r) < sqrtBType;
      type2 += abs(T(2) - r) < sqrtBType;
      type3 += abs(T(3) - r) < sqrtBType;
    }
    const bool screw = T(1) - nB < sqrtBType;
    b = {b.x / nB, b.y / nB, b.z / nB};
    const T nBnT_2 = nB * nT / T(2);
    if (!((type1 == 3 && screw) || (type1 == 2 && type2 == 1 && screw) ||
          (type1 == 1 && type2 == 1 && type3 == 1 && screw))) {
      add_outer(drag, T(P.line) - T(P.climb), t, t, nBnT_2, T(P.climb));
      continue;
    }
    const T tDb = dot(t, b);
    const T cosSq = tDb * tDb;
    const T sinSq = T(1) - cosSq;
    add_outer(drag, T(P.line) - T(P.screw), t, t, nBnT_2, T(P.screw));
    if (sinSq < eps) continue;
    const T sq = sqrt(sinSq);
    const V3<T> bt = cross(b, t);
    const V3<T> p = {bt.x / sq, bt.y / sq, bt.z / sq};
    const V3<T> q = cross(p, t);
    const T screwSq = T(P.screw) * T(P.screw);
    const T glide = T(1) / sqrt(sinSq / (T(P.edge) * T(P.edge)) + cosSq / screwSq);
    const T climb = sqrt(sinSq * (T(P.climb) * T(P.climb)) + cosSq * screwSq);
    // totalDrag += nBnT_2 * ((glide - ξs) q ⊗ q + (climb - ξs) p ⊗ p)
    const T gq[3] = {(glide - T(P.screw)) * q.x, (glide - T(P.screw)) * q.y, (glide - T(P.screw)) * q.z};
    const T cp[3] = {(climb - T(P.screw)) * p.x, (climb - T(P.screw)) * p.y, (climb - T(P.screw)) * p.z};
    const T qq[3] = {q.x, q.y, q.z}, pp[3] = {p.x, p.y, p.z};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) drag.a[i][j] = drag.a[i][j] + nBnT_2 * (gq[i] * qq[j] + cp[i] * pp[j]);
  }
  vel = solve3(drag, force);
}

// ---------------------------------------------------------------------------
// Field-point stress of one segment at one point — body of the point loop of
// _calc_σTilde! (DislocationFEM.jl:135-299).  Adds to sig[0..5] in the order
// (xx, yy, zz, xy, xz, yz).  t is normalize(n2 - n1) computed once per segment
// (DislocationFEM.jl:133).  StaticArrays' normalize is inv(norm(v)) * v.
template <class T> inline V3<T> normalize(const V3<T>& v) {
  T inv = T(1) / norm(v);
  return inv * v;
}

template <class T>
inline void sigma_tilde_point(const Consts<T>& K, const V3<T>& b, const V3<T>& n1, const V3<T>& n2, const V3<T>& t,
                              const V3<T>& x, T* sig) {
  using std::sqrt;
  const T mu4pi = K.mu4pi, mu4pinu = K.mu4pinu, nuMu4pinu = K.nuMu4pinu, a2 = K.aSq;
  const T a2mu8pi = a2 * K.mu8pi;

  V3<T> R = x - n1;
  T Rdt = dot(R, t);
  V3<T> nd = R - Rdt * t;
  T d2 = dot(nd, nd);

  T s1 = -Rdt;
  T s2 = -dot(x - n2, t);
  T a2_d2 = a2 + d2;
  T a2d2inv = T(1) / a2_d2;

  T Ra = sqrt(a2_d2 + s1 * s1);
  T Rainv = T(1) / Ra;
  T Ra3inv = Rainv * Rainv * Rainv;
  T sRa3inv = s1 * Ra3inv;

  T s_03a = s1 * Rainv * a2d2inv;
  T s_13a = -Rainv;
  T s_05a = (T(2) * s_03a + sRa3inv) * a2d2inv;
  T s_15a = -Ra3inv;
  T s_25a = s_03a - sRa3inv;

  Ra = sqrt(a2_d2 + s2 * s2);
  Rainv = T(1) / Ra;
  Ra3inv = Rainv * Rainv * Rainv;
  sRa3inv = s2 * Ra3inv;

  T s_03b = s2 * Rainv * a2d2inv;
  T s_13b = -Rainv;
  T s_05b = (T(2) * s_03b + sRa3inv) * a2d2inv;
  T s_15b = -Ra3inv;
  T s_25b = s_03b - sRa3inv;

  T s_03 = s_03b - s_03a;
  T s_13 = s_13b - s_13a;
  T s_05 = s_05b - s_05a;
  T s_15 = s_15b - s_15a;
  T s_25 = s_25b - s_25a;

  V3<T> txb = cross(t, b);
  V3<T> dxb = cross(nd, b);

  T dxbdt = dot(dxb, t);

  T dmdxx = nd.x * nd.x;
  T dmdyy = nd.y * nd.y;
  T dmdzz = nd.z * nd.z;
  T dmdxy = nd.x * nd.y;
  T dmdyz = nd.y * nd.z;
  T dmdxz = nd.x * nd.z;

  T tmtxx = t.x * t.x;
  T tmtyy = t.y * t.y;
  T tmtzz = t.z * t.z;
  T tmtxy = t.x * t.y;
  T tmtyz = t.y * t.z;
  T tmtxz = t.x * t.z;

  T tmdxx = T(2) * t.x * nd.x;
  T tmdyy = T(2) * t.y * nd.y;
  T tmdzz = T(2) * t.z * nd.z;
  T tmdxy = t.x * nd.y + t.y * nd.x;
  T tmdyz = t.y * nd.z + t.z * nd.y;
  T tmdxz = t.x * nd.z + t.z * nd.x;

  T tmtxbxx = T(2) * t.x * txb.x;
  T tmtxbyy = T(2) * t.y * txb.y;
  T tmtxbzz = T(2) * t.z * txb.z;
  T tmtxbxy = t.x * txb.y + t.y * txb.x;
  T tmtxbyz = t.y * txb.z + t.z * txb.y;
  T tmtxbxz = t.x * txb.z + t.z * txb.x;

  T dmtxbxx = T(2) * nd.x * txb.x;
  T dmtxbyy = T(2) * nd.y * txb.y;
  T dmtxbzz = T(2) * nd.z * txb.z;
  T dmtxbxy = nd.x * txb.y + nd.y * txb.x;
  T dmtxbyz = nd.y * txb.z + nd.z * txb.y;
  T dmtxbxz = nd.x * txb.z + nd.z * txb.x;

  T tmdxbxx = T(2) * t.x * dxb.x;
  T tmdxbyy = T(2) * t.y * dxb.y;
  T tmdxbzz = T(2) * t.z * dxb.z;
  T tmdxbxy = t.x * dxb.y + t.y * dxb.x;
  T tmdxbyz = t.y * dxb.z + t.z * dxb.y;
  T tmdxbxz = t.x * dxb.z + t.z * dxb.x;

  T common = mu4pinu * dxbdt;

  T I_03xx = common + mu4pinu * dmtxbxx - mu4pi * tmdxbxx;
  T I_03yy = common + mu4pinu * dmtxbyy - mu4pi * tmdxbyy;
  T I_03zz = common + mu4pinu * dmtxbzz - mu4pi * tmdxbzz;
  T I_03xy = mu4pinu * dmtxbxy - mu4pi * tmdxbxy;
  T I_03yz = mu4pinu * dmtxbyz - mu4pi * tmdxbyz;
  T I_03xz = mu4pinu * dmtxbxz - mu4pi * tmdxbxz;

  T I_13xx = -nuMu4pinu * tmtxbxx;
  T I_13yy = -nuMu4pinu * tmtxbyy;
  T I_13zz = -nuMu4pinu * tmtxbzz;
  T I_13xy = -nuMu4pinu * tmtxbxy;
  T I_13yz = -nuMu4pinu * tmtxbyz;
  T I_13xz = -nuMu4pinu * tmtxbxz;

  T I_05xx = common * (a2 + dmdxx) - a2mu8pi * tmdxbxx;
  T I_05yy = common * (a2 + dmdyy) - a2mu8pi * tmdxbyy;
  T I_05zz = common * (a2 + dmdzz) - a2mu8pi * tmdxbzz;
  T I_05xy = common * dmdxy - a2mu8pi * tmdxbxy;
  T I_05yz = common * dmdyz - a2mu8pi * tmdxbyz;
  T I_05xz = common * dmdxz - a2mu8pi * tmdxbxz;

  T I_15xx = a2mu8pi * tmtxbxx - common * tmdxx;
  T I_15yy = a2mu8pi * tmtxbyy - common * tmdyy;
  T I_15zz = a2mu8pi * tmtxbzz - common * tmdzz;
  T I_15xy = a2mu8pi * tmtxbxy - common * tmdxy;
  T I_15yz = a2mu8pi * tmtxbyz - common * tmdyz;
  T I_15xz = a2mu8pi * tmtxbxz - common * tmdxz;

  T I_25xx = common * tmtxx;
  T I_25yy = common * tmtyy;
  T I_25zz = common * tmtzz;
  T I_25xy = common * tmtxy;
  T I_25yz = common * tmtyz;
  T I_25xz = common * tmtxz;

  sig[0] = sig[0] + (I_03xx * s_03 + I_13xx * s_13 + I_05xx * s_05 + I_15xx * s_15 + I_25xx * s_25);
  sig[1] = sig[1] + (I_03yy * s_03 + I_13yy * s_13 + I_05yy * s_05 + I_15yy * s_15 + I_25yy * s_25);
  sig[2] = sig[2] + (I_03zz * s_03 + I_13zz * s_13 + I_05zz * s_05 + I_15zz * s_15 + I_25zz * s_25);
  sig[3] = sig[3] + (I_03xy * s_03 + I_13xy * s_13 + I_05xy * s_05 + I_15xy * s_15 + I_25xy * s_25);
  sig[4] = sig[4] + (I_03xz * s_03 + I_13xz * s_13 + I_05xz * s_05 + I_15xz * s_15 + I_25xz * s_25);
  sig[5] = sig[5] + (I_03yz * s_03 + I_13yz * s_13 + I_05yz * s_05 + I_15yz * s_15 + I_25yz * s_25);
}

// ---------------------------------------------------------------------------
// minimumDistance (Misc.jl:314-367): closest points of x0→x1 and y0→y1 as
// fractions L1, L2 along each, the squared distance there and its rate of
// change from the node velocities.  Kept as the reference writes it, including
// the near-parallel branch's L1 = floor(idx / 2), which gives (L1, L2) = (1, 1)
// for the second candidate (y1 - x0) — MiscTest.jl:135-140 holds that result.
template <class T> struct MinDist {
  T distSq, dDistSqDt, L1, L2;
};

template <class T> inline T clamp01(T x) { return x > T(1) ? T(1) : (x < T(0) ? T(0) : x); }

template <class T>
inline MinDist<T> minimum_distance(const V3<T>& x0, const V3<T>& x1, const V3<T>& y0, const V3<T>& y1,
                                   const V3<T>& vx0, const V3<T>& vx1, const V3<T>& vy0, const V3<T>& vy1) {
  using std::abs;
  const T eps = std::numeric_limits<T>::epsilon();
  const V3<T> seg1 = x1 - x0, seg2 = y1 - y0, vseg1 = vx1 - vx0, vseg2 = vy1 - vy0;
  const T A = dot(seg1, seg1);
  const T B = dot(T(2) * seg1, x0 - y0);
  const T C = dot(T(2) * seg1, seg2);
  const T D = dot(T(2) * seg2, y0 - x0);
  const T E = dot(seg2, seg2);
  const T G = C * C - T(4) * A * E;
  T L1, L2;
  if (A < eps) {
    L1 = T(0);
    L2 = E < eps ? T(0) : -D / E / T(2);
  } else if (E < eps) {
    L2 = T(0);
    L1 = -B / A / T(2);
  } else if (abs(G) < eps) {
    const T d[4] = {dot(y0 - x0, y0 - x0), dot(y1 - x0, y1 - x0), dot(y0 - x1, y0 - x1), dot(y1 - x1, y1 - x1)};
    int idx = 1;  // findmin: the first minimum (a NaN counts as the smallest)
    for (int k = 1; k < 4 && !std::isnan(d[idx - 1]); ++k)
      if (std::isnan(d[k]) || d[k] < d[idx - 1]) idx = k + 1;
    L1 = std::floor(T(idx) / T(2));
    L2 = T((idx - 1) % 2);
  } else {
    L2 = (T(2) * A * D + B * C) / G;
    L1 = (C * L2 - B) / A / T(2);
  }
  L1 = clamp01(L1);
  L2 = clamp01(L2);
  const V3<T> P = x0 + seg1 * L1 - y0 - seg2 * L2;
  const V3<T> V = vx0 + vseg1 * L1 - vy0 - vseg2 * L2;
  return {dot(P, P), T(2) * dot(V, P), L1, L2};
}

// detectCollision (DislocationTopologyCollision.jl:1-221).  type: 0 :null,
// 1 :hinge, 2 :twoLine.  Indices are 1-based (0 when there is no collision).
// L1, L2 are what the reference returns: the variables its loops overwrite on
// every minimumDistance call, i.e. those of the LAST pair it evaluated (in the
// twoLine pass if that pass ran and evaluated a pair, else in the hinge pass),
// not necessarily those of the reported pair; pairDistSq, pairL1, pairL2
// belong to the reported pair.
struct Collision {
  int32_t collision, type;
  int64_t n1s1, n2s1, n1s2, n2s2, s1, s2;
  double L1, L2, pairDistSq, pairL1, pairL2;
};

inline bool mobile_label(int32_t l) { return l == 1 || l == 3; }  // intMobDln, srfMobDln

// The reference scans skipSegs linearly for (a, b) in either order; the same
// test as a lookup in the canonical (min, max) pairs, sorted.
struct SkipSet {
  std::vector<std::pair<int64_t, int64_t>> v;
  SkipSet(const int64_t* skip, int64_t nSkip) {
    for (int64_t q = 0; q < nSkip; ++q)
      v.push_back({std::min(skip[2 * q], skip[2 * q + 1]), std::max(skip[2 * q], skip[2 * q + 1])});
    std::sort(v.begin(), v.end());
  }
  bool operator()(int64_t a, int64_t b) const {
    return !v.empty() && std::binary_search(v.begin(), v.end(), std::make_pair(std::min(a, b), std::max(a, b)));
  }
};

template <class T>
Collision detect_collision(T collisionDistSq, const T* coord, const T* nodeVel, const int32_t* label,
                           const int64_t* links, const T* bVec, const int64_t* conn, int64_t ldConn, int64_t numNode,
                           int64_t numSeg, const int64_t* skip, int64_t nSkip) {
  const T eps = std::numeric_limits<T>::epsilon();
  const SkipSet skipped(skip, nSkip);
  Collision r{};
  T smallest = T(0);
  T L1 = T(0), L2 = T(0);
  auto X = [&](int64_t n) { return V3<T>{coord[3 * n], coord[3 * n + 1], coord[3 * n + 2]}; };
  auto Vn = [&](int64_t n) { return V3<T>{nodeVel[3 * n], nodeVel[3 * n + 1], nodeVel[3 * n + 2]}; };
  // findConnectedNode (DislocationTopology.jl:22-32): (link, other node), 1-based.
  auto connected = [&](int64_t i, int64_t c, int64_t& link, int64_t& node) {
    link = conn[ldConn * i + 2 * c - 1];
    const int64_t col = conn[ldConn * i + 2 * c];
    node = links[2 * (link - 1) + (3 - col) - 1];
  };
  // Hinges: pairs of links at one mobile node.  link1 / node1 / tN1 persist
  // across the k loop, swapped whenever connection k is longer (the reference
  // assigns its j-loop variables inside the k loop).
  for (int64_t i = 0; i < numNode; ++i) {
    if (!mobile_label(label[i])) continue;
    const int64_t nc = conn[ldConn * i];
    for (int64_t j = 1; j <= nc; ++j) {
      int64_t link1, node1;
      connected(i, j, link1, node1);
      V3<T> t = X(i) - X(node1 - 1);
      T tN1 = dot(t, t);
      for (int64_t k = j + 1; k <= nc; ++k) {
        int64_t link2, node2;
        connected(i, k, link2, node2);
        t = X(i) - X(node2 - 1);
        T tN2 = dot(t, t);
        if (tN1 < tN2) {
          std::swap(link1, link2);
          std::swap(node1, node2);
          std::swap(tN1, tN2);
        }
        if (skipped(link1, link2)) continue;
        const V3<T> y0 = X(node2 - 1), vy0 = Vn(node2 - 1);
        const MinDist<T> m = minimum_distance(X(i), X(node1 - 1), y0, y0, Vn(i), Vn(node1 - 1), vy0, vy0);
        L1 = m.L1;
        L2 = m.L2;
        if (m.distSq < collisionDistSq && m.dDistSqDt < -eps) {
          const T inv = T(1) / m.distSq;
          if (inv > smallest) {
            smallest = inv;
            r = {1, 1, i + 1, node1, node2, node2, link1, link2, 0, 0, (double)m.distSq, (double)m.L1,
                 (double)m.L2};
          }
        }
      }
    }
  }
  if (r.collision) {
    r.L1 = L1;
    r.L2 = L2;
    return r;
  }
  // Two lines: unconnected pairs of segments with all four nodes mobile.
  for (int64_t i = 0; i < numSeg; ++i) {
    const int64_t a1 = links[2 * i], a2 = links[2 * i + 1];
    if (!mobile_label(label[a1 - 1]) || !mobile_label(label[a2 - 1])) continue;
    const V3<T> x0 = X(a1 - 1), x1 = X(a2 - 1), vx0 = Vn(a1 - 1), vx1 = Vn(a2 - 1);
    const V3<T> bi = {bVec[3 * i], bVec[3 * i + 1], bVec[3 * i + 2]};
    for (int64_t j = i + 1; j < numSeg; ++j) {
      const int64_t c1 = links[2 * j], c2 = links[2 * j + 1];
      if (a1 == c1 || a1 == c2 || a2 == c1 || a2 == c2) continue;
      if (!mobile_label(label[c1 - 1]) || !mobile_label(label[c2 - 1])) continue;
      const V3<T> y0 = X(c1 - 1), y1 = X(c2 - 1);
      const V3<T> bj = {bVec[3 * j], bVec[3 * j + 1], bVec[3 * j + 2]};
      const V3<T> bm = bi - bj, bp = bi + bj;
      const T tt = dot(x1 - x0, y1 - y0);
      if ((dot(bm, bm) < eps && tt > eps) || (dot(bp, bp) < eps && tt < eps)) continue;  // superdislocations
      if (skipped(i + 1, j + 1)) continue;
      const MinDist<T> m = minimum_distance(x0, x1, y0, y1, vx0, vx1, Vn(c1 - 1), Vn(c2 - 1));
      L1 = m.L1;
      L2 = m.L2;
      if (m.distSq < collisionDistSq && m.dDistSqDt < -eps) {
        const T inv = T(1) / m.distSq;
        if (inv > smallest) {
          smallest = inv;
          r = {1, 2, a1, a2, c1, c2, i + 1, j + 1, 0, 0, (double)m.distSq, (double)m.L1, (double)m.L2};
        }
      }
    }
  }
  r.L1 = L1;
  r.L2 = L2;
  return r;
}

// ---------------------------------------------------------------------------
// calc_uTilde (DislocationFEM.jl:355-581): displacements at FE nodes from
// Barnett triangles (Bromage & Tarleton 2018) closing each segment on a point.

// safeNorm (Misc.jl:289-300): returns |x| and normalises x, or eps and zero.
template <class T> inline T safe_norm(V3<T>& x) {
  const T eps = std::numeric_limits<T>::epsilon();
  T n = norm(x);
  if (n > eps) {
    x = normalize(x);
  } else {
    x = {T(0), T(0), T(0)};
    n = eps;
  }
  return n;
}
// π as the reference's Float64 arithmetic uses it, and to full precision for
// the long double evaluation.
template <class T> inline T pi_of() { return T(3.141592653589793); }
template <> inline long double pi_of<long double>() { return 3.141592653589793238462643383279502884L; }
template <class T> inline T jl_sign(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : x); }
// Julia's max(x, 0): -0.0 and negatives give +0.0, NaN stays.
template <class T> inline T jl_max0(T x) { return std::isnan(x) ? x : ((x < T(0) || std::signbit(x)) ? T(0) : x); }
template <class T> inline T clamp11(T x) { return x > T(1) ? T(1) : (x < T(-1) ? T(-1) : x); }

// One triangle ABC with Burgers vector b; full = the form with matParams
// (solid angle, f and g terms, DislocationFEM.jl:600-660), else the solid-angle
// form (:661-707).  AB, BC, CA are the safeNorm'ed edge directions.
template <class T> struct UTri {
  V3<T> A, B, C, b, AB, BC, CA;
  bool full;
};

template <class T> inline UTri<T> make_tri(const V3<T>& A, const V3<T>& B, const V3<T>& C, const V3<T>& b, bool full) {
  UTri<T> t{A, B, C, b, B - A, C - B, A - C, full};
  safe_norm(t.AB);
  safe_norm(t.BC);
  safe_norm(t.CA);
  return t;
}

template <class T> inline V3<T> tri_u(const UTri<T>& t, T omNuInv8pi, T om2NuOmNuInv8pi, const V3<T>& P) {
  using std::acos;
  using std::atan;
  using std::log;
  using std::sqrt;
  using std::tan;
  const T fourPi = T(4) * pi_of<T>();
  V3<T> RA = t.A - P, RB = t.B - P, RC = t.C - P;
  const T RAn = safe_norm(RA), RBn = safe_norm(RB), RCn = safe_norm(RC);
  const T RAdRB = clamp11(dot(RA, RB)), RBdRC = clamp11(dot(RB, RC)), RCdRA = clamp11(dot(RC, RA));
  const T ta = acos(RAdRB), tb = acos(RBdRC), tc = acos(RCdRA);
  const T th = (ta + tb + tc) / T(2);
  const T factor = jl_max0(tan(th / T(2)) * tan((th - ta) / T(2)) * tan((th - tb) / T(2)) * tan((th - tc) / T(2)));
  T omega = T(4) * atan(sqrt(factor));
  omega = -jl_sign(dot(RA, cross(t.CA, t.AB))) * omega;
  const V3<T> nb = -t.b;
  V3<T> u = {nb.x * omega / fourPi, nb.y * omega / fourPi, nb.z * omega / fourPi};
  if (!t.full) return u;
  const V3<T> fAB = cross(t.b, t.AB) * log((RBn / RAn) * (T(1) + dot(RB, t.AB)) / (T(1) + dot(RA, t.AB)));
  const V3<T> fBC = cross(t.b, t.BC) * log((RCn / RBn) * (T(1) + dot(RC, t.BC)) / (T(1) + dot(RB, t.BC)));
  const V3<T> fCA = cross(t.b, t.CA) * log((RAn / RCn) * (T(1) + dot(RA, t.CA)) / (T(1) + dot(RC, t.CA)));
  auto g = [](T s, const V3<T>& v, T den) { return V3<T>{s * v.x / den, s * v.y / den, s * v.z / den}; };
  const V3<T> gAB = g(dot(t.b, cross(RA, RB)), RA + RB, T(1) + RAdRB);
  const V3<T> gBC = g(dot(t.b, cross(RB, RC)), RB + RC, T(1) + RBdRC);
  const V3<T> gCA = g(dot(t.b, cross(RC, RA)), RC + RA, T(1) + RCdRA);
  return u - om2NuOmNuInv8pi * (fAB + fBC + fCA) + omNuInv8pi * (gAB + gBC + gCA);
}

// The mesh data calc_uTilde reads: face normals and midpoints (3 × nF), the
// projection directions (3 × nN), the volume as a box [lo, hi] for the "inside
// the mesh" test (LazySets' polytope membership in the reference, here an
// inclusive box test widened by tol), and the closure point C.
template <class T> struct UMesh {
  const T* faceNorm;
  const T* faceMidPt;
  int64_t nF;
  const T* normals;
  int64_t nN;
  V3<T> lo, hi, C;
  T tol;
};

template <class T> inline bool inside_mesh(const UMesh<T>& m, const V3<T>& p) {
  return p.x >= m.lo.x - m.tol && p.x <= m.hi.x + m.tol && p.y >= m.lo.y - m.tol && p.y <= m.hi.y + m.tol &&
         p.z >= m.lo.z - m.tol && p.z <= m.hi.z + m.tol;
}

// findIntersectVolume (DislocationTopologySpecial.jl:7-34) with
// linePlaneIntersect (Misc.jl:223-235): the smallest squared distance from l0
// to the intersection of the line (l0, l) with a face plane inside the mesh.
template <class T> inline T find_intersect_volume(const UMesh<T>& m, const V3<T>& l, const V3<T>& l0, V3<T>& node) {
  T distMin = std::numeric_limits<T>::infinity();
  node = {T(0), T(0), T(0)};
  for (int64_t i = 0; i < m.nF; ++i) {
    const V3<T> n = {m.faceNorm[3 * i], m.faceNorm[3 * i + 1], m.faceNorm[3 * i + 2]};
    const V3<T> p0 = {m.faceMidPt[3 * i], m.faceMidPt[3 * i + 1], m.faceMidPt[3 * i + 2]};
    const T den = dot(l, n);
    const T num = dot(p0 - l0, n);
    if (den == T(0)) continue;  // parallel: no point (or the Inf marker), skipped either way
    const T d = num / den;
    const V3<T> it = l0 + d * l;
    if (std::isinf(it.x) || std::isinf(it.y) || std::isinf(it.z) || !inside_mesh(m, it)) continue;
    const V3<T> dv = it - l0;
    const T oldMin = distMin;
    const T s = dv.x * dv.x + dv.y * dv.y + dv.z * dv.z;
    distMin = s < oldMin ? s : oldMin;
    if (distMin < oldMin) node = it;
  }
  return distMin;
}

// The triangles of _calc_uTilde! (DislocationFEM.jl:399-632) in the order the
// reference evaluates them: one full triangle (A, B, C) per internal segment;
// for a segment with an external node, five solid-angle triangles through the
// points A' and B' the nodes were projected out from and C' = (A + B') / 2.
// Segments joining a surface node to an external node only record that
// connection (and only for the segments after them, as the reference's loop
// builds the record as it goes).
template <class T>
std::vector<UTri<T>> u_tilde_triangles(const UMesh<T>& m, const T* coord, const int32_t* label, const int64_t* links,
                                       const T* bVec, int64_t numNode, int64_t numSeg) {
  auto srf = [](int32_t l) { return l == 3 || l == 4; };  // srfMobDln, srfFixDln
  const int32_t ext = 5;                                  // extDln
  std::vector<UTri<T>> tris;
  std::vector<int64_t> surfNodeCons((size_t)numNode, 0);
  auto X = [&](int64_t n) { return V3<T>{coord[3 * n], coord[3 * n + 1], coord[3 * n + 2]}; };
  for (int64_t i = 0; i < numSeg; ++i) {
    const int64_t l1 = links[2 * i], l2 = links[2 * i + 1];
    if (srf(label[l1 - 1]) && label[l2 - 1] == ext) {
      surfNodeCons[l2 - 1] = l1;
      continue;
    }
    if (srf(label[l2 - 1]) && label[l1 - 1] == ext) {
      surfNodeCons[l1 - 1] = l2;
      continue;
    }
    const V3<T> A = X(l1 - 1), B = X(l2 - 1);
    const V3<T> b = {bVec[3 * i], bVec[3 * i + 1], bVec[3 * i + 2]};
    if (label[l1 - 1] != ext && label[l2 - 1] != ext) {
      tris.push_back(make_tri(A, B, m.C, b, true));
      continue;
    }
    const T inf = std::numeric_limits<T>::infinity();
    T distMinA = inf, distMinB = inf, distMinC = inf;
    V3<T> intersectA = {inf, inf, inf}, intersectB = {inf, inf, inf};
    for (int64_t j = 0; j < m.nN; ++j) {
      const V3<T> l = {m.normals[3 * j], m.normals[3 * j + 1], m.normals[3 * j + 2]};
      V3<T> iA, iB;
      const T dA = find_intersect_volume(m, l, A, iA);
      const T dB = find_intersect_volume(m, l, B, iB);
      if (dA < distMinA) distMinA = dA, intersectA = iA;
      if (dB < distMinB) distMinB = dB, intersectB = iB;
    }
    // Out of an edge or a corner: walk the face planes towards the centre.
    // distMinC is shared by the two walks, as in the reference.
    auto walk = [&](V3<T> P) {
      for (int64_t f = 0; f < m.nF; ++f) {
        const V3<T> n = {m.faceNorm[3 * f], m.faceNorm[3 * f + 1], m.faceNorm[3 * f + 2]};
        const V3<T> mp = {m.faceMidPt[3 * f], m.faceMidPt[3 * f + 1], m.faceMidPt[3 * f + 2]};
        const T q = dot(P + mp, n);
        const T dist = q * q;
        const V3<T> it = P - n * std::sqrt(dist);
        const T dc = norm(it - m.C);
        if (dc <= distMinC) distMinC = dc, P = it;
      }
      return P;
    };
    if (std::isinf(distMinA)) intersectA = walk(A);
    if (std::isinf(distMinB)) intersectB = walk(B);
    V3<T> Ap = intersectA, Bp = intersectB;
    if (surfNodeCons[l1 - 1] != 0) Ap = X(surfNodeCons[l1 - 1] - 1);
    if (surfNodeCons[l2 - 1] != 0) Bp = X(surfNodeCons[l2 - 1] - 1);
    const V3<T> Cp = {(A.x + Bp.x) / T(2), (A.y + Bp.y) / T(2), (A.z + Bp.z) / T(2)};
    tris.push_back(make_tri(Ap, Bp, m.C, b, false));
    tris.push_back(make_tri(Ap, A, Cp, b, false));
    tris.push_back(make_tri(A, B, Cp, b, false));
    tris.push_back(make_tri(B, Bp, Cp, b, false));
    tris.push_back(make_tri(Bp, Ap, Cp, b, false));
  }
  return tris;
}

}  // namespace ddd_oracle
