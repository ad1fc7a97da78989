// calc_uTilde's field kernel, reformulated FP64 (compiled with --fmad=false):
// the same triangles, unit vectors and sums as u_tilde.cu's reference-order
// kernel, with
//   * log and atan on the integer pipes (intmath_f64.cuh);
//   * the solid angle's magnitude from one atan2 (Van Oosterom & Strackee
//     1983: tan(Ω/2) = R_A·(R_B×R_C) / (1 + R_A·R_B + R_B·R_C + R_C·R_A) for
//     unit R) instead of l'Huilier's three acos, four tan and one atan, its
//     sign from the reference's own expression -sign(R_A·(CA×AB));
//   * one division per log term and per g term;
//   * no f and g terms for an edge (B_i, C) shared by consecutive triangles of
//     a loop (same b, both closed on C): the two triangles' terms for that
//     edge cancel (the g terms exactly, the f terms up to rounding), so both
//     are left out, which removes rounding noise rather than adding any.
// Where the point lies (nearly) in the triangle's plane, |R_A·(R_B×R_C)| <=
// 1e-10, the solid angle is discontinuous and the reference's result is
// decided by its rounding; there the kernel evaluates the reference's
// l'Huilier expression on the same unit vectors, bit for bit as the
// reference-order kernel.  Elsewhere the atan2 form is better conditioned than
// l'Huilier's (acos of dot products near 1) and agrees with it to the
// reference arithmetic's own rounding level.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "intmath_f64.cuh"

namespace ddd {
namespace {

constexpr int PT = 128;

// atan2(y, x) for y > 0 on the integer pipes: the quotient rounded once, then
// im::atan (within ~1 ulp; CUDA documents 2 ulp for its atan2).
__device__ __forceinline__ double atan2_pos(double y, double x) {
  const double pi = 3.141592653589793;
  if (x > 0.0) return im::atan(y / x);
  if (x < 0.0) return pi - im::atan(y / -x);
  return 0.5 * pi;
}
constexpr int TCH = 32;
constexpr int TROW = kUTriRows;

struct V {
  double x, y, z;
};
__device__ __forceinline__ V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V operator*(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V cross(V a, V b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// safeNorm (Misc.jl:289-300), as the reference-order kernel: |x| (eps when
// below eps) and inv(|x|) * x (or zero).
__device__ __forceinline__ double unit(V& x) {
  const double n = sqrt(dot(x, x));
  if (n > DBL_EPSILON) {
    const double inv = 1.0 / n;
    x = {inv * x.x, inv * x.y, inv * x.z};
    return n;
  }
  x = {0.0, 0.0, 0.0};
  return DBL_EPSILON;
}
// Julia's max(x, 0): negatives and -0.0 give +0.0; NaN stays NaN.
__device__ __forceinline__ double jl_max0(double x) { return isnan(x) ? x : ((x < 0.0 || signbit(x)) ? 0.0 : x); }
__device__ __forceinline__ double clamp11(double x) { return x > 1.0 ? 1.0 : (x < -1.0 ? -1.0 : x); }
__device__ __forceinline__ double jl_sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : x); }

__global__ void __launch_bounds__(PT) u_field_fast(const double* __restrict__ tri, int64_t nTri, int64_t chunk,
                                                   const double* __restrict__ points, int64_t M, double k1, double k2,
                                                   V Cl, double* __restrict__ part) {
  __shared__ double sm[TCH][TROW + 1];
  const int64_t p = blockIdx.x * (int64_t)PT + threadIdx.x;
  const bool on = p < M;
  const V P = on ? V{points[3 * p], points[3 * p + 1], points[3 * p + 2]} : V{0.0, 0.0, 0.0};
  V RCc = Cl - P;
  const double RCcn = unit(RCc);
  V prevRB = {0.0, 0.0, 0.0};
  double prevRBn = 0.0;
  bool prevValid = false;
  V acc = {0.0, 0.0, 0.0};
  const int64_t tBeg = blockIdx.y * chunk, tEnd = tBeg + chunk < nTri ? tBeg + chunk : nTri;
  for (int64_t t0 = tBeg; t0 < tEnd; t0 += TCH) {
    const int n = (int)(tEnd - t0 < TCH ? tEnd - t0 : TCH);
    __syncthreads();
    for (int q = threadIdx.x; q < n * TROW; q += PT) {
      const int tt = q % n, k = q / n;
      sm[tt][k] = tri[k * nTri + t0 + tt];
    }
    __syncthreads();
    if (!on) continue;
    for (int tt = 0; tt < n; ++tt) {
      const double* s = sm[tt];
      const int link = (int)s[22];
      V RA, RB = V{s[3], s[4], s[5]} - P, RC;
      double RAn, RCn;
      if ((link & 2) && prevValid) {
        RA = prevRB;
        RAn = prevRBn;
      } else {
        RA = V{s[0], s[1], s[2]} - P;
        RAn = unit(RA);
      }
      const double RBn = unit(RB);
      if (link & 1) {
        RC = RCc;
        RCn = RCcn;
      } else {
        RC = V{s[6], s[7], s[8]} - P;
        RCn = unit(RC);
      }
      prevRB = RB;
      prevRBn = RBn;
      prevValid = true;
      const V AB = {s[12], s[13], s[14]}, BC = {s[15], s[16], s[17]}, CA = {s[18], s[19], s[20]};
      const double ab = dot(RA, RB), bc = dot(RB, RC), ca = dot(RC, RA);
      const double num = dot(RA, cross(RB, RC));
      const double sgn = -jl_sign(dot(RA, cross(CA, AB)));
      double om;
      if (fabs(num) > 1e-10) {
        om = sgn * (2.0 * atan2_pos(fabs(num), 1.0 + ab + bc + ca));
      } else {  // (nearly) in the triangle's plane: the reference's expression
        const double ta = acos(clamp11(ab)), tb = acos(clamp11(bc)), tc = acos(clamp11(ca));
        const double th = (ta + tb + tc) / 2.0;
        const double f =
            jl_max0(tan(th / 2.0) * tan((th - ta) / 2.0) * tan((th - tb) / 2.0) * tan((th - tc) / 2.0));
        om = sgn * (4.0 * im::atan(sqrt(f)));
      }
      const double fourPi = 4.0 * 3.141592653589793;
      acc = acc + V{-s[9] * om / fourPi, -s[10] * om / fourPi, -s[11] * om / fourPi};
      if (s[21] == 0.0) continue;
      const V b = {s[9], s[10], s[11]};
      const double lAB = im::log((RBn * (1.0 + dot(RB, AB))) / (RAn * (1.0 + dot(RA, AB))));
      V fs = V{s[23], s[24], s[25]} * lAB;
      V gs = (RA + RB) * (dot(b, cross(RA, RB)) / (1.0 + clamp11(ab)));
      if (!(link & 4)) {
        const double lBC = im::log((RCn * (1.0 + dot(RC, BC))) / (RBn * (1.0 + dot(RB, BC))));
        fs = fs + V{s[26], s[27], s[28]} * lBC;
        gs = gs + (RB + RC) * (dot(b, cross(RB, RC)) / (1.0 + clamp11(bc)));
      }
      if (!(link & 8)) {
        const double lCA = im::log((RAn * (1.0 + dot(RA, CA))) / (RCn * (1.0 + dot(RC, CA))));
        fs = fs + V{s[29], s[30], s[31]} * lCA;
        gs = gs + (RC + RA) * (dot(b, cross(RC, RA)) / (1.0 + clamp11(ca)));
      }
      acc = acc - fs * k2 + gs * k1;
    }
  }
  if (on) {
    double* u = part + 3 * (blockIdx.y * M + p);
    u[0] = acc.x;
    u[1] = acc.y;
    u[2] = acc.z;
  }
}

}  // namespace

int u_field_fast_blocks_per_sm() {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, u_field_fast, PT, 0) != cudaSuccess) return 1;
  return occ;
}

cudaError_t launch_u_field_fast(const double* tri, int64_t nTri, int64_t chunk, int64_t K, const double* points,
                                int64_t M, double omNuInv8pi, double om2NuOmNuInv8pi, const double C[3], double* part,
                                cudaStream_t st) {
  if (M <= 0) return cudaSuccess;
  u_field_fast<<<dim3((unsigned)((M + PT - 1) / PT), (unsigned)K), PT, 0, st>>>(
      tri, nTri, chunk, points, M, omNuInv8pi, om2NuOmNuInv8pi, V{C[0], C[1], C[2]}, part);
  return cudaGetLastError();
}

}  // namespace ddd
