// Host build of the fast FP64 form of the seg-seg force (DDD_MODE_FP64_FAST):
// ddd.jl_gb300/csrc/pair_f64fast.cuh compiled as plain C++ without contraction,
// so its general branch gives the GPU's values bit for bit (with the
// integer-pipe or table-driven logarithm and arctangent).  Pairs that take the near-parallel
// branch, which the GPU form evaluates in the reference's strict arithmetic,
// use the oracle's restatement here.  Test infrastructure only: it measures the
// form's accuracy against long double on a CPU; the product runs the header on
// the GPU.
#include <cstdint>
#include <vector>

#include "../../oracle/ddd_oracle.hpp"
#include "pair_f64fast.cuh"

namespace {

struct HostSeg {
  ddd::fx::X3 n1, n2, b, t;
  double tN;
};

}  // namespace

// All-pairs forces in calcSegSegForceSer!'s order (DislocationForces.jl:778-829):
// F (3 x 2 x numSeg, zeroed here) += the four node forces of every pair i < j,
// external segments skipped on both sides.  fmath 2: the integer-pipe log/atan,
// 1: the FP64 table-driven ones, 0: the C library's.
extern "C" void fast_segseg_ser(int fmath, const double* k5, const double* coord, const double* bVec,
                                const int64_t* segIdx, int64_t ld, const uint8_t* extSeg, int64_t numSeg,
                                double* F) {
  using ddd::fx::X3;
  ddd::fx::KFast K{k5[0], k5[1], k5[2], k5[3], k5[0] * k5[2], k5[0] * k5[3]};
  ddd_oracle::Consts<double> KO;
  KO.aSq = k5[0];
  KO.mu4pi = k5[1];
  KO.mu8pi = k5[2];
  KO.mu4pinu = k5[3];
  KO.nuMu4pinu = k5[4];
  KO.mu8piaSq = KO.aSq * KO.mu8pi;
  KO.mu4pinuaSq = KO.aSq * KO.mu4pinu;
  std::vector<HostSeg> s(numSeg);
  for (int64_t i = 0; i < numSeg; ++i) {
    const int64_t l = segIdx[i] - 1, a = segIdx[i + ld] - 1, b = segIdx[i + 2 * ld] - 1;
    HostSeg& q = s[i];
    q.n1 = {coord[3 * a], coord[3 * a + 1], coord[3 * a + 2]};
    q.n2 = {coord[3 * b], coord[3 * b + 1], coord[3 * b + 2]};
    q.b = {bVec[3 * l], bVec[3 * l + 1], bVec[3 * l + 2]};
    const X3 t = q.n2 - q.n1;
    q.tN = 1.0 / std::sqrt(t.x * t.x + t.y * t.y + t.z * t.z);
    q.t = t * q.tN;
  }
  for (int64_t k = 0; k < 6 * numSeg; ++k) F[k] = 0.0;
  auto add = [&](int64_t seg, int node, const X3& v) {
    double* d = F + 6 * seg + 3 * node;
    d[0] += v.x;
    d[1] += v.y;
    d[2] += v.z;
  };
  for (int64_t i = 0; i < numSeg; ++i) {
    if (extSeg[i]) continue;
    for (int64_t j = i + 1; j < numSeg; ++j) {
      if (extSeg[j]) continue;
      const HostSeg &a = s[i], &b = s[j];
      const double c = ddd::fx::dot(a.t, b.t);
      X3 F1, F2, F3, F4;
      if (1.0 - c * c > 1.4901161193847656e-08) {
        if (fmath == 2)
          ddd::fx::general_pair<true, true, ddd::fx::kMathInt>(K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t,
                                                               b.tN, c, F1, F2, F3, F4);
        else if (fmath == 1)
          ddd::fx::general_pair<true, true, ddd::fx::kMathTable>(K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t,
                                                                 b.tN, c, F1, F2, F3, F4);
        else
          ddd::fx::general_pair<true, true, ddd::fx::kMathCuda>(K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t,
                                                                b.tN, c, F1, F2, F3, F4);
      } else {
        ddd_oracle::V3<double> out[4];
        ddd_oracle::seg_seg_force<double>(KO, {a.b.x, a.b.y, a.b.z}, {a.n1.x, a.n1.y, a.n1.z}, {a.n2.x, a.n2.y, a.n2.z},
                                   {b.b.x, b.b.y, b.b.z}, {b.n1.x, b.n1.y, b.n1.z}, {b.n2.x, b.n2.y, b.n2.z}, out);
        F1 = {out[0].x, out[0].y, out[0].z};
        F2 = {out[1].x, out[1].y, out[1].z};
        F3 = {out[2].x, out[2].y, out[2].z};
        F4 = {out[3].x, out[3].y, out[3].z};
      }
      add(i, 0, F1);
      add(i, 1, F2);
      add(j, 0, F3);
      add(j, 1, F4);
    }
  }
}

// The logarithm and arctangent at n points: kind 2 the integer-pipe ones
// (intmath_f64.cuh), 1 the FP64 table-driven ones (fastmath_f64.cuh).
extern "C" void fast_log_atan(int kind, const double* x, int64_t n, double* lg, double* at) {
  for (int64_t i = 0; i < n; ++i) {
    lg[i] = kind == 2 ? ddd::im::log(x[i]) : ddd::fm::log(x[i]);
    at[i] = kind == 2 ? ddd::im::atan(x[i]) : ddd::fm::atan(x[i]);
  }
}

// σ̃ at M points (x0 3×M) by the fast form of sigma_fx.cuh: each point's sum
// over the segments in list order, as calc_σTilde.  sigma is 6×M.
#include "sigma_fx.cuh"
extern "C" void fast_sigma(const double* k5, const double* x0, int64_t M, const double* coord, const double* bVec,
                           const int64_t* segIdx, int64_t ld, int64_t numSeg, double* sigma) {
  using ddd::sx::X3;
  const ddd::sx::KS K{k5[0], k5[1], k5[3], k5[4], k5[0] * k5[2]};
  std::vector<ddd::sx::SegS> s(numSeg);
  for (int64_t i = 0; i < numSeg; ++i) {
    const int64_t l = segIdx[i] - 1, a = segIdx[i + ld] - 1, b = segIdx[i + 2 * ld] - 1;
    const X3 n1 = {coord[3 * a], coord[3 * a + 1], coord[3 * a + 2]};
    const X3 v = {coord[3 * b] - n1.x, coord[3 * b + 1] - n1.y, coord[3 * b + 2] - n1.z};
    const double L = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z), iL = 1.0 / L;
    const X3 t = {iL * v.x, iL * v.y, iL * v.z};
    const X3 bb = {bVec[3 * l], bVec[3 * l + 1], bVec[3 * l + 2]};
    s[i] = {n1, t, bb, {t.y * bb.z - t.z * bb.y, t.z * bb.x - t.x * bb.z, t.x * bb.y - t.y * bb.x}, L};
  }
  for (int64_t j = 0; j < M; ++j) {
    double sig[6] = {0, 0, 0, 0, 0, 0};
    const X3 x = {x0[3 * j], x0[3 * j + 1], x0[3 * j + 2]};
    for (int64_t q = 0; q < numSeg; ++q) ddd::sx::sigma_point(K, s[q], x, sig);
    for (int k = 0; k < 6; ++k) sigma[6 * j + k] = sig[k];
  }
}
