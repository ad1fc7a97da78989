// Host build of the precision forms' pair arithmetic: ddd.jl_gb300/csrc/
// pair_df.cuh compiled as plain C++ (df64.cuh falls back to std:: functions),
// so that the df64 and f32c general-branch formulas can be checked against the
// FP64 oracle on a CPU.  Test infrastructure only; the product runs these
// formulas on the GPU.  Build with -ffp-contract=off: the double-float
// error-free transforms need every FP32 operation rounded on its own.
//
// Inputs per segment, 13 doubles, as the GPU's FP64 segment structure holds
// them: n1 xyz, n2 xyz, b xyz, t xyz (unit direction), tN = 1/|n2 - n1|.
// The GPU splits each into a (hi, lo) float pair; so does this file.
#include <cstdint>

#include "pair_df.cuh"

using namespace ddd;

namespace {

DV3 dv3(const double* v) { return {df_from_double(v[0]), df_from_double(v[1]), df_from_double(v[2])}; }

void store(const DV3& f, double* out) {
  out[0] = df_to_double(f.x);
  out[1] = df_to_double(f.y);
  out[2] = df_to_double(f.z);
}

}  // namespace

// k: aSq, mu4pi, mu8pi, mu4pinu (FP64, as ddd_consts).  form 0: df64 (every
// general-pair operation in double-float); form 1: f32c (corner terms in
// double-float, V-vector assembly in FP32).  For pair q (segments p[2q],
// p[2q+1], 0-based rows of segs), out[12q ..] = F1, F2 (nodes of the first
// segment), F3, F4 (nodes of the second).
extern "C" void df_pair_forces(int form, const double* k, const double* segs, const int64_t* p, int64_t nPairs,
                               double* out) {
  const double aSq = k[0], mu4pi = k[1], mu8pi = k[2], mu4pinu = k[3];
  const double mu8piaSq = aSq * mu8pi, mu4pinuaSq = aSq * mu4pinu;
  const KConstsDF K{df_from_double(aSq), df_from_double(mu4pi), df_from_double(mu4pinu), df_from_double(mu8piaSq),
                    df_from_double(mu4pinuaSq)};
  const KConstsF KF{(float)mu4pi, (float)mu4pinu, (float)mu8piaSq, (float)mu4pinuaSq};
  for (int64_t q = 0; q < nPairs; ++q) {
    const double* a = segs + 13 * p[2 * q];
    const double* b = segs + 13 * p[2 * q + 1];
    const DV3 n11 = dv3(a), n12 = dv3(a + 3), b1 = dv3(a + 6), t1 = dv3(a + 9);
    const DV3 n21 = dv3(b), n22 = dv3(b + 3), b2 = dv3(b + 6), t2 = dv3(b + 9);
    const df64 t1N = df_from_double(a[12]), t2N = df_from_double(b[12]);
    const df64 c = dot(t1, t2);
    DV3 F1, F2, F3, F4;
    if (form == 0)
      general_pair_df<true, true>(K, b1, n11, n12, t1, t1N, b2, n21, n22, t2, t2N, c, F1, F2, F3, F4);
    else
      general_pair_mixed<true, true, true>(K, KF, f3(b1), n11, n12, t1, t1N.hi, f3(b2), n21, n22, t2, t2N.hi, c, F1,
                                           F2, F3, F4);
    store(F1, out + 12 * q);
    store(F2, out + 12 * q + 3);
    store(F3, out + 12 * q + 6);
    store(F4, out + 12 * q + 9);
  }
}

// The mixed σ̃ form (sigma_point_mixed): k5 = aSq, mu4pi, mu8pi, mu4pinu,
// nuMu4pinu.  Each point's six components (xx, yy, zz, xy, xz, yz) summed
// over the segments in order in df64, as the GPU kernel does; out[6j ..].
extern "C" void df_sigma_points(const double* k5, const double* segs, int64_t nSeg, const double* x, int64_t M,
                                double* out) {
  KConstsSig K;
  K.aSq = df_from_double(k5[0]);
  K.mu4pi = (float)k5[1];
  K.mu4pinu = (float)k5[3];
  K.nuMu4pinu = (float)k5[4];
  K.aSq32 = (float)k5[0];
  K.aSqMu8pi = (float)(k5[0] * k5[2]);
  for (int64_t j = 0; j < M; ++j) {
    const DV3 xj = dv3(x + 3 * j);
    df64 sig[6];
    for (int c = 0; c < 6; ++c) sig[c] = df(0.0f);
    for (int64_t s = 0; s < nSeg; ++s) {
      const double* a = segs + 13 * s;
      const F3 b = {(float)a[6], (float)a[7], (float)a[8]};
      sigma_point_mixed(K, b, dv3(a), dv3(a + 3), dv3(a + 9), xj, sig);
    }
    for (int c = 0; c < 6; ++c) out[6 * j + c] = df_to_double(sig[c]);
  }
}

// The planned far-field form on the mixed arithmetic: a pair's nodal forces by
// nq-point Gauss quadrature (nq = 2 or 3) of the partner's mixed-form σ̃, the
// force per unit parameter (σ b) × l and the node sums in FP32 (l = n2 - n1).
// Same statement as oracle_segseg_pair_quad, in the arithmetic a GPU kernel of
// that form would use.  k5 and segs as df_sigma_points; pairs as
// df_pair_forces.
extern "C" void df_pair_quad_forces(const double* k5, const double* segs, const int64_t* p, int64_t nPairs, int nq,
                                    double* out) {
  static const float X[2][3] = {{0.21132486540518713f, 0.78867513459481287f, 0.0f},
                                {0.11270166537925831f, 0.5f, 0.88729833462074169f}};
  static const float W[2][3] = {{0.5f, 0.5f, 0.0f}, {0.27777777777777778f, 0.44444444444444444f, 0.27777777777777778f}};
  KConstsSig K;
  K.aSq = df_from_double(k5[0]);
  K.mu4pi = (float)k5[1];
  K.mu4pinu = (float)k5[3];
  K.nuMu4pinu = (float)k5[4];
  K.aSq32 = (float)k5[0];
  K.aSqMu8pi = (float)(k5[0] * k5[2]);
  const int r = nq == 3 ? 1 : 0;
  for (int64_t q = 0; q < nPairs; ++q) {
    const double* S[2] = {segs + 13 * p[2 * q], segs + 13 * p[2 * q + 1]};
    for (int side = 0; side < 2; ++side) {
      const double* me = S[side];
      const double* ot = S[1 - side];
      const DV3 n1 = dv3(me), l = dv3(me + 3) - dv3(me);
      const F3 bm = {(float)me[6], (float)me[7], (float)me[8]};
      const F3 lf = f3(l);
      const F3 bo = {(float)ot[6], (float)ot[7], (float)ot[8]};
      F3 Fa = {0.f, 0.f, 0.f}, Fb = {0.f, 0.f, 0.f};
      for (int g = 0; g < (r ? 3 : 2); ++g) {
        const DV3 x = n1 + df(X[r][g]) * l;
        df64 sig[6];
        for (int c = 0; c < 6; ++c) sig[c] = df(0.0f);
        sigma_point_mixed(K, bo, dv3(ot), dv3(ot + 3), dv3(ot + 9), x, sig);
        float s6[6];
        for (int c = 0; c < 6; ++c) s6[c] = sig[c].hi + sig[c].lo;
        const F3 sb = {s6[0] * bm.x + s6[3] * bm.y + s6[4] * bm.z, s6[3] * bm.x + s6[1] * bm.y + s6[5] * bm.z,
                       s6[4] * bm.x + s6[5] * bm.y + s6[2] * bm.z};
        const F3 f = cross(sb, lf);
        Fa = Fa + (W[r][g] * (1.0f - X[r][g])) * f;
        Fb = Fb + (W[r][g] * X[r][g]) * f;
      }
      double* o = out + 12 * q + 6 * side;
      o[0] = Fa.x, o[1] = Fa.y, o[2] = Fa.z, o[3] = Fb.x, o[4] = Fb.y, o[5] = Fb.z;
    }
  }
}
