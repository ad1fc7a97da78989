// Host build of the far-field quadrature (ddd.jl_gb300/csrc/farfield_quad.cuh),
// with its inputs prepared as the GPU pass prepares them: the midpoint
// difference from FP32 (hi, lo) midpoints, the segment vector, direction,
// length and Burgers vector rounded to FP32.  Test infrastructure only: it
// checks the form's accuracy on a CPU; the product runs the header on the GPU.
// Near pairs of the network-level function take the oracle's restatement of the
// reference (tests may use the oracle).
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../oracle/ddd_oracle.hpp"
#include "farfield_quad.cuh"

using ddd::qf::V3f;

namespace {

struct Prep {
  float mhi[3], mlo[3];
  V3f l, t, b;
  float L;
};

Prep prep(const double* s) {  // s: n1 xyz, n2 xyz, b xyz (FP64)
  Prep p;
  double l[3], L2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double m = 0.5 * (s[k] + s[3 + k]);
    p.mhi[k] = (float)m;
    p.mlo[k] = (float)(m - (double)p.mhi[k]);
    l[k] = s[3 + k] - s[k];
    L2 += l[k] * l[k];
  }
  const double L = std::sqrt(L2);
  p.L = (float)L;
  p.l = {(float)l[0], (float)l[1], (float)l[2]};
  p.t = {(float)(l[0] / L), (float)(l[1] / L), (float)(l[2] / L)};
  p.b = {(float)s[6], (float)s[7], (float)s[8]};
  return p;
}

}  // namespace

// For pair q (segments p[2q], p[2q+1], rows of segs with 9 doubles: n1, n2, b),
// out[12q ..] = forces on n1, n2 of the first segment, then of the second.
// k5 = aSq, mu4pi, mu8pi, mu4pinu, nuMu4pinu; nq = 2 or 3.
extern "C" void quad_pair_forces(const double* k5, const double* segs, const int64_t* pr, int64_t nPairs, int nq,
                                 double* out) {
  const ddd::qf::QConst K{(float)k5[0], (float)k5[1], (float)k5[3], (float)k5[4], (float)(k5[0] * k5[2])};
  for (int64_t q = 0; q < nPairs; ++q) {
    const Prep a = prep(segs + 9 * pr[2 * q]), b = prep(segs + 9 * pr[2 * q + 1]);
    const V3f dm = {(a.mhi[0] - b.mhi[0]) + (a.mlo[0] - b.mlo[0]), (a.mhi[1] - b.mhi[1]) + (a.mlo[1] - b.mlo[1]),
                    (a.mhi[2] - b.mhi[2]) + (a.mlo[2] - b.mlo[2])};
    const V3f dmr = {-dm.x, -dm.y, -dm.z};
    V3f F1, F2, F3, F4;
    if (nq == 3) {
      ddd::qf::side<3>(K, dm, a.l, a.b, b.t, b.L, b.b, F1, F2);
      ddd::qf::side<3>(K, dmr, b.l, b.b, a.t, a.L, a.b, F3, F4);
    } else {
      ddd::qf::side<2>(K, dm, a.l, a.b, b.t, b.L, b.b, F1, F2);
      ddd::qf::side<2>(K, dmr, b.l, b.b, a.t, a.L, a.b, F3, F4);
    }
    const V3f F[4] = {F1, F2, F3, F4};
    for (int k = 0; k < 4; ++k) {
      out[12 * q + 3 * k] = F[k].x;
      out[12 * q + 3 * k + 1] = F[k].y;
      out[12 * q + 3 * k + 2] = F[k].z;
    }
  }
}

// Forces on the given rows of a whole network (segs: n x 9 doubles, n1, n2, b)
// as ddd_surrogate_force with far_mode = nq computes them: far pairs (the FP32
// trust test R^2 >= kappa^2 max(L_i, L_j)^2 on FP32 midpoints and lengths) by
// the quadrature, taking the reference's near-parallel construction where its
// FP64 branch test says so (qf::par_pair, the kernel's own code), near pairs by
// the oracle's FP64 restatement of the reference.  two (nRows x n bytes, or
// NULL): far pairs flagged there take the 2-point rule whatever nq is (the
// kernel's per-tile-pair switch, decided by the caller).  out: 6 per row
// (node 1, node 2).  Summation in j order, FP64.
extern "C" void quad_network_rows(const double* k5, const double* segs, int64_t n, double kappa, int nq,
                                  const int64_t* rows, int64_t nRows, const uint8_t* two, double* out) {
  using namespace ddd::qf;
  const QConst K{(float)k5[0], (float)k5[1], (float)k5[3], (float)k5[4], (float)(k5[0] * k5[2])};
  ddd_oracle::Consts<double> KO;
  KO.aSq = k5[0];
  KO.mu4pi = k5[1];
  KO.mu8pi = k5[2];
  KO.mu4pinu = k5[3];
  KO.nuMu4pinu = k5[4];
  KO.mu8piaSq = KO.aSq * KO.mu8pi;
  KO.mu4pinuaSq = KO.aSq * KO.mu4pinu;
  std::vector<Prep> P(n);
  std::vector<SegD> D(n);
  std::vector<float> Lf(n);
  for (int64_t i = 0; i < n; ++i) {
    const double* s = segs + 9 * i;
    P[i] = prep(s);
    double l2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      D[i].n1[k] = s[k];
      D[i].l[k] = s[3 + k] - s[k];
      l2 += D[i].l[k] * D[i].l[k];
    }
    const double tN = 1.0 / std::sqrt(l2);  // the FP64 kernels' direction and inverse length
    for (int k = 0; k < 3; ++k) D[i].t[k] = D[i].l[k] * tN;
    Lf[i] = (float)(1.0 / tN);
    P[i].t = {(float)D[i].t[0], (float)D[i].t[1], (float)D[i].t[2]};
    P[i].L = Lf[i];
  }
  const float k2 = (float)(kappa * kappa);
  for (int64_t r = 0; r < nRows; ++r) {
    const int64_t i = rows[r];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t j = 0; j < n; ++j) {
      if (j == i) continue;
      const Prep &a = P[i], &b = P[j];
      const float dx = b.mhi[0] - a.mhi[0], dy = b.mhi[1] - a.mhi[1], dz = b.mhi[2] - a.mhi[2];
      const float R2 = (dx * dx + dy * dy) + dz * dz;
      const float Lm = a.L > b.L ? a.L : b.L;
      double F[6];
      if (R2 >= k2 * (Lm * Lm)) {
        const V3f dm = {(a.mhi[0] - b.mhi[0]) + (a.mlo[0] - b.mlo[0]), (a.mhi[1] - b.mhi[1]) + (a.mlo[1] - b.mlo[1]),
                        (a.mhi[2] - b.mhi[2]) + (a.mlo[2] - b.mlo[2])};
        V3f Fa, Fb, Fc, Fd;
        double c = 0.0;
        const float c32 = dot(a.t, b.t);
        const bool par = 1.0f - c32 * c32 <= 1e-5f && par_decision(D[i].t, D[j].t, c);
        const int nqp = two && two[r * n + j] ? 2 : nq;
        if (!par) {
          if (nqp == 3)
            side<3>(K, dm, a.l, a.b, b.t, b.L, b.b, Fa, Fb);
          else
            side<2>(K, dm, a.l, a.b, b.t, b.L, b.b, Fa, Fb);
        } else if (i < j) {  // segment i is the reference's seg 1
          const V3f ma = {a.mhi[0], a.mhi[1], a.mhi[2]}, mb = {b.mhi[0], b.mhi[1], b.mhi[2]};
          const bool flip = dot(a.t, b.t) < 0.0f;
          if (nqp == 3)
            par_pair<3>(K, D[i], D[j], flip, dm, ma, mb, a.t, b.t, a.l, a.b, b.l, b.b, Fa, Fb, Fc, Fd);
          else
            par_pair<2>(K, D[i], D[j], flip, dm, ma, mb, a.t, b.t, a.l, a.b, b.l, b.b, Fa, Fb, Fc, Fd);
        } else {  // segment i is seg 2: its forces are the pair's Fc, Fd
          const V3f dmr = {-dm.x, -dm.y, -dm.z};
          const V3f ma = {a.mhi[0], a.mhi[1], a.mhi[2]}, mb = {b.mhi[0], b.mhi[1], b.mhi[2]};
          const bool flip = dot(a.t, b.t) < 0.0f;
          if (nqp == 3)
            par_pair<3>(K, D[j], D[i], flip, dmr, mb, ma, b.t, a.t, b.l, b.b, a.l, a.b, Fc, Fd, Fa, Fb);
          else
            par_pair<2>(K, D[j], D[i], flip, dmr, mb, ma, b.t, a.t, b.l, b.b, a.l, a.b, Fc, Fd, Fa, Fb);
        }
        F[0] = Fa.x, F[1] = Fa.y, F[2] = Fa.z, F[3] = Fb.x, F[4] = Fb.y, F[5] = Fb.z;
      } else {
        const double *s = segs + 9 * i, *q = segs + 9 * j;
        ddd_oracle::V3<double> o[4];
        if (i < j) {
          ddd_oracle::seg_seg_force<double>(KO, {s[6], s[7], s[8]}, {s[0], s[1], s[2]}, {s[3], s[4], s[5]},
                                            {q[6], q[7], q[8]}, {q[0], q[1], q[2]}, {q[3], q[4], q[5]}, o);
          F[0] = o[0].x, F[1] = o[0].y, F[2] = o[0].z, F[3] = o[1].x, F[4] = o[1].y, F[5] = o[1].z;
        } else {
          ddd_oracle::seg_seg_force<double>(KO, {q[6], q[7], q[8]}, {q[0], q[1], q[2]}, {q[3], q[4], q[5]},
                                            {s[6], s[7], s[8]}, {s[0], s[1], s[2]}, {s[3], s[4], s[5]}, o);
          F[0] = o[2].x, F[1] = o[2].y, F[2] = o[2].z, F[3] = o[3].x, F[4] = o[3].y, F[5] = o[3].z;
        }
      }
      for (int k = 0; k < 6; ++k) acc[k] += F[k];
    }
    for (int k = 0; k < 6; ++k) out[6 * r + k] = acc[k];
  }
}

// The near-parallel construction's source count (qf::par_sources) for n
// configurations (FP64 rows: ta xyz, lb xyz, nb1abs xyz), with the FP32 inputs
// formed as the far pass forms them: ta and lb rounded, and the source's node
// from its FP32 midpoint minus half its FP32 vector.  nsrc[q] = the returned
// count (bit 1 set when the connectors were added).
extern "C" void quad_par_sources(int side, const double* cfg, int64_t n, int* nsrc) {
  for (int64_t q = 0; q < n; ++q) {
    const double* ta = cfg + 9 * q;
    const double* lb = ta + 3;
    const double* na = ta + 6;
    const V3f t = {(float)ta[0], (float)ta[1], (float)ta[2]};
    const V3f lv = {(float)lb[0], (float)lb[1], (float)lb[2]};
    const V3f m = {(float)(na[0] + 0.5 * lb[0]), (float)(na[1] + 0.5 * lb[1]), (float)(na[2] + 0.5 * lb[2])};
    const V3f a0 = m - 0.5f * lv;
    struct Abs {
      const double* p;
      double operator()(int k) const { return p[k]; }
    } abs{na};
    ddd::qf::Src src[3];
    nsrc[q] = side == 1 ? ddd::qf::par_sources<1>(ta, lb, t, lv, V3f{0.f, 0.f, 1.f}, a0, abs, src)
                        : ddd::qf::par_sources<2>(ta, lb, t, lv, V3f{0.f, 0.f, 1.f}, a0, abs, src);
  }
}
