// The field-point stress σ̃ of one segment at one point in a reformulated FP64
// form with about half the FP64 instructions of the reference's literal
// evaluation (sigma_point in pair_f64.cuh), for DDD_MODE_FP64_FAST.
// Same formula (DislocationFEM.jl:135-299); differences:
//   * the six components from seven scalars and four vectors: with
//     alpha = c (s03 + a^2 s05), beta = mu4pinu s03, gamma = -(mu4pi s03 +
//     a^2 mu8pi s05), delta = a^2 mu8pi s15 - nu mu4pinu s13, eps = c s05,
//     zeta = -c s15, eta = c s25 (c = mu4pinu (nd x b).t, s.. the endpoint
//     differences) and u = beta nd + delta t, g = gamma t, v = eps nd + zeta t,
//     w = zeta nd + eta t, component (p, q) is
//       [p = q] alpha + u_p tb_q + u_q tb_p + g_p db_q + g_q db_p + nd_p v_q
//       + t_p w_q,
//     tb = t x b, db = nd x b: the reference's I03..I25 terms regrouped (each
//     product of two of nd, t, tb, db appears once);
//   * t x b and the segment length come with the segment (once per segment,
//     not per point), and s2 = s1 + L;
//   * 1/Ra as one reciprocal square root instead of a square root and a
//     division;
//   * explicit fused multiply-adds throughout.
// The reference arithmetic's own error is ~1e-15 normwise (1e-12 per point
// where σ̃ is small against long double); this form stays within the same
// per-point bound (1e-10 |σ| + 1e-12 max |σ|) with room to spare, measured
// against long double on a CPU build of this header.
#pragma once
#include "fastmath_f64.cuh"

namespace ddd {
namespace sx {

struct X3 {
  double x, y, z;
};

// One segment as the fast σ̃ kernel reads it: first node, unit direction,
// Burgers vector, t x b and the length.
struct SegS {
  X3 n1, t, b, tb;
  double L;
};

struct KS {
  double a2, mu4pi, mu4pinu, nuMu4pinu, a2mu8pi;
};

FM_HD double rsqrt_(double v) {
#if defined(__CUDA_ARCH__)
  return ::rsqrt(v);
#else
  return 1.0 / std::sqrt(v);
#endif
}

// Endpoint terms at coordinate s along the segment's line: s03, s13, s05,
// s15, s25 of the reference (DislocationFEM.jl:167-199).
FM_HD void endpoint(double A, double Ainv, double s, double& s03, double& s13, double& s05, double& s15, double& s25) {
  using fm::fma_;
  const double r = rsqrt_(fma_(s, s, A));  // 1/Ra
  const double r2 = r * r;
  const double r3 = r2 * r;
  const double sr3 = s * r3;
  s03 = (s * r) * Ainv;
  s13 = -r;
  s05 = fma_(2.0, s03, sr3) * Ainv;
  s15 = -r3;
  s25 = s03 - sr3;
}

// σ̃ of segment sg at point x, added into sig[6] (xx, yy, zz, xy, xz, yz).
FM_HD void sigma_point(const KS& K, const SegS& sg, X3 x, double* sig) {
  using fm::fma_;
  const X3 R = {x.x - sg.n1.x, x.y - sg.n1.y, x.z - sg.n1.z};
  const X3 t = sg.t;
  const double Rdt = fma_(R.z, t.z, fma_(R.y, t.y, R.x * t.x));
  const X3 d = {fma_(-Rdt, t.x, R.x), fma_(-Rdt, t.y, R.y), fma_(-Rdt, t.z, R.z)};
  const double A = fma_(d.z, d.z, fma_(d.y, d.y, fma_(d.x, d.x, K.a2)));
  const double Ainv = 1.0 / A;
  const double s1 = -Rdt, s2 = s1 + sg.L;
  double a03, a13, a05, a15, a25, b03, b13, b05, b15, b25;
  endpoint(A, Ainv, s1, a03, a13, a05, a15, a25);
  endpoint(A, Ainv, s2, b03, b13, b05, b15, b25);
  const double s03 = b03 - a03, s13 = b13 - a13, s05 = b05 - a05, s15 = b15 - a15, s25 = b25 - a25;

  const X3 b = sg.b, tb = sg.tb;
  const X3 db = {fma_(d.y, b.z, -(d.z * b.y)), fma_(d.z, b.x, -(d.x * b.z)), fma_(d.x, b.y, -(d.y * b.x))};
  const double c = K.mu4pinu * fma_(db.z, t.z, fma_(db.y, t.y, db.x * t.x));
  const double alpha = c * fma_(K.a2, s05, s03);
  const double beta = K.mu4pinu * s03;
  const double gamma = -fma_(K.a2mu8pi, s05, K.mu4pi * s03);
  const double delta = fma_(K.a2mu8pi, s15, -(K.nuMu4pinu * s13));
  const double eps = c * s05, zeta = -(c * s15), eta = c * s25;
  const double u[3] = {fma_(delta, t.x, beta * d.x), fma_(delta, t.y, beta * d.y), fma_(delta, t.z, beta * d.z)};
  const double g[3] = {gamma * t.x, gamma * t.y, gamma * t.z};
  const double v[3] = {fma_(zeta, t.x, eps * d.x), fma_(zeta, t.y, eps * d.y), fma_(zeta, t.z, eps * d.z)};
  const double w[3] = {fma_(eta, t.x, zeta * d.x), fma_(eta, t.y, zeta * d.y), fma_(eta, t.z, zeta * d.z)};
  const double dd[3] = {d.x, d.y, d.z}, tt[3] = {t.x, t.y, t.z}, tbv[3] = {tb.x, tb.y, tb.z},
               dbv[3] = {db.x, db.y, db.z};
#pragma unroll
  for (int cpt = 0; cpt < 6; ++cpt) {
    const int p = cpt < 3 ? cpt : (cpt == 5 ? 1 : 0);
    const int q = cpt < 3 ? cpt : (cpt == 3 ? 1 : 2);
    double acc = cpt < 3 ? sig[cpt] + alpha : sig[cpt];
    acc = fma_(u[p], tbv[q], acc);
    acc = fma_(u[q], tbv[p], acc);
    acc = fma_(g[p], dbv[q], acc);
    acc = fma_(g[q], dbv[p], acc);
    acc = fma_(dd[p], v[q], acc);
    acc = fma_(tt[p], w[q], acc);
    sig[cpt] = acc;
  }
}

}  // namespace sx
}  // namespace ddd
