// Host build of the far-field quadrature (ddd.jl_gb300/csrc/farfield_quad.cuh),
// with its inputs prepared as the GPU pass prepares them: the midpoint
// difference from FP32 (hi, lo) midpoints, the segment vector, direction,
// length and Burgers vector rounded to FP32.  Test infrastructure only: it
// checks the form's accuracy on a CPU; the product runs the header on the GPU.
#include <cstdint>

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
