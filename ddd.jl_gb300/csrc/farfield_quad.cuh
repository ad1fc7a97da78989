// Far-field pair force by Gauss-Legendre quadrature on both segments, in FP32.
//
// The force on segment f (nodes n1f, n2f, Burgers b_f, l_f = n2f - n1f) from
// the stress of segment o is the line integral
//   F_k = int_0^1 N_k(xi) (sigma_o(x(xi)) b_f) x l_f dxi,  x(xi) = n1f + xi l_f,
// N_1 = 1 - xi, N_2 = xi (DislocationForces.jl:292-300 for the force density).
// sigma_o is the non-singular stress of segment o (DislocationFEM.jl:135-299):
// with R = x - n1o, s1 = -R.t_o, nd = R - (R.t_o) t_o, A = a^2 + |nd|^2 and
// endpoint functions of s (Ra = sqrt(A + s^2))
//   s03 = s/(Ra A), s13 = -1/Ra, s05 = (2 s03 + s/Ra^3)/A, s15 = -1/Ra^3,
//   s25 = s03 - s/Ra^3,
// sigma = sum_term I_term [s_term(s1 + L_o) - s_term(s1)], the I_term tensors
// built from t_o, nd and b_o.  Each endpoint difference is the integral of
// the s-derivative, and those are free of cancellation:
//   s03' = 1/Ra^3, s13' = s/Ra^3, s05' = 3/Ra^5, s15' = 3s/Ra^5, s25' = 3s^2/Ra^5,
// so for a far pair both integrals go to Gauss-Legendre rules in plain FP32
// (the analytic four-corner form and the endpoint differences cancel as the
// pair separates, which is what the df64 forms pay for).  The I_term tensors
// are contracted with b_f first:
//   V03 = c b_f + mu4pinu (nd (txb.b_f) + txb (nd.b_f)) - mu4pi (t (dxb.b_f) + dxb (t.b_f))
//   V13 = -nu mu4pinu (t (txb.b_f) + txb (t.b_f))
//   V05 = c (a^2 b_f + nd (nd.b_f)) - a^2 mu8pi (t (dxb.b_f) + dxb (t.b_f))
//   V15 = a^2 mu8pi (t (txb.b_f) + txb (t.b_f)) - c (t (nd.b_f) + nd (t.b_f))
//   V25 = c t (t.b_f)
// with t = t_o, txb = t_o x b_o, dxb = nd x b_o, c = mu4pinu (dxb.t_o); then
// sigma b_f = L_o sum_h w_h sum_term s_term'(s1 + L_o xi_h) V_term.
//
// Accuracy (measured against the long-double analytic force, 3-point rules):
// median 1.5e-10 / max 2e-9 relative at R/L = 30, ~1e-8 at R/L = 1000, where
// the analytic FP64 formula itself is off by ~3e-5; the FP32 arithmetic adds
// ~1e-7.  The caller keeps this form to pairs R >= kappa max(L_f, L_o).
//
// Device functions under nvcc; plain inline C++ under a host compiler.
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define QF_HD __host__ __device__ __forceinline__
#else
#define QF_HD inline
#endif

namespace ddd {
namespace qf {

struct QConst {
  float a2, mu4pi, mu4pinu, nuMu4pinu, a2mu8pi;
};

// Gauss-Legendre points and weights on [0, 1].
template <int NQ>
struct Rule;
template <>
struct Rule<2> {
  static QF_HD float x(int i) { return i == 0 ? 0.21132486540518712f : 0.78867513459481288f; }
  static QF_HD float w(int) { return 0.5f; }
};
template <>
struct Rule<3> {
  static QF_HD float x(int i) { return i == 0 ? 0.11270166537925831f : (i == 1 ? 0.5f : 0.88729833462074169f); }
  static QF_HD float w(int i) { return i == 1 ? 0.44444444444444444f : 0.27777777777777778f; }
};

// The argument is a squared distance between points of a far pair's segments
// (>= ((kappa - 1) L)^2 > 0), never subnormal, so the flush-to-zero form of the
// hardware approximation gives the same value without the subnormal handling
// that rsqrtf carries.
QF_HD float rsqrt_(float v) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(v));
#else
  const float y = 1.0f / std::sqrt(v);
#endif
  return y * (1.5f - 0.5f * v * y * y);  // one Newton step
}

struct V3f {
  float x, y, z;
};
QF_HD V3f operator+(V3f a, V3f b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
QF_HD V3f operator-(V3f a, V3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
QF_HD V3f operator*(float s, V3f a) { return {s * a.x, s * a.y, s * a.z}; }
QF_HD float dot(V3f a, V3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
QF_HD V3f cross(V3f a, V3f b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// Forces on the field segment's two nodes (Fa on n1f, Fb on n2f) from the
// source segment o.  dm = m_f - m_o (midpoint difference, FP32 to ~1e-7
// relative), lf = n2f - n1f, bf its Burgers vector; to, Lo, bo of the source.
//
// sigma b_f at a field point is Lo sum_term S_term V_term (S_term the weighted
// source integrals of the s-derivatives).  Expanding the five V_term, the sum
// is a combination of five vectors only, b_f, nd, t x b, t and nd x b:
//   beta_b   = c (S03 + a^2 S05)
//   beta_nd  = mu4pinu S03 (txb.b_f) + c (S05 (nd.b_f) - S15 (t.b_f))
//   beta_txb = mu4pinu S03 (nd.b_f) + (t.b_f) h
//   beta_t   = -(dxb.b_f) g + (txb.b_f) h + c (S25 (t.b_f) - S15 (nd.b_f))
//   beta_dxb = -(t.b_f) g
// with g = mu4pi S03 + a^2 mu8pi S05 and h = a^2 mu8pi S15 - nu mu4pinu S13
// (V15's t-only part and V13 both fold into h).  Lo is folded into the source
// weights.
template <int NQ>
QF_HD void side(const QConst& K, V3f dm, V3f lf, V3f bf, V3f to, float Lo, V3f bo, V3f& Fa, V3f& Fb) {
  const V3f txb = cross(to, bo);
  const float tb = dot(to, bf), txbb = dot(txb, bf);
  const V3f R0 = dm + (0.5f * Lo) * to;  // x - n1o at xi = 1/2
  Fa = {0.f, 0.f, 0.f};
  Fb = {0.f, 0.f, 0.f};
#pragma unroll
  for (int g = 0; g < NQ; ++g) {
    const float xi = Rule<NQ>::x(g);
    const V3f R = R0 + (xi - 0.5f) * lf;
    const float Rdt = dot(R, to);
    const V3f nd = R - Rdt * to;
    const float A = K.a2 + dot(nd, nd);
    const float s1 = -Rdt;
    const V3f dxb = cross(nd, bo);
    const float c = K.mu4pinu * dot(dxb, to);
    const float ndb = dot(nd, bf), dxbb = dot(dxb, bf);
    float S03 = 0.f, S13 = 0.f, S05 = 0.f, S15 = 0.f, S25 = 0.f;
#pragma unroll
    for (int h = 0; h < NQ; ++h) {
      const float s = s1 + Lo * Rule<NQ>::x(h);
      const float ri = rsqrt_(A + s * s);
      const float ri2 = ri * ri;
      const float w3 = (Lo * Rule<NQ>::w(h)) * ri2 * ri;
      const float w5 = 3.0f * w3 * ri2;
      S03 += w3;
      S13 += w3 * s;
      S05 += w5;
      S15 += w5 * s;
      S25 += w5 * s * s;
    }
    const float gq = K.mu4pi * S03 + K.a2mu8pi * S05;
    const float hq = K.a2mu8pi * S15 - K.nuMu4pinu * S13;
    const float m03 = K.mu4pinu * S03;
    const float bb = c * (S03 + K.a2 * S05);
    const float bn = m03 * txbb + c * (S05 * ndb - S15 * tb);
    const float bx = m03 * ndb + tb * hq;
    const float bt = txbb * hq - dxbb * gq + c * (S25 * tb - S15 * ndb);
    const float bd = -tb * gq;
    const V3f sb = bb * bf + bn * nd + bx * txb + bt * to + bd * dxb;
    const V3f f = cross(sb, lf);
    const float w = Rule<NQ>::w(g);
    Fa = Fa + (w * (1.0f - xi)) * f;
    Fb = Fb + (w * xi) * f;
  }
}

// sqrt(eps(Float64)) and hCotanθc of the reference's near-parallel branch
// (DislocationForces.jl:892,1194).
constexpr double kParEps = 1.4901161193847656e-08;
constexpr double kParHCot = 4075.672300430329;

// A source segment of a near-parallel pair as the reference rebuilds it:
// offset of its midpoint from the original source segment's midpoint,
// direction, length and Burgers vector (FP32).
struct Src {
  V3f off, to;
  float Lo;
  V3f bo;
};

QF_HD double dotd(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// One side of calcParSegSegForce (DislocationForces.jl:1204-1317, :1319-1433):
// the source segment nb1 -> nb1 + lb (nb1 = -lb/2 relative to the source's
// midpoint, nb1abs its absolute position) is projected onto the field
// segment's direction ta and pulled in by the critical angle: with
// proj = (lb.ta) ta, diff = lb - proj, the segment nbm1 = nb1 + diff/2 +
// hCot |diff| ta -> nbm2 = nb1 + proj + diff/2 - hCot |diff| ta.  When the
// rejection is not negligible against the positions (magDiffSq >
// sqrt(eps) (|nbm1|^2 + |nbm2|^2), absolute coordinates; SIDE 1 takes
// magDiffSq = diff.diff, SIDE 2 |diff|^2) the two connectors nb1 -> nbm1 and
// nbm2 -> nb1 + lb are sources too.  Writes up to three sources; returns how
// many.  The force on the field segment is the sum of their quadratures: the
// reference evaluates the same geometry analytically.
//
// Only the rejection needs FP64 (it is |lb| sin(angle), far below |lb|): lb.ta,
// diff and diff.diff are formed from the FP64 ta and lb as the reference forms
// them.  Everything else comes in FP32, as the general path already holds it:
// t and lv (ta and lb rounded), the Burgers vector b, and a0, the source's
// first node in absolute coordinates to ~1e-7 relative.  The sources simplify
// exactly: the main source runs along ta with signed length lb.ta - 2 hCot
// |diff| and its midpoint is the source's own (nb1 + lb/2), and both
// connectors are the vector diff/2 + hCot |diff| ta.  The connector test is
// decided in FP32 (a0's error is far inside the margin) unless it falls within
// 1e-5 of its threshold, where it is evaluated in FP64 exactly as written
// above, on nb1abs(k), the FP64 node.
template <int SIDE, class Abs>
QF_HD int par_sources(const double* ta, const double* lb, V3f t, V3f lv, V3f b, V3f a0, const Abs& nb1abs,
                      Src* out) {
  const double tmp = dotd(lb, ta);
  const double proj[3] = {tmp * ta[0], tmp * ta[1], tmp * ta[2]};
  const double diff[3] = {lb[0] - proj[0], lb[1] - proj[1], lb[2] - proj[2]};
  const double dd = dotd(diff, diff);
  const V3f d = {(float)diff[0], (float)diff[1], (float)diff[2]};
  const V3f n1 = -0.5f * lv;  // the FP32 rounding of -lb/2 (exact scaling)
  const float h = (float)kParHCot * std::sqrt((float)dd);  // hCot |diff|
  int n = 0;
  const float Lm = (float)tmp - 2.0f * h;  // signed length of nbm1 -> nbm2 along ta
  if (Lm != 0.0f) {
    out[n].off = n1 + 0.5f * lv;
    out[n].to = Lm > 0.0f ? t : V3f{-t.x, -t.y, -t.z};
    out[n].Lo = std::fabs(Lm);
    out[n].bo = b;
    ++n;
  }
  // Connector test: |nbm1|^2 + |nbm2|^2 in FP32, FP64 next to the threshold.
  const V3f c = 0.5f * d + h * t;  // nb1 -> nbm1, and nbm2 -> nb1 + lb
  const V3f a1 = a0 + c, a2 = a0 + (float)tmp * t + 0.5f * d - h * t;
  const float thr = (float)kParEps * (dot(a1, a1) + dot(a2, a2));
  const float ddf = (float)dd;
  bool conn;
  if (ddf > thr * 1.00001f) {
    conn = true;
  } else if (ddf < thr * 0.99999f) {
    conn = false;
  } else {
    const double magDiff = sqrt(dd);
    double e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
      const double na = nb1abs(k);
      const double tv1 = 0.5 * diff[k], tv2 = kParHCot * magDiff * ta[k];
      e1[k] = na + tv1 + tv2;
      e2[k] = na + proj[k] + tv1 - tv2;
    }
    const double magDiffSq = SIDE == 1 ? dd : magDiff * magDiff;
    conn = magDiffSq > kParEps * (dotd(e1, e1) + dotd(e2, e2));
  }
  const float Lc = std::sqrt(dot(c, c));
  if (conn && Lc > 0.0f) {
    const V3f tc = (1.0f / Lc) * c;
    out[n] = {n1 + 0.5f * c, tc, Lc, b};
    ++n;
    out[n] = {n1 + (float)tmp * t + 0.5f * d - h * t + 0.5f * c, tc, Lc, b};
    ++n;
  }
  return n;
}

// FP64 record of one segment for the near-parallel path: node 1, n2 - n1 and
// the unit direction (the values the FP64 kernels use).
struct SegD {
  double n1[3], l[3], t[3];
};

// The reference's branch decision on the FP64 directions (c = t_i.t_j and
// 1 - c^2 rounded as DislocationForces.jl:888-892 rounds them): true for the
// near-parallel branch.
QF_HD bool par_decision(const double* ti, const double* tj, double& c) {
#if defined(__CUDA_ARCH__)
  c = __dadd_rn(__dadd_rn(__dmul_rn(ti[0], tj[0]), __dmul_rn(ti[1], tj[1])), __dmul_rn(ti[2], tj[2]));
  return !(__dsub_rn(1.0, __dmul_rn(c, c)) > kParEps);
#else
  c = ti[0] * tj[0] + ti[1] * tj[1] + ti[2] * tj[2];
  return !(1.0 - c * c > kParEps);
#endif
}

// FP64 node 1 of a segment, or its node 2 (n1 + l, as the reference forms
// the reversed segment's start) when flipped: the connector test's operand.
struct NodeAbs {
  const SegD* s;
  bool end2;
  QF_HD double operator()(int k) const { return end2 ? s->n1[k] + s->l[k] : s->n1[k]; }
};

// A near-parallel pair (segment i = seg 1, j = seg 2 of calcParSegSegForce):
// forces on i (Fa, Fb) and on j (Fc, Fd) from the reference's rebuilt sources.
// FP64 from si, sj: the directions t and segment vectors l (the rejection's
// operands) and the nodes (the connector test near its threshold).  FP32 as
// the general path takes them: dm = m_i - m_j, the midpoints mi, mj, the unit
// directions ti, tj (the FP64 ones rounded), segment vectors and Burgers
// vectors.  Seg 1 is flipped when c = t_i.t_j < 0 (flip; for a near-parallel
// pair |c| > 1 - 1e-8, so the FP32 dot product has the same sign), as the
// reference does: side 1 then projects onto -t_i, and side 2's source is
// seg 1 reversed (its Burgers vector negated).
template <int NQ>
QF_HD void par_pair(const QConst& K, const SegD& si, const SegD& sj, bool flip, V3f dm, V3f mi, V3f mj, V3f ti,
                    V3f tj, V3f li, V3f bi, V3f lj, V3f bj, V3f& Fa, V3f& Fb, V3f& Fc, V3f& Fd) {
  Src src[3];
  Fa = Fb = Fc = Fd = {0.f, 0.f, 0.f};
  {  // side 1: field i (direction t_i, or -t_i when flipped), source j
    const double ta[3] = {flip ? -si.t[0] : si.t[0], flip ? -si.t[1] : si.t[1], flip ? -si.t[2] : si.t[2]};
    const V3f t = flip ? V3f{-ti.x, -ti.y, -ti.z} : ti;
    const int n = par_sources<1>(ta, sj.l, t, lj, bj, mj - 0.5f * lj, NodeAbs{&sj, false}, src);
    for (int q = 0; q < n; ++q) {
      V3f a, b;
      side<NQ>(K, dm - src[q].off, li, bi, src[q].to, src[q].Lo, src[q].bo, a, b);
      Fa = Fa + a;
      Fb = Fb + b;
    }
  }
  {  // side 2: field j (direction t_j), source i (reversed when flipped)
    const double lb[3] = {flip ? -si.l[0] : si.l[0], flip ? -si.l[1] : si.l[1], flip ? -si.l[2] : si.l[2]};
    const V3f lv = flip ? V3f{-li.x, -li.y, -li.z} : li;
    const V3f b = flip ? V3f{-bi.x, -bi.y, -bi.z} : bi;
    const int n = par_sources<2>(sj.t, lb, tj, lv, b, mi - 0.5f * lv, NodeAbs{&si, flip}, src);
    const V3f dmj = {-dm.x, -dm.y, -dm.z};
    for (int q = 0; q < n; ++q) {
      V3f a, bq;
      side<NQ>(K, dmj - src[q].off, lj, bj, src[q].to, src[q].Lo, src[q].bo, a, bq);
      Fc = Fc + a;
      Fd = Fd + bq;
    }
  }
}

}  // namespace qf
}  // namespace ddd
