// df64 policies of the shared tile body (tile_body.cuh): the general-branch
// pair arithmetic in double-float (pairs of FP32 on the FP32 pipes).
//   FORM 0: every general-pair operation in df64 (general_pair_df);
//   FORM 1: corner antiderivatives and moments in df64, V-vector assembly and
//           node sums in FP32 (general_pair_mixed), the "f32c" form.
// Used by the precision-form kernels (segseg_df.cu), the batched persistent
// kernel (segseg_batch.cu) and the surrogate's exact passes
// (surrogate_force.cu).  Include from translation units compiled with
// --fmad=false (df64 needs exact TwoSum/TwoProd).
#pragma once
#include <cstdint>

#include "pair_df.cuh"
#include "pair_f64.cuh"
#include "tile_body.cuh"

namespace ddd {

// Band around sqrt(eps) inside which the df64 value of 1 - c^2 is not trusted
// to decide the branch; there the FP64 value decides.
constexpr float kThrHi = 1.4901312e-08f;  // sqrt(eps) * (1 + 1e-5)
constexpr float kThrLo = 1.4901012e-08f;  // sqrt(eps) * (1 - 1e-5)

struct SegDF {
  DV3 b, n1, n2, t;
  df64 tN;
};

// Segment i of the df64 SoA (26 float rows of ld: row 2k = hi, row 2k+1 = lo
// of FP64 row k).
__device__ __forceinline__ SegDF load_seg_df(const float* __restrict__ s, int64_t ld, int64_t i) {
  auto g = [&](int k) { return df64{s[(2 * k) * ld + i], s[(2 * k + 1) * ld + i]}; };
  SegDF r;
  r.n1 = {g(0), g(1), g(2)};
  r.n2 = {g(3), g(4), g(5)};
  r.b = {g(6), g(7), g(8)};
  r.t = {g(9), g(10), g(11)};
  r.tN = g(12);
  return r;
}

__device__ __forceinline__ void add_df(float2& acc, df64 v) {
  df64 s = df64{acc.x, acc.y} + v;
  acc.x = s.hi;
  acc.y = s.lo;
}

template <int FORM>
struct PolDF {
  using Seg = SegDF;
  using Scalar = df64;
  using Vec = DV3;
  using Acc = DV3;
  struct Consts {
    KConstsDF K;
    KConstsF KF;
  };
  template <int T>
  struct Tile {
    float seg[26][T];
    float2 fj[T / 32][6][T];
  };
  static __device__ __forceinline__ Seg load_global(const TileArgs& A, int64_t i) {
    return load_seg_df(A.soadf, A.npad, i);
  }
  template <int T>
  static __device__ __forceinline__ void load_tile(const TileArgs& A, Tile<T>& s, int64_t j0, int t) {
#pragma unroll
    for (int k = 0; k < 26; ++k) s.seg[k][t] = A.soadf[k * A.npad + j0 + t];
  }
  template <int T>
  static __device__ __forceinline__ void zero_cols(Tile<T>& s, int t) {
#pragma unroll
    for (int w = 0; w < T / 32; ++w)
#pragma unroll
      for (int c = 0; c < 6; ++c) s.fj[w][c][t] = make_float2(0.0f, 0.0f);
  }
  template <int T>
  static __device__ __forceinline__ Seg load_smem(const Tile<T>& s, int j) {
    auto g = [&](int q) { return df64{s.seg[2 * q][j], s.seg[2 * q + 1][j]}; };
    Seg r;
    r.n1 = {g(0), g(1), g(2)};
    r.n2 = {g(3), g(4), g(5)};
    r.b = {g(6), g(7), g(8)};
    r.t = {g(9), g(10), g(11)};
    r.tN = g(12);
    return r;
  }
  // The branch of the FP64 kernel: decided in df64 away from the threshold,
  // in FP64 (the FP64 kernel's own operations) within 1e-5 of it.
  static __device__ __forceinline__ bool is_general(const TileArgs& A, const Seg& a, const Seg& b, int64_t gi,
                                                    int64_t gj, df64& c) {
    c = dot(a.t, b.t);
    df64 omc = df(1.0f) - c * c;
    if (omc.hi > kThrHi) return true;
    if (omc.hi < kThrLo) return false;
    const int64_t n = A.npad;
    D3 ti = {A.soa[9 * n + gi], A.soa[10 * n + gi], A.soa[11 * n + gi]};
    D3 tj = {A.soa[9 * n + gj], A.soa[10 * n + gj], A.soa[11 * n + gj]};
    double c64 = dot(ti, tj);
    return (1.0 - c64 * c64) > kSqrtEps;
  }
  template <bool BOTH>
  static __device__ __forceinline__ void general(const Consts& KP, const TileArgs&, const Seg& a, const Seg& b,
                                                 df64 c, DV3& F1, DV3& F2, DV3& F3, DV3& F4) {
    if (FORM == 0)
      general_pair_df<true, BOTH>(KP.K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
    else
      general_pair_mixed<true, BOTH, true>(KP.K, KP.KF, f3(a.b), a.n1, a.n2, a.t, a.tN.hi, f3(b.b), b.n1, b.n2, b.t,
                                           b.tN.hi, c, F1, F2, F3, F4);
  }
  // Dense pass of the classified modes: one general-branch pair, both sides.
  static __device__ __forceinline__ void dense_general(const Consts& KP, const TileArgs& A, int64_t gi, int64_t gj,
                                                       D3& F1, D3& F2, D3& F3, D3& F4) {
    const Seg a = load_seg_df(A.soadf, A.npad, gi), b = load_seg_df(A.soadf, A.npad, gj);
    DV3 G1, G2, G3, G4;
    general<true>(KP, A, a, b, dot(a.t, b.t), G1, G2, G3, G4);
    F1 = acc_to_d3(G1);
    F2 = acc_to_d3(G2);
    F3 = acc_to_d3(G3);
    F4 = acc_to_d3(G4);
  }
  template <int T>
  static __device__ __forceinline__ void add_col(Tile<T>& s, int warp, int j, const DV3& F3, const DV3& F4) {
    add_df(s.fj[warp][0][j], F3.x);
    add_df(s.fj[warp][1][j], F3.y);
    add_df(s.fj[warp][2][j], F3.z);
    add_df(s.fj[warp][3][j], F4.x);
    add_df(s.fj[warp][4][j], F4.y);
    add_df(s.fj[warp][5][j], F4.z);
  }
  static __device__ __forceinline__ DV3 acc_zero() { return {df(0.f), df(0.f), df(0.f)}; }
  static __device__ __forceinline__ void acc_add(DV3& a, const DV3& v) { a = a + v; }
  static __device__ __forceinline__ D3 acc_to_d3(const DV3& a) {
    return {df_to_double(a.x), df_to_double(a.y), df_to_double(a.z)};
  }
  template <int T>
  static __device__ __forceinline__ double col_sum(const Tile<T>& s, int c, int t) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < T / 32; ++w) v += (double)s.fj[w][c][t].x + (double)s.fj[w][c][t].y;
    return v;
  }
};

// Host-side split of the FP64 constants into (hi, lo) floats, and FP32 copies.
inline KConstsDF kconsts_df(const KConsts& K) {
  auto s = [](double d) {
    float hi = (float)d;
    return df64{hi, (float)(d - (double)hi)};
  };
  return KConstsDF{s(K.aSq), s(K.mu4pi), s(K.mu4pinu), s(K.mu8piaSq), s(K.mu4pinuaSq)};
}
inline KConstsF kconsts_f(const KConsts& K) {
  return KConstsF{(float)K.mu4pi, (float)K.mu4pinu, (float)K.mu8piaSq, (float)K.mu4pinuaSq};
}

}  // namespace ddd
