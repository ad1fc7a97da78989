// Precision forms of the all-pairs and index-list seg-seg force: the general
// branch (the bulk of the pair arithmetic, ~95% of pairs) in df64 — pairs of
// FP32 on the FP32 pipes, ~48-bit significands — while FP64 is kept for
//   * the near-parallel branch (calcParSegSegForce, the strict FP64 code),
//   * the branch decision (computed in df64, settled in FP64 whenever it falls
//     within 1e-5 of the sqrt(eps) threshold, so pairs take exactly the branch
//     the FP64 kernel gives them),
//   * the per-node accumulation across tiles (partials and reduction in FP64).
// Within a tile a thread's 128 general-pair contributions add in df64.
// Tiling, scheduling, near-parallel compaction and the deterministic
// reduction are those of the FP64 kernel (segseg_f64.cu).
//
// Compiled with --fmad=false: df64 needs exact TwoSum/TwoProd, and the FP64
// near-parallel code then rounds as the strict kernel does.
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_df.cuh"
#include "pair_f64.cuh"
#include "tile_body.cuh"

namespace ddd {

namespace {

constexpr int TILE = 128;
// Band around sqrt(eps) inside which the df64 value of 1 - c^2 is not trusted
// to decide the branch; there the FP64 value decides.
constexpr float kThrHi = 1.4901312e-08f;  // sqrt(eps) * (1 + 1e-5)
constexpr float kThrLo = 1.4901012e-08f;  // sqrt(eps) * (1 - 1e-5)

struct SegDF {
  DV3 b, n1, n2, t;
  df64 tN;
};

// soadf: 26 float rows of npad: row 2k = hi, row 2k+1 = lo of FP64 row k.
__global__ void prep_df(const double* __restrict__ soa, int64_t npad, float* __restrict__ soadf) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= npad) return;
#pragma unroll
  for (int k = 0; k < 13; ++k) {
    df64 v = df_from_double(soa[k * npad + i]);
    soadf[(2 * k) * npad + i] = v.hi;
    soadf[(2 * k + 1) * npad + i] = v.lo;
  }
}

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

}  // namespace

// df64 policies of the shared tile body.  FORM 0: every general-pair operation
// in df64 (general_pair_df).  FORM 1: corner antiderivatives and moments in
// df64, V-vector assembly and node sums in FP32 (general_pair_mixed).
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

namespace {

__device__ __forceinline__ void tile_index_df(int64_t b, int64_t& I, int64_t& J) {
  int64_t Jc = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while (Jc * (Jc + 1) / 2 > b) --Jc;
  while ((Jc + 1) * (Jc + 2) / 2 <= b) ++Jc;
  J = Jc;
  I = b - Jc * (Jc + 1) / 2;
}

template <int MODE, int FORM>
__global__ void __launch_bounds__(TILE, 2)
segseg_tile_df(TileArgs A, typename PolDF<FORM>::Consts KP, const int64_t* __restrict__ rows, int64_t nRows,
               int64_t nJt, double* __restrict__ partial, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& sm = *reinterpret_cast<TileSmemT<TILE, PolDF<FORM>>*>(smem_raw);
  int64_t I, J;
  if (MODE == 0) {
    tile_index_df(blockIdx.x, I, J);
  } else {
    I = blockIdx.x / nJt;
    J = blockIdx.x % nJt;
  }
  tile_body<TILE, MODE, PolDF<FORM>>(A, KP, sm, I * TILE, J * TILE, MODE == 0 && I == J, rows, nRows,
                                     partial + (int64_t)blockIdx.x * (MODE == 0 ? 12 : 6) * TILE, counters);
}

KConstsDF to_df(const KConsts& K) {
  // Host-side split of the FP64 constants into (hi, lo) floats.
  auto s = [](double d) {
    float hi = (float)d;
    return df64{hi, (float)(d - (double)hi)};
  };
  return KConstsDF{s(K.aSq), s(K.mu4pi), s(K.mu4pinu), s(K.mu8piaSq), s(K.mu4pinuaSq)};
}

KConstsF to_f(const KConsts& K) {
  return KConstsF{(float)K.mu4pi, (float)K.mu4pinu, (float)K.mu8piaSq, (float)K.mu4pinuaSq};
}

bool g_attr_df[2][2] = {{false, false}, {false, false}};

template <int MODE, int FORM>
cudaError_t set_attr_df() {
  if (!g_attr_df[MODE][FORM]) {
    cudaError_t e = cudaFuncSetAttribute(segseg_tile_df<MODE, FORM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TileSmemT<TILE, PolDF<FORM>>));
    if (e != cudaSuccess) return e;
    g_attr_df[MODE][FORM] = true;
  }
  return cudaSuccess;
}

}  // namespace

size_t segseg_df_soa_bytes(int64_t npad) { return (size_t)npad * 26 * sizeof(float); }

cudaError_t launch_prep_df(const double* soa, int64_t npad, float* soadf, cudaStream_t st) {
  prep_df<<<(unsigned)((npad + 255) / 256), 256, 0, st>>>(soa, npad, soadf);
  return cudaGetLastError();
}

cudaError_t launch_segseg_all_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                 int64_t npad, double* partial, double* out, int64_t numSeg,
                                 unsigned long long* counters, cudaStream_t st, int form) {
  cudaError_t e = form ? set_attr_df<0, 1>() : set_attr_df<0, 0>();
  if (e != cudaSuccess) return e;
  const int64_t nt = npad / TILE;
  const int64_t nb = nt * (nt + 1) / 2;
  const TileArgs A{K, soa, skip, npad, soadf, nullptr};
  if (form)
    segseg_tile_df<0, 1><<<(unsigned)nb, TILE, sizeof(TileSmemT<TILE, PolDF<1>>), st>>>(
        A, PolDF<1>::Consts{to_df(K), to_f(K)}, nullptr, 0, 0, partial, counters);
  else
    segseg_tile_df<0, 0><<<(unsigned)nb, TILE, sizeof(TileSmemT<TILE, PolDF<0>>), st>>>(
        A, PolDF<0>::Consts{to_df(K), to_f(K)}, nullptr, 0, 0, partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return strict::launch_reduce_all(partial, npad, numSeg, out, st);
}

cudaError_t launch_segseg_rows_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                  int64_t npad, const int64_t* rows, int64_t nRows, double* partial, double* out,
                                  unsigned long long* counters, cudaStream_t st, int form) {
  cudaError_t e = form ? set_attr_df<1, 1>() : set_attr_df<1, 0>();
  if (e != cudaSuccess) return e;
  const int64_t nJt = npad / TILE;
  const int64_t nrt = (nRows + TILE - 1) / TILE;
  const unsigned grid = (unsigned)(nrt * nJt);
  const TileArgs A{K, soa, skip, npad, soadf, nullptr};
  if (form)
    segseg_tile_df<1, 1><<<grid, TILE, sizeof(TileSmemT<TILE, PolDF<1>>), st>>>(
        A, PolDF<1>::Consts{to_df(K), to_f(K)}, rows, nRows, nJt, partial, counters);
  else
    segseg_tile_df<1, 0><<<grid, TILE, sizeof(TileSmemT<TILE, PolDF<0>>), st>>>(
        A, PolDF<0>::Consts{to_df(K), to_f(K)}, rows, nRows, nJt, partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return strict::launch_reduce_rows(partial, npad, nRows, out, st);
}

}  // namespace ddd
