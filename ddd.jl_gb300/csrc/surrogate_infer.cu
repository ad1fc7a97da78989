// Fused inference of the far-field surrogate over tile pairs.
//
// A persistent CTA (one per SM, 3 warpgroups = 384 threads) takes tile pairs
// (I <= J, 128 sorted segments a side) from a work list.  The MLP weights (FP16,
// 96 KB) stay in shared memory for the CTA's lifetime; each warpgroup has its
// own 32 KB activation buffer, its own 128 TMEM columns and its own mbarrier, so
// the warpgroups run independent layer pipelines and the tensor core works on
// one warpgroup's layer while the others run their epilogues.
//
// Warpgroup g handles the steps k = g, g + 3, ... of the tile pair.  At step k
// thread t forms pair (row t, column (t + k) mod 128), writes its 8 geometric
// features (hi and lo FP16 parts) as row t of a 128 x 16 FP16 operand, and the
// layer chain runs as
//   X (128x16) [W1|W1]^T -> TMEM (128x128 FP32) -> +b1, 2 GELU (two per
//   instruction), FP16 -> H (smem)
//   H (W2/2)^T -> TMEM -> ... -> H (W3/2)^T -> TMEM -> ... -> H (W4/2)^T -> TMEM
// The activations are stored doubled (x (1 + tanh(.)), one instruction fewer
// than 0.5 x (1 + tanh(.))) and W2..W4 are staged halved: both scalings are by
// a power of two, so every product, and every accumulator, is bit-identical to
// the plain GELU with the plain weights (weights below FP16's normal range
// excepted, which lose their last bit).
// one thread issuing the tcgen05.mma instructions, the warpgroup waiting on its
// mbarrier (bounded), each thread reading back its own accumulator row
// (tcgen05.ld) for the epilogue.  The 108 coefficients, contracted with the
// pair's Burgers-vector products, give the 12 scaled outputs, which become the
// pair's four node forces in the global frame.  Pairs outside the trust region (pair_is_far
// false), inactive segments and the lower half of diagonal tiles produce zero
// force here; the exact pass adds the near pairs afterwards.
//
// Row forces accumulate in registers, column forces in per-warpgroup shared
// arrays (the lanes of a warpgroup never share a column at one step); at the end
// of the tile pair the four warpgroups' sums are added in a fixed order and
// written, as doubles, to the tile pair's slot in the same [side][component][T]
// layout as the exact tile kernels.  No floating-point atomics.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "surrogate.cuh"
#include "tc_util.cuh"

using namespace ddd::sur;

namespace ddd {
namespace {

constexpr int TT = 128;  // tile size (segments)
constexpr int NWG = 3;   // warpgroups per CTA
constexpr int kThreads = NWG * 128;
// Shared-memory layout (bytes).  The X operand of a step (128 x 16 FP16) sits
// at the start of the warpgroup's H buffer: layer 1 has read it before the
// first epilogue overwrites it.
constexpr int kW1 = 0;                            // 128 x 16 FP16, K-major
constexpr int kW2 = kW1 + kHidden * kFeatIn * 2;  // 128 x 128
constexpr int kW3 = kW2 + kHidden * kHidden * 2;  // 128 x 128
constexpr int kW4 = kW3 + kHidden * kHidden * 2;  // 112 x 128
constexpr int kHBytes = TT * kHidden * 2;
constexpr int kH = kW4 + kOut * kHidden * 2;             // NWG x (128 x 128)
constexpr int kJ = kH + NWG * kHBytes;                   // kMsRows x 128 FP32 column-tile data
constexpr int kFJ = kJ + kMsRows * TT * 4;               // NWG x 6 x 128 FP32 column forces
constexpr int kBias = kFJ + NWG * 6 * TT * 4;            // b1, b2, b3 (128 each), b4 (112)
constexpr int kSmem = kBias + (3 * kHidden + kOut) * 4;  // 212,928 B
static_assert(kSmem <= 227 * 1024, "shared memory");
static_assert(6 * TT * 4 <= kHBytes, "row-sum staging fits in one H buffer");

// Per-segment data of the surrogate from the sorted FP64 SoA (13 rows: n1 xyz,
// n2 xyz, b xyz, t xyz, 1/|l|) and its skip flags.
__global__ void prep_mlp_seg(const double* __restrict__ soa, const uint8_t* __restrict__ skip, int64_t npad,
                             float* __restrict__ ms) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= npad) return;
  const bool sk = skip[i] != 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ms[(kMsM + k) * npad + i] = (float)(0.5 * (soa[k * npad + i] + soa[(3 + k) * npad + i]));
    ms[(kMsT + k) * npad + i] = (float)soa[(9 + k) * npad + i];
    ms[(kMsB + k) * npad + i] = (float)soa[(6 + k) * npad + i];
  }
  ms[kMsL * npad + i] = sk ? 0.0f : (float)(1.0 / soa[12 * npad + i]);
}

__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

// Barrier over the warpgroup that also returns whether `v` holds on all its threads.
__device__ __forceinline__ bool wg_all(bool v, int id) {
  uint32_t r;
  asm volatile(
      "{\n"
      ".reg .pred p, q;\n"
      "setp.ne.u32 q, %1, 0;\n"
      "bar.red.and.pred p, %2, 128, q;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16};"
      :
      : "r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
        "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Columns c..c+15 of the thread's accumulator row set to bias[c..c+15]: the
// next layer's MMAs then accumulate onto its bias.
__device__ __forceinline__ void bias_to_tmem(uint32_t tm_row, const float* bias, int c) {
  uint32_t v[16];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 b = *reinterpret_cast<const float4*>(bias + c + 4 * i);
    v[4 * i] = __float_as_uint(b.x);
    v[4 * i + 1] = __float_as_uint(b.y);
    v[4 * i + 2] = __float_as_uint(b.z);
    v[4 * i + 3] = __float_as_uint(b.w);
  }
  tmem_st16(tm_row + (uint32_t)c, v);
}

// 16 FP16 values (8 packed pairs) of row `row`, columns c0..c0+15, of a K-major tile.
__device__ __forceinline__ void store_h16(unsigned char* base, int row, int c0, int KC, const __half2* p) {
  *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, c0, KC)) = *reinterpret_cast<const uint4*>(&p[0]);
  *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, c0 + 8, KC)) = *reinterpret_cast<const uint4*>(&p[4]);
}

// The layer's MMAs (one thread of the warpgroup issues them) and the wait for
// their completion; false (on every thread of the warpgroup) if the wait ran out.
__device__ __forceinline__ bool layer(uint32_t tm, const unsigned char* A, const unsigned char* B, int K, int N,
                                      uint64_t* mbar, uint32_t& phase, bool leader, int bar) {
  tc::fence_async_smem();
  tc::fence_before_sync();
  wg_sync(bar);
  if (leader) {
    tc::fence_after_sync();
    const uint32_t a = tc::smem_addr(A), b = tc::smem_addr(B);
    const uint32_t sbo = (uint32_t)(K / 8) * 128u;
    const uint32_t idesc = tc::idesc_f16_f32(128, N);  // A and B both FP16
    for (int kk = 0; kk < K; kk += 16)  // onto the bias already in TMEM
      tc::mma_bf16(tm, tc::smem_desc(a + (uint32_t)(kk / 8) * 128u, 128u, sbo),
                   tc::smem_desc(b + (uint32_t)(kk / 8) * 128u, 128u, sbo), idesc, 1u);
    tc::mma_commit(mbar);
  }
  bool ok = tc::mbar_wait(mbar, phase);
  ok = wg_all(ok, bar);
  phase ^= 1u;
  tc::fence_after_sync();
  return ok;
}

// Row t of the warpgroup's 128-column accumulator (the layer's bias included:
// the MMAs accumulated onto it), GELU on FP16 pairs, into H (FP16).  As each
// 32-column chunk is read, the next layer's bias (nNext columns) takes its
// place.  32 columns per tcgen05.wait::ld (64 measured 10% slower: register
// pressure).
__device__ __forceinline__ void hidden_epilogue(uint32_t tm_row, const float* biasNext, int nNext, unsigned char* H,
                                                int t) {
#pragma unroll 1
  for (int c0 = 0; c0 < kHidden; c0 += 32) {
    uint32_t r[32];
    tmem_ld16_async(tm_row + (uint32_t)c0, r);
    tmem_ld16_async(tm_row + (uint32_t)c0 + 16u, r + 16);
    tmem_wait_ld();
    __half2 h[16];
#pragma unroll
    for (int i = 0; i < 16; ++i)
      h[i] = gelu2_h2(__floats2half2_rn(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1])));
    store_h16(H, t, c0, kHidden, h);
    store_h16(H, t, c0 + 16, kHidden, h + 8);
    if (c0 < nNext) bias_to_tmem(tm_row, biasNext, c0);
    if (c0 + 16 < nNext) bias_to_tmem(tm_row, biasNext, c0 + 16);
  }
  tmem_wait_st();
}

__global__ void __launch_bounds__(kThreads, 1)
mlp_far_tiles(const float* __restrict__ ms, int64_t npad, const int4* __restrict__ items, int32_t nItems,
              int32_t* __restrict__ next, const __half* __restrict__ W1, const __half* __restrict__ W2,
              const __half* __restrict__ W3, const __half* __restrict__ W4,
              const float* __restrict__ params, float mu4pi, float kappa2, double* __restrict__ partial,
              int32_t* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t mbar[NWG];
  __shared__ uint32_t s_tm;
  __shared__ int32_t s_item;
  const int tid = threadIdx.x, wg = tid >> 7, t = tid & 127, q = t >> 5;
  const int bar = 1 + wg;  // named barrier of the warpgroup (0 is __syncthreads)
  const bool leader = t == 0;
  float* sJ = reinterpret_cast<float*>(smem + kJ);
  float* sFJ = reinterpret_cast<float*>(smem + kFJ) + wg * 6 * TT;
  float* sBias = reinterpret_cast<float*>(smem + kBias);
  unsigned char* H = smem + kH + wg * kHBytes;

  // Weights (K-major core-matrix layout) and biases into shared memory, once.
  auto stage = [&](const __half* W, int rows, int K, int off, bool halve) {
    const __half2 hf = __float2half2_rn(0.5f);
    for (int idx = tid; idx < rows * (K / 8); idx += kThreads) {
      const int r = idx / (K / 8), kb = idx % (K / 8);
      uint4 v = *reinterpret_cast<const uint4*>(W + (size_t)r * K + kb * 8);
      if (halve) {
        __half2* h = reinterpret_cast<__half2*>(&v);
#pragma unroll
        for (int q2 = 0; q2 < 4; ++q2) h[q2] = __hmul2(h[q2], hf);
      }
      *reinterpret_cast<uint4*>(smem + off + tc::kmajor_offset(r, kb * 8, K)) = v;
    }
  };
  stage(W1, kHidden, kFeatIn, kW1, false);
  stage(W2, kHidden, kHidden, kW2, true);
  stage(W3, kHidden, kHidden, kW3, true);
  stage(W4, kOut, kHidden, kW4, true);
  for (int i = tid; i < kHidden; i += kThreads) {
    sBias[i] = params[kOffB1 + i];
    sBias[kHidden + i] = params[kOffB2 + i];
    sBias[2 * kHidden + i] = params[kOffB3 + i];
  }
  if (tid < kOut) sBias[3 * kHidden + tid] = params[kOffB4 + tid];
  if (tid < 32) tc::tmem_alloc(&s_tm, 512);
  if (tid == 0)
    for (int g = 0; g < NWG; ++g) tc::mbar_init(&mbar[g], 1);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = s_tm + (uint32_t)(wg * kHidden);      // this warpgroup's columns
  const uint32_t tm_row = tm + ((uint32_t)(q * 32) << 16);  // this warp's lanes
  uint32_t phase = 0;
  bool ok = true;
  bool pending = false;  // this warpgroup's last commit did not arrive in time
  for (int c = 0; c < kHidden; c += 16) bias_to_tmem(tm_row, sBias, c);  // layer 1 of the first step
  tmem_wait_st();

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int32_t w = s_item;
    if (w >= nItems) break;
    const int4 it = items[w];
    const int64_t i0 = it.y, j0 = it.z;
    const bool diag = it.w != 0;
    for (int idx = tid; idx < kMsRows * TT; idx += kThreads) sJ[idx] = ms[(idx / TT) * npad + j0 + (idx % TT)];
#pragma unroll
    for (int c = 0; c < 6; ++c) sFJ[c * TT + t] = 0.0f;
    float mi[3], ti[3], bi[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      mi[r] = ms[(kMsM + r) * npad + i0 + t];
      ti[r] = ms[(kMsT + r) * npad + i0 + t];
      bi[r] = ms[(kMsB + r) * npad + i0 + t];
    }
    const float Li = ms[kMsL * npad + i0 + t];
    float fi[6] = {0, 0, 0, 0, 0, 0};
    __syncthreads();

    for (int k = wg; k < TT; k += NWG) {
      const int jl = (t + k) & (TT - 1);
      float f[kGeo], bp[kBProd];
      Frame fr;
      float r[3];
      const bool far = pair_is_far(mi[0], mi[1], mi[2], Li, sJ[(kMsM + 0) * TT + jl], sJ[(kMsM + 1) * TT + jl],
                                   sJ[(kMsM + 2) * TT + jl], sJ[kMsL * TT + jl], kappa2, r[0], r[1], r[2]);
      if (far && (!diag || jl > t)) {
        const float tj[3] = {sJ[(kMsT + 0) * TT + jl], sJ[(kMsT + 1) * TT + jl], sJ[(kMsT + 2) * TT + jl]};
        const float bj[3] = {sJ[(kMsB + 0) * TT + jl], sJ[(kMsB + 1) * TT + jl], sJ[(kMsB + 2) * TT + jl]};
        pair_features(r, ti, tj, bi, bj, Li, sJ[kMsL * TT + jl], mu4pi, f, bp, fr);
      } else {
#pragma unroll
        for (int c = 0; c < kGeo; ++c) f[c] = 0.0f;
#pragma unroll
        for (int c = 0; c < kBProd; ++c) bp[c] = 0.0f;
        fr.scale = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) fr.e1[c] = fr.e2[c] = fr.e3[c] = 0.0f;
      }
      float row[kFeatIn];
      split_features(f, row);
      __half2 x[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) x[i] = __floats2half2_rn(row[2 * i], row[2 * i + 1]);
      store_h16(H, t, 0, kFeatIn, x);

      if (!(ok = layer(tm, H, smem + kW1, kFeatIn, kHidden, &mbar[wg], phase, leader, bar))) {
        pending = true;
        break;
      }
      hidden_epilogue(tm_row, sBias + kHidden, kHidden, H, t);
      if (!(ok = layer(tm, H, smem + kW2, kHidden, kHidden, &mbar[wg], phase, leader, bar))) {
        pending = true;
        break;
      }
      hidden_epilogue(tm_row, sBias + 2 * kHidden, kHidden, H, t);
      if (!(ok = layer(tm, H, smem + kW3, kHidden, kHidden, &mbar[wg], phase, leader, bar))) {
        pending = true;
        break;
      }
      hidden_epilogue(tm_row, sBias + 3 * kHidden, kOut, H, t);
      if (!(ok = layer(tm, H, smem + kW4, kHidden, kOut, &mbar[wg], phase, leader, bar))) {
        pending = true;
        break;
      }
      // Contraction: out[o] = sum_ac bp[ac] Y[12 ac + o] (Y includes b4); then
      // b1 into the columns for the next step's first layer.
      float out[kUsedOut];
#pragma unroll
      for (int o = 0; o < kUsedOut; ++o) out[o] = 0.0f;
#pragma unroll
      for (int c0 = 0; c0 < kCoef; c0 += 16) {
        uint32_t yr[16];
        tmem_ld16_async(tm_row + (uint32_t)c0, yr);
        tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int j = c0 + i;
          if (j < kCoef) out[j % kUsedOut] += bp[j / kUsedOut] * __uint_as_float(yr[i]);
        }
      }
#pragma unroll 1
      for (int c = 0; c < kHidden; c += 16) bias_to_tmem(tm_row, sBias, c);
      tmem_wait_st();
      float F[12];
#pragma unroll
      for (int n = 0; n < 4; ++n) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          F[3 * n + c] = fr.scale * (out[3 * n] * fr.e1[c] + out[3 * n + 1] * fr.e2[c] + out[3 * n + 2] * fr.e3[c]);
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) fi[c] += F[c];
#pragma unroll
      for (int c = 0; c < 6; ++c) sFJ[c * TT + jl] += F[6 + c];
    }
    tc::fence_before_sync();
    // Every warpgroup leaves the step loop with the same `ok`; agree across the CTA.
    if (__syncthreads_or(!ok)) {
      ok = false;
      break;
    }
    // Row sums: each warpgroup's per-row values into its (idle) H buffer, then a
    // fixed-order sum over the warpgroups.
    float* sFI = reinterpret_cast<float*>(H);
#pragma unroll
    for (int c = 0; c < 6; ++c) sFI[c * TT + t] = fi[c];
    __syncthreads();
    double* p = partial + (int64_t)it.x * 12 * TT;
    if (wg < 2) {
      // warpgroup 0: row forces, warpgroup 1: column forces
      const int side = wg;
      for (int c = 0; c < 6; ++c) {
        double v = 0.0;
#pragma unroll
        for (int g = 0; g < NWG; ++g) {
          const float* src = side == 0 ? reinterpret_cast<const float*>(smem + kH + g * kHBytes)
                                       : reinterpret_cast<const float*>(smem + kFJ) + g * 6 * TT;
          v += (double)src[c * TT + t];
        }
        p[(6 * side + c) * TT + t] = v;
      }
    }
  }
  if (!ok && tid == 0) atomicExch(err, 1);
  // A warpgroup whose wait ran out may still have MMAs writing its TMEM
  // columns; they retire only through the commit's arrival on its mbarrier
  // (the phase `layer` already stepped past), so wait for it, bounded again,
  // before the CTA frees the columns.  If that wait also runs out the columns
  // are freed anyway: a CTA must release its TMEM before it exits.
  if (pending) tc::mbar_wait(&mbar[wg], phase ^ 1u);
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(s_tm, 512);
}

}  // namespace

size_t mlp_seg_bytes(int64_t npad) { return (size_t)npad * kMsRows * sizeof(float); }

cudaError_t launch_prep_mlp_seg(const double* soa, const uint8_t* skip, int64_t npad, float* ms, cudaStream_t st) {
  prep_mlp_seg<<<(unsigned)((npad + 255) / 256), 256, 0, st>>>(soa, skip, npad, ms);
  return cudaGetLastError();
}

cudaError_t prepare_mlp_far_tiles() {
  static std::atomic<uint64_t> attr{0};
  return set_smem_once(mlp_far_tiles, kSmem, attr);
}

cudaError_t launch_mlp_far_tiles(const float* ms, int64_t npad, const int4* items, int32_t nItems, int32_t* next,
                                 const void* const* W, const float* params, float mu4pi, float kappa2,
                                 double* partial, int32_t* err, int grid, cudaStream_t st) {
  cudaError_t e = prepare_mlp_far_tiles();
  if (e != cudaSuccess) return e;
  if (nItems <= 0) return cudaSuccess;
  mlp_far_tiles<<<grid, kThreads, kSmem, st>>>(ms, npad, items, nItems, next, (const __half*)W[0],
                                               (const __half*)W[1], (const __half*)W[2], (const __half*)W[3],
                                               params, mu4pi, kappa2, partial, err);
  return cudaGetLastError();
}

}  // namespace ddd
