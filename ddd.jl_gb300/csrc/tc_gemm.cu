// Tensor-core GEMM on tcgen05: D[M x N] (FP32) = A[M x K] * B[N x K]^T, A and B
// both BF16 or both F16 (the instruction descriptor carries the type), row-major
// with K contiguous (both operands K-major), M a multiple of 128,
// N a multiple of 16 up to 256, K a multiple of 16.  The building block of the
// surrogate's training and inference; one CTA (4 warps) per 128-row block.
//
// Per K chunk of up to 64: all threads stage A and B into shared memory in the
// no-swizzle core-matrix layout (16-byte vector copies), fence the writes to
// the async proxy, one thread issues the MMAs (K = 16 each) into the TMEM
// accumulator and commits them to an mbarrier, everyone waits (bounded) before
// the next chunk overwrites the operands.  The epilogue reads the accumulator
// lanes with tcgen05.ld (warp w owns rows 32w..32w+31) and stores FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "tc_util.cuh"

namespace ddd {

namespace {

constexpr int KC = 64;

__global__ void __launch_bounds__(128, 1)
tc_gemm_tn(int M, int N, int K, const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
           float* __restrict__ D, int* __restrict__ err, uint32_t idesc) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;                 // 128 x KC 16-bit
  unsigned char* sB = smem + 128 * KC * 2;  // N x KC 16-bit
  __shared__ uint64_t mbar;
  __shared__ uint32_t s_taddr;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int m0 = blockIdx.x * 128;
  uint32_t ncols = 32;
  while ((int)ncols < N) ncols <<= 1;

  if (warp == 0) tc::tmem_alloc(&s_taddr, ncols);
  if (t == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = s_taddr;
  uint32_t phase = 0;
  bool ok = true;

  for (int k0 = 0; k0 < K && ok; k0 += KC) {
    const int kc = min(KC, K - k0);
    // Stage A rows m0..m0+127 and all N rows of B for columns k0..k0+kc-1.
    const int vecPerRow = kc / 8;
    for (int idx = t; idx < 128 * vecPerRow; idx += 128) {
      const int r = idx / vecPerRow, kb = idx % vecPerRow;
      const uint4 v = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + kb * 8);
      *reinterpret_cast<uint4*>(sA + tc::kmajor_offset(r, kb * 8, kc)) = v;
    }
    for (int idx = t; idx < N * vecPerRow; idx += 128) {
      const int r = idx / vecPerRow, kb = idx % vecPerRow;
      const uint4 v = *reinterpret_cast<const uint4*>(B + (size_t)r * K + k0 + kb * 8);
      *reinterpret_cast<uint4*>(sB + tc::kmajor_offset(r, kb * 8, kc)) = v;
    }
    tc::fence_async_smem();
    __syncthreads();
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t aBase = tc::smem_addr(sA), bBase = tc::smem_addr(sB);
      const uint32_t sbo = (uint32_t)(kc / 8) * 128u;
      for (int kk = 0; kk < kc; kk += 16) {
        const uint64_t ad = tc::smem_desc(aBase + (uint32_t)(kk / 8) * 128u, 128u, sbo);
        const uint64_t bd = tc::smem_desc(bBase + (uint32_t)(kk / 8) * 128u, 128u, sbo);
        tc::mma_bf16(taddr, ad, bd, idesc, (k0 > 0 || kk > 0) ? 1u : 0u);
      }
      tc::mma_commit(&mbar);
    }
    // Every thread leaves with the same verdict: a thread whose wait ran out
    // makes the whole CTA stop.
    ok = __syncthreads_and(tc::mbar_wait(&mbar, phase)) != 0;
    phase ^= 1u;
    tc::fence_after_sync();
  }

  if (ok) {
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(size_t)row * N + c0 + i] = v[i];
    }
  } else {
    if (t == 0) atomicExch(err, 1);
    // The MMAs of the abandoned chunk may still be writing these TMEM columns:
    // an MMA retires only through its commit's arrival on the mbarrier, so wait
    // (bounded again) for that arrival before the columns are freed.  If this
    // wait also runs out, the columns are freed anyway: a CTA must release its
    // TMEM before it exits.
    tc::mbar_wait(&mbar, phase ^ 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, ncols);
}

// Self-test of the bounded mbarrier wait that every tcgen05 kernel here uses:
// one warp, one mbarrier expecting one arrival.  With arrive != 0 thread 0
// arrives before the wait (the wait must succeed); with arrive == 0 nothing
// ever arrives, so every thread's wait runs out after max_clocks SM clocks and
// the kernel records the timeout in *err and returns.  No MMA is issued and no
// TMEM is held, so nothing is left in flight when the wait gives up.
__global__ void bounded_wait_probe(long long max_clocks, int arrive, int* __restrict__ err) {
  __shared__ uint64_t mbar;
  if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncwarp();
  if (arrive && threadIdx.x == 0) {
    uint64_t state;
    asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(tc::smem_addr(&mbar)) : "memory");
    (void)state;
  }
  const bool ok = tc::mbar_wait(&mbar, 0u, max_clocks);
  if (!ok) atomicExch(err, 1);
}

}  // namespace

cudaError_t launch_bounded_wait_probe(long long max_clocks, int arrive, int* err, cudaStream_t st) {
  bounded_wait_probe<<<1, 32, 0, st>>>(max_clocks, arrive, err);
  return cudaGetLastError();
}

size_t tc_gemm_smem_bytes(int N) { return (size_t)(128 + N) * KC * 2; }

static cudaError_t launch_tc_gemm(int M, int N, int K, const void* A, const void* B, float* D, int* err,
                                  cudaStream_t st, bool f16) {
  const int smem = (int)tc_gemm_smem_bytes(N);
  static std::atomic<uint64_t> attr{0};
  cudaError_t e = set_smem_once(tc_gemm_tn, 64 * 1024, attr);
  if (e != cudaSuccess) return e;
  tc_gemm_tn<<<M / 128, 128, smem, st>>>(M, N, K, (const uint16_t*)A, (const uint16_t*)B, D, err,
                                         tc::idesc_f32acc(128, N, f16));
  return cudaGetLastError();
}

cudaError_t launch_tc_gemm_bf16(int M, int N, int K, const void* A, const void* B, float* D, int* err,
                                cudaStream_t st) {
  return launch_tc_gemm(M, N, K, A, B, D, err, st, false);
}

cudaError_t launch_tc_gemm_f16(int M, int N, int K, const void* A, const void* B, float* D, int* err,
                               cudaStream_t st) {
  return launch_tc_gemm(M, N, K, A, B, D, err, st, true);
}

}  // namespace ddd
