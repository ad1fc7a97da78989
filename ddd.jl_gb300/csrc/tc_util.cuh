// Blackwell (sm_100-family) tensor-core primitives as inline PTX: TMEM
// allocation, tcgen05.mma (kind::f16, BF16 or F16 inputs, FP32 accumulators in TMEM),
// commit to an mbarrier, bounded mbarrier waits, tcgen05.ld of accumulators.
//
// Operand staging: K-major tiles without swizzle, built from 8 x 16-byte "core
// matrices" (8 rows x 8 BF16).  Element (row r, k) of a tile with KC columns
// lives at byte ((r/8)*(KC/8) + k/8)*128 + (r%8)*16 + (k%8)*2, so core matrices
// adjacent in K are 128 B apart (the descriptor's leading-dimension offset) and
// core matrices adjacent in M/N are (KC/8)*128 B apart (its stride offset).
//
// Every wait is bounded: on timeout the caller records an error and returns,
// after releasing its TMEM columns.
#pragma once
#include <cstdint>

namespace ddd {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, k) in a K-major no-swizzle tile with KC columns.
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int KC) {
  return (uint32_t)((((r >> 3) * (KC >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (all >> 4), the fixed version bits 46-48 =
// 0b001, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A and B both BF16 (or both F16
// with f16 = true; the two operands always share one type), both K-major,
// dense, shape M x N (M = 128 here, N multiple of 16 up to 256).
__host__ __device__ __forceinline__ uint32_t idesc_f32acc(int M, int N, bool f16) {
  uint32_t d = 0;
  d |= 1u << 4;                        // D format: F32
  if (!f16) d |= (1u << 7) | (1u << 10);  // A and B format: BF16 (F16 = 0)
  d |= (uint32_t)(N >> 3) << 17;       // N / 8
  d |= (uint32_t)(M >> 4) << 24;       // M / 16
  return d;
}
__host__ __device__ __forceinline__ uint32_t idesc_bf16_f32(int M, int N) { return idesc_f32acc(M, N, false); }
__host__ __device__ __forceinline__ uint32_t idesc_f16_f32(int M, int N) { return idesc_f32acc(M, N, true); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Makes this thread's shared-memory writes visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// The operand type is in idesc; the instruction is the same for BF16 and F16.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.u32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on the mbarrier when all previously issued MMAs of this thread complete.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}

// Waits for the phase with the given parity to complete; false once about two
// seconds (4e9 SM clocks) have passed without it.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, long long max_clocks = 4000000000LL) {
  const uint32_t a = smem_addr(mbar);
  const long long start = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - start > max_clocks) return false;
  }
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace ddd
