// The fast FP64 form of the all-pairs and index-list seg-seg force
// (DDD_MODE_FP64_FAST): the FP64 kernel's tiles, schedule, near-parallel
// compaction and deterministic reduction (tile_body.cuh, segseg_f64.cu) with
// the general branch of pair_f64fast.cuh — one division per corner instead of
// four, logarithms and arctangents in integer fixed point on the integer pipes
// (intmath_f64.cuh, off the FP64 pipe), explicit fused multiply-adds
// where the reference's terms do not cancel.  The near-parallel branch, the
// branch decision and the segment preparation stay the strict FP64 code.
//
// Compiled with --fmad=false: every fusion is the explicit one of
// pair_f64fast.cuh, so a host build of that header gives the same bits, and
// the near-parallel branch rounds as the strict kernel does.
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_f64.cuh"
#include "tile_pol_fx.cuh"

namespace ddd {

namespace {

constexpr int TILE = 128;

__device__ __forceinline__ void tile_index_fx(int64_t b, int64_t& I, int64_t& J) {
  int64_t Jc = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while (Jc * (Jc + 1) / 2 > b) --Jc;
  while ((Jc + 1) * (Jc + 2) / 2 <= b) ++Jc;
  J = Jc;
  I = b - Jc * (Jc + 1) / 2;
}

// MODE 0: all pairs, one CTA per tile pair I <= J of the band starting at slot
// `base`; MODE 1: index rows, one CTA per (row tile, column tile).
template <int MODE>
__global__ void __launch_bounds__(TILE, 2)
segseg_tile_fx(TileArgs A, const int64_t* __restrict__ rows, int64_t nRows, int64_t nJt, int64_t base,
               double* __restrict__ partial, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& sm = *reinterpret_cast<TileSmemT<TILE, PolF64Fast>*>(smem_raw);
  int64_t I, J;
  if (MODE == 0) {
    tile_index_fx(base + blockIdx.x, I, J);
  } else {
    I = blockIdx.x / nJt;
    J = blockIdx.x % nJt;
  }
  tile_body<TILE, MODE, PolF64Fast>(A, PolF64Fast::Consts{}, sm, I * TILE, J * TILE, MODE == 0 && I == J, rows,
                                    nRows, partial + (int64_t)blockIdx.x * (MODE == 0 ? 12 : 6) * TILE, counters);
}

template <int MODE>
cudaError_t set_attr_fx() {
  static std::atomic<uint64_t> done{0};
  return set_smem_once(segseg_tile_fx<MODE>, (int)sizeof(TileSmemT<TILE, PolF64Fast>), done);
}

}  // namespace

cudaError_t launch_segseg_all_fx(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                 double* partial, double* out, int64_t numSeg, unsigned long long* counters,
                                 cudaStream_t st, int64_t capSlots) {
  cudaError_t e = set_attr_fx<0>();
  if (e != cudaSuccess) return e;
  const int64_t nt = npad / TILE;
  const int64_t nb = nt * (nt + 1) / 2;
  const TileArgs A{K, soa, skip, npad, nullptr, nullptr};
  // One launch over all slots, or (partial sums larger than capSlots slots)
  // bands of J columns in order, each reduced into the running output.
  for (int64_t J0 = 0; J0 < nt;) {
    const int64_t J1 = capSlots >= nb ? nt : strict::segseg_band_end(J0, nt, capSlots);
    const int64_t b0 = J0 * (J0 + 1) / 2, nbb = J1 * (J1 + 1) / 2 - b0;
    segseg_tile_fx<0><<<(unsigned)nbb, TILE, sizeof(TileSmemT<TILE, PolF64Fast>), st>>>(A, nullptr, 0, 0, b0,
                                                                                         partial, counters);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = capSlots >= nb ? strict::launch_reduce_all(partial, npad, numSeg, out, st)
                       : strict::launch_reduce_band(partial, J0, J1, numSeg, out, st);
    if (e != cudaSuccess) return e;
    J0 = J1;
  }
  return cudaSuccess;
}

cudaError_t launch_segseg_rows_fx(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                  const int64_t* rows, int64_t nRows, double* partial, double* out,
                                  unsigned long long* counters, cudaStream_t st) {
  cudaError_t e = set_attr_fx<1>();
  if (e != cudaSuccess) return e;
  const int64_t nJt = npad / TILE;
  const int64_t nrt = (nRows + TILE - 1) / TILE;
  const TileArgs A{K, soa, skip, npad, nullptr, nullptr};
  segseg_tile_fx<1><<<(unsigned)(nrt * nJt), TILE, sizeof(TileSmemT<TILE, PolF64Fast>), st>>>(A, rows, nRows, nJt, 0,
                                                                                              partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return strict::launch_reduce_rows(partial, npad, nRows, out, st);
}

}  // namespace ddd
