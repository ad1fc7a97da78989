// FP64 seg–seg force kernels (the plain, reference-matching method).
//
// Data layout in HBM (built by prep_segments from the caller's network arrays):
//   SoA, 16 double arrays of length Npad = ceil(N / TILE) * TILE, in the order
//   n1x n1y n1z n2x n2y n2z bx by bz tx ty tz tN (13 used) + a uint8 skip flag
//   (extSeg or padding).  72 B/segment of caller data, 104 B packed.
//
// All-pairs (calcSegSegForce, DislocationForces.jl:719-829):
//   grid = one CTA per tile pair (I <= J) of TILE x TILE segments.  Thread t owns
//   segment i = I*TILE + t (registers); the J tile sits in shared memory.  At
//   step k thread t evaluates j = (t + k) mod TILE, so all threads of a warp touch
//   distinct j and the j-side forces accumulate race-free into a per-warp shared
//   array (no atomics).  Near-parallel pairs (1 - c^2 <= sqrt(eps)) are only
//   flagged in a per-thread bitmask during that sweep; afterwards the CTA
//   compacts them into a shared list (fixed order: by i, then by step) and
//   evaluates them densely, 128 at a time, so the ~5x-costlier branch does not
//   serialise warps.  The CTA writes its two partial force blocks (forces on the
//   I tile, forces on the J tile) to scratch; segseg_reduce sums them per segment
//   in a fixed order.  Everything is deterministic: same inputs, same bits.
// Index list (calcSegSegForce(..., idx), DislocationForces.jl:831-877):
//   same kernel with ROWS mode: row slots come from idx, every j != i is paired,
//   only Fnode1/Fnode2 are computed, partials per (row tile, J tile).
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_f64.cuh"
#include "tile_body.cuh"

// This file is compiled twice: DDD_VARIANT=strict with --fmad=false (every
// multiply and add rounded separately, as the reference's Julia code does) and
// DDD_VARIANT=fast with FMA contraction.
#ifndef DDD_VARIANT
#define DDD_VARIANT strict
#endif

namespace ddd {
namespace DDD_VARIANT {

constexpr int TILE = 128;

// ---------------------------------------------------------------------------
// Gather the caller's network arrays (Julia column-major, 1-based) into the
// packed SoA, with per-segment direction and inverse length.  Segments at or
// beyond numSeg (padding) and extSeg segments get skip = 1.
__global__ void prep_segments(const double* __restrict__ coord, const double* __restrict__ bVec,
                              const int64_t* __restrict__ segIdx, int64_t ld, const uint8_t* __restrict__ extSeg,
                              int64_t numSeg, int64_t npad, double* __restrict__ soa, uint8_t* __restrict__ skip) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= npad) return;
  double v[13];
  uint8_t sk = 1;
  if (i < numSeg) {
    int64_t l = segIdx[i] - 1, a = segIdx[i + ld] - 1, b = segIdx[i + 2 * ld] - 1;
    D3 n1 = {coord[3 * a], coord[3 * a + 1], coord[3 * a + 2]};
    D3 n2 = {coord[3 * b], coord[3 * b + 1], coord[3 * b + 2]};
    D3 bv = {bVec[3 * l], bVec[3 * l + 1], bVec[3 * l + 2]};
    D3 t;
    double tN;
    seg_direction(n1, n2, t, tN);
    v[0] = n1.x; v[1] = n1.y; v[2] = n1.z;
    v[3] = n2.x; v[4] = n2.y; v[5] = n2.z;
    v[6] = bv.x; v[7] = bv.y; v[8] = bv.z;
    v[9] = t.x; v[10] = t.y; v[11] = t.z; v[12] = tN;
    sk = extSeg ? (extSeg[i] ? 1 : 0) : 0;
  } else {
#pragma unroll
    for (int k = 0; k < 13; ++k) v[k] = 0.0;
    v[3] = 1.0;  // a unit-length dummy segment, never evaluated
    v[9] = 1.0;
    v[12] = 1.0;
  }
#pragma unroll
  for (int k = 0; k < 13; ++k) soa[k * npad + i] = v[k];
  skip[i] = sk;
}

// Device-resident variant: packed 9 x ld SoA (n1, n2, b) already on the GPU.
__global__ void prep_segments_packed(const double* __restrict__ in, int64_t ldIn, const uint8_t* __restrict__ extSeg,
                                     int64_t numSeg, int64_t npad, double* __restrict__ soa,
                                     uint8_t* __restrict__ skip) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= npad) return;
  double v[13];
  uint8_t sk = 1;
  if (i < numSeg) {
    D3 n1 = {in[i], in[ldIn + i], in[2 * ldIn + i]};
    D3 n2 = {in[3 * ldIn + i], in[4 * ldIn + i], in[5 * ldIn + i]};
    D3 bv = {in[6 * ldIn + i], in[7 * ldIn + i], in[8 * ldIn + i]};
    D3 t;
    double tN;
    seg_direction(n1, n2, t, tN);
    v[0] = n1.x; v[1] = n1.y; v[2] = n1.z;
    v[3] = n2.x; v[4] = n2.y; v[5] = n2.z;
    v[6] = bv.x; v[7] = bv.y; v[8] = bv.z;
    v[9] = t.x; v[10] = t.y; v[11] = t.z; v[12] = tN;
    sk = extSeg ? (extSeg[i] ? 1 : 0) : 0;
  } else {
#pragma unroll
    for (int k = 0; k < 13; ++k) v[k] = 0.0;
    v[3] = 1.0;
    v[9] = 1.0;
    v[12] = 1.0;
  }
#pragma unroll
  for (int k = 0; k < 13; ++k) soa[k * npad + i] = v[k];
  skip[i] = sk;
}

__device__ __forceinline__ void tile_index(int64_t b, int64_t& I, int64_t& J) {
  // b enumerates (I <= J) column by column: J-th column holds I = 0..J.
  int64_t Jc = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while (Jc * (Jc + 1) / 2 > b) --Jc;
  while ((Jc + 1) * (Jc + 2) / 2 <= b) ++Jc;
  J = Jc;
  I = b - Jc * (Jc + 1) / 2;
}

// MODE 0: all pairs (symmetric, i < j), one CTA per tile pair I <= J; the
//         launch covers slots base.. (a band of J columns), its partial blocks
//         indexed from base.
// MODE 1: index rows (all j != i, F12 only), one CTA per (row tile, column tile).
template <int MODE>
__global__ void __launch_bounds__(TILE, 2)
segseg_tile_f64(TileArgs A, const int64_t* __restrict__ rows, int64_t nRows, int64_t nJt, int64_t base,
                double* __restrict__ partial, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& sm = *reinterpret_cast<TileSmemT<TILE, PolF64>*>(smem_raw);
  int64_t I, J;
  if (MODE == 0) {
    tile_index(base + blockIdx.x, I, J);
  } else {
    I = blockIdx.x / nJt;
    J = blockIdx.x % nJt;
  }
  tile_body<TILE, MODE, PolF64>(A, PolF64::Consts{}, sm, I * TILE, J * TILE, MODE == 0 && I == J, rows, nRows,
                                partial + (int64_t)blockIdx.x * (MODE == 0 ? 12 : 6) * TILE, counters);
}

// Sum the partial blocks of each segment in a fixed order and write the
// segForce layout F[k + 3*(node + 2*s)].
// All-pairs: segment s in tile A collects row blocks (A, J) for J = A..nt-1,
// then column blocks (I, A) for I = 0..A.
__global__ void segseg_reduce_all(const double* __restrict__ partial, int64_t nt, int64_t numSeg,
                                  double* __restrict__ out) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= numSeg) return;
  const int64_t A = s / TILE;
  const int t = (int)(s % TILE);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t Jt = A; Jt < nt; ++Jt) {
    const int64_t b = Jt * (Jt + 1) / 2 + A;  // block index of (I=A, J=Jt)
    const double* p = partial + b * 12 * TILE;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[c * TILE + t];
  }
  for (int64_t It = 0; It <= A; ++It) {
    const int64_t b = A * (A + 1) / 2 + It;  // block index of (I=It, J=A)
    const double* p = partial + b * 12 * TILE;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[(6 + c) * TILE + t];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) out[6 * s + c] = acc[c];
}

// Banded all-pairs: one launch of the tile kernel covered the J columns
// [J0, J1), slots J0(J0+1)/2 .. J1(J1+1)/2 - 1, stored from the band's first
// slot.  Segment s in tile A < J1 adds its row blocks (A, J) for J in
// [max(A, J0), J1), then, when A lies in the band, its column blocks (I, A)
// for I = 0..A.  The band holding A starts the sum, later bands add to it: a
// fixed order, so the result is deterministic (it is the unbanded sum
// regrouped, equal to rounding).
__global__ void segseg_reduce_band(const double* __restrict__ partial, int64_t J0, int64_t J1, int64_t numSeg,
                                   double* __restrict__ out) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= numSeg) return;
  const int64_t A = s / TILE;
  if (A >= J1) return;
  const int t = (int)(s % TILE);
  const int64_t base = J0 * (J0 + 1) / 2;
  const bool first = A >= J0;
  double acc[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) acc[c] = first ? 0.0 : out[6 * s + c];
  for (int64_t Jt = first ? A : J0; Jt < J1; ++Jt) {
    const double* p = partial + (Jt * (Jt + 1) / 2 + A - base) * 12 * TILE;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[c * TILE + t];
  }
  if (first) {
    for (int64_t It = 0; It <= A; ++It) {
      const double* p = partial + (A * (A + 1) / 2 + It - base) * 12 * TILE;
#pragma unroll
      for (int c = 0; c < 6; ++c) acc[c] += p[(6 + c) * TILE + t];
    }
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) out[6 * s + c] = acc[c];
}

// Index rows: row r (slot in the idx list) collects its nJt column blocks.
__global__ void segseg_reduce_rows(const double* __restrict__ partial, int64_t nJt, int64_t nRows,
                                   double* __restrict__ out) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nRows) return;
  const int64_t A = r / TILE;
  const int t = (int)(r % TILE);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t Jt = 0; Jt < nJt; ++Jt) {
    const double* p = partial + (A * nJt + Jt) * 6 * TILE;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[c * TILE + t];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) out[6 * r + c] = acc[c];
}

// ---------------------------------------------------------------------------
// Host launchers.
int64_t segseg_npad(int64_t numSeg) { return ((numSeg + TILE - 1) / TILE) * TILE; }
size_t segseg_soa_bytes(int64_t npad) { return (size_t)npad * 13 * sizeof(double); }
size_t segseg_partial_bytes_all(int64_t npad) {
  int64_t nt = npad / TILE;
  return (size_t)(nt * (nt + 1) / 2) * 12 * TILE * sizeof(double);
}
size_t segseg_partial_bytes_rows(int64_t nRows, int64_t npad) {
  int64_t nrt = (nRows + TILE - 1) / TILE, nJt = npad / TILE;
  return (size_t)(nrt * nJt) * 6 * TILE * sizeof(double);
}

cudaError_t launch_prep_segments(const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld,
                                 const uint8_t* extSeg, int64_t numSeg, int64_t npad, double* soa, uint8_t* skip,
                                 cudaStream_t st) {
  prep_segments<<<(unsigned)((npad + 255) / 256), 256, 0, st>>>(coord, bVec, segIdx, ld, extSeg, numSeg, npad, soa,
                                                                skip);
  return cudaGetLastError();
}

cudaError_t launch_prep_segments_packed(const double* in, int64_t ldIn, const uint8_t* extSeg, int64_t numSeg,
                                        int64_t npad, double* soa, uint8_t* skip, cudaStream_t st) {
  prep_segments_packed<<<(unsigned)((npad + 255) / 256), 256, 0, st>>>(in, ldIn, extSeg, numSeg, npad, soa, skip);
  return cudaGetLastError();
}

template <int MODE>
static cudaError_t set_attr() {
  static std::atomic<uint64_t> done{0};
  return set_smem_once(segseg_tile_f64<MODE>, (int)sizeof(TileSmemT<TILE, PolF64>), done);
}

// Loads the all-pairs kernels on the current device (under lazy module loading
// the driver loads a kernel, and reserves its memory, at first use) and sets
// the tile kernel's shared-memory attribute, without launching anything.
cudaError_t preload_all_f64() {
  cudaError_t e = set_attr<0>();
  cudaFuncAttributes fa;
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, prep_segments_packed);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, segseg_reduce_all);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, segseg_reduce_band);
  return e;
}

cudaError_t launch_reduce_all(const double* partial, int64_t npad, int64_t numSeg, double* out, cudaStream_t st) {
  segseg_reduce_all<<<(unsigned)((numSeg + 127) / 128), 128, 0, st>>>(partial, npad / TILE, numSeg, out);
  return cudaGetLastError();
}

int64_t segseg_band_end(int64_t J0, int64_t nt, int64_t capSlots) {
  const int64_t b0 = J0 * (J0 + 1) / 2;
  int64_t J1 = J0 + 1;
  while (J1 < nt && (J1 + 1) * (J1 + 2) / 2 - b0 <= capSlots) ++J1;
  return J1;
}

cudaError_t launch_reduce_band(const double* partial, int64_t J0, int64_t J1, int64_t numSeg, double* out,
                               cudaStream_t st) {
  const int64_t n = numSeg < J1 * TILE ? numSeg : J1 * TILE;
  segseg_reduce_band<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(partial, J0, J1, n, out);
  return cudaGetLastError();
}

cudaError_t launch_reduce_rows(const double* partial, int64_t npad, int64_t nRows, double* out, cudaStream_t st) {
  segseg_reduce_rows<<<(unsigned)((nRows + 127) / 128), 128, 0, st>>>(partial, npad / TILE, nRows, out);
  return cudaGetLastError();
}

cudaError_t launch_segseg_all_f64(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                  double* partial, double* out, int64_t numSeg, unsigned long long* counters,
                                  cudaStream_t st, int64_t capSlots) {
  cudaError_t e = set_attr<0>();
  if (e != cudaSuccess) return e;
  const int64_t nt = npad / TILE;
  const int64_t nb = nt * (nt + 1) / 2;
  const TileArgs A{K, soa, skip, npad, nullptr, nullptr};
  if (capSlots >= nb) {
    segseg_tile_f64<0><<<(unsigned)nb, TILE, sizeof(TileSmemT<TILE, PolF64>), st>>>(A, nullptr, 0, 0, 0, partial,
                                                                                    counters);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    segseg_reduce_all<<<(unsigned)((numSeg + 127) / 128), 128, 0, st>>>(partial, nt, numSeg, out);
    return cudaGetLastError();
  }
  // Partial sums larger than capSlots slots: bands of J columns, in order.
  for (int64_t J0 = 0; J0 < nt;) {
    const int64_t J1 = segseg_band_end(J0, nt, capSlots);
    const int64_t b0 = J0 * (J0 + 1) / 2, nbb = J1 * (J1 + 1) / 2 - b0;
    segseg_tile_f64<0><<<(unsigned)nbb, TILE, sizeof(TileSmemT<TILE, PolF64>), st>>>(A, nullptr, 0, 0, b0, partial,
                                                                                     counters);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = launch_reduce_band(partial, J0, J1, numSeg, out, st);
    if (e != cudaSuccess) return e;
    J0 = J1;
  }
  return cudaSuccess;
}

cudaError_t launch_segseg_rows_f64(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                   const int64_t* rows, int64_t nRows, double* partial, double* out,
                                   unsigned long long* counters, cudaStream_t st) {
  cudaError_t e = set_attr<1>();
  if (e != cudaSuccess) return e;
  const int64_t nJt = npad / TILE;
  const int64_t nrt = (nRows + TILE - 1) / TILE;
  const TileArgs A{K, soa, skip, npad, nullptr, nullptr};
  segseg_tile_f64<1><<<(unsigned)(nrt * nJt), TILE, sizeof(TileSmemT<TILE, PolF64>), st>>>(A, rows, nRows, nJt, 0,
                                                                                           partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  segseg_reduce_rows<<<(unsigned)((nRows + 127) / 128), 128, 0, st>>>(partial, nJt, nRows, out);
  return cudaGetLastError();
}

}  // namespace DDD_VARIANT
}  // namespace ddd
