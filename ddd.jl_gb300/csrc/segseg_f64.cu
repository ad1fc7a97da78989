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

// This file is compiled twice: DDD_VARIANT=strict with --fmad=false (every
// multiply and add rounded separately, as the reference's Julia code does) and
// DDD_VARIANT=fast with FMA contraction.
#ifndef DDD_VARIANT
#define DDD_VARIANT strict
#endif

namespace ddd {
namespace DDD_VARIANT {

constexpr int TILE = 128;
constexpr int NWARP = TILE / 32;
constexpr int CHUNK = TILE;  // near-parallel pairs evaluated per round

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

__device__ __forceinline__ SegF64 load_seg_global(const double* __restrict__ soa, int64_t npad, int64_t i) {
  SegF64 s;
  s.n1 = {soa[i], soa[npad + i], soa[2 * npad + i]};
  s.n2 = {soa[3 * npad + i], soa[4 * npad + i], soa[5 * npad + i]};
  s.b = {soa[6 * npad + i], soa[7 * npad + i], soa[8 * npad + i]};
  s.t = {soa[9 * npad + i], soa[10 * npad + i], soa[11 * npad + i]};
  s.tN = soa[12 * npad + i];
  return s;
}

struct TileSmem {
  double seg[13][TILE];           // J tile, SoA
  double fj[NWARP][6][TILE];      // per-warp j-side forces
  double cf[CHUNK][12];           // near-parallel chunk results
  uint16_t plist[TILE * TILE];    // near-parallel list: (i_local << 8) | j_local
  int cnt[TILE];                  // near-parallel count per i thread (prefix-summed)
  uint8_t skip[TILE];
};

__device__ __forceinline__ SegF64 load_seg_smem(const TileSmem& sm, int j) {
  SegF64 s;
  s.n1 = {sm.seg[0][j], sm.seg[1][j], sm.seg[2][j]};
  s.n2 = {sm.seg[3][j], sm.seg[4][j], sm.seg[5][j]};
  s.b = {sm.seg[6][j], sm.seg[7][j], sm.seg[8][j]};
  s.t = {sm.seg[9][j], sm.seg[10][j], sm.seg[11][j]};
  s.tN = sm.seg[12][j];
  return s;
}

__device__ __forceinline__ void tile_index(int64_t b, int64_t& I, int64_t& J) {
  // b enumerates (I <= J) column by column: J-th column holds I = 0..J.
  int64_t Jc = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while (Jc * (Jc + 1) / 2 > b) --Jc;
  while ((Jc + 1) * (Jc + 2) / 2 <= b) ++Jc;
  J = Jc;
  I = b - Jc * (Jc + 1) / 2;
}

// MODE 0: all pairs (symmetric, i < j).  MODE 1: index rows (all j != i, F12 only).
template <int MODE>
__global__ void __launch_bounds__(TILE, 2)
segseg_tile_f64(KConsts K, const double* __restrict__ soa, const uint8_t* __restrict__ skipArr, int64_t npad,
                const int64_t* __restrict__ rows, int64_t nRows, int64_t nJt, double* __restrict__ partial,
                unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
  const int t = threadIdx.x;
  const int warp = t >> 5;

  int64_t I, J;
  if (MODE == 0) {
    tile_index(blockIdx.x, I, J);
  } else {
    I = blockIdx.x / nJt;
    J = blockIdx.x % nJt;
  }
  const bool diag = (MODE == 0) && (I == J);

  // Row segment of this thread.
  int64_t gi;
  bool iActive;
  if (MODE == 0) {
    gi = I * TILE + t;
    iActive = skipArr[gi] == 0;
  } else {
    int64_t r = I * TILE + t;
    iActive = r < nRows;
    gi = iActive ? rows[r] : 0;
    iActive = iActive && skipArr[gi] == 0;
  }
  SegF64 si = load_seg_global(soa, npad, gi);

  // J tile into shared memory.
  const int64_t j0 = J * TILE;
#pragma unroll
  for (int k = 0; k < 13; ++k) sm.seg[k][t] = soa[k * npad + j0 + t];
  sm.skip[t] = skipArr[j0 + t];
#pragma unroll
  for (int w = 0; w < NWARP; ++w)
#pragma unroll
    for (int c = 0; c < 6; ++c) sm.fj[w][c][t] = 0.0;
  __syncthreads();

  D3 fi1 = {0, 0, 0}, fi2 = {0, 0, 0};
  uint32_t pmask[TILE / 32] = {0, 0, 0, 0};
  unsigned long long nGeneral = 0;

  // ---- Sweep: general pairs now, near-parallel pairs flagged. ----
  for (int k = 0; k < TILE; ++k) {
    const int jl = (t + k) & (TILE - 1);
    bool act = iActive && sm.skip[jl] == 0;
    if (MODE == 0) act = act && (!diag || jl > t);
    if (MODE == 1) act = act && (j0 + jl != gi);
    if (act) {
      SegF64 sj = load_seg_smem(sm, jl);
      double c = dot(si.t, sj.t);
      double omcSq = 1.0 - c * c;
      if (omcSq > kSqrtEps) {
        D3 F1, F2, F3, F4;
        if (MODE == 0) {
          general_pair<true, true>(K, si.b, si.n1, si.n2, si.t, si.tN, sj.b, sj.n1, sj.n2, sj.t, sj.tN, c, F1, F2,
                                   F3, F4);
          double* fj = &sm.fj[warp][0][0];
          fj[0 * TILE + jl] += F3.x;
          fj[1 * TILE + jl] += F3.y;
          fj[2 * TILE + jl] += F3.z;
          fj[3 * TILE + jl] += F4.x;
          fj[4 * TILE + jl] += F4.y;
          fj[5 * TILE + jl] += F4.z;
        } else {
          general_pair<true, false>(K, si.b, si.n1, si.n2, si.t, si.tN, sj.b, sj.n1, sj.n2, sj.t, sj.tN, c, F1, F2,
                                    F3, F4);
        }
        fi1 = fi1 + F1;
        fi2 = fi2 + F2;
        ++nGeneral;
      } else {
        pmask[jl >> 5] |= 1u << (jl & 31);
      }
    }
    __syncwarp();
  }

  // ---- Near-parallel pairs: compact, then evaluate densely. ----
  int myCnt = __popc(pmask[0]) + __popc(pmask[1]) + __popc(pmask[2]) + __popc(pmask[3]);
  sm.cnt[t] = myCnt;
  __syncthreads();
  // Exclusive scan over 128 counts (one warp, deterministic).
  if (warp == 0) {
    int v[4];
    int s = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[q] = sm.cnt[4 * t + q];
      s += v[q];
    }
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int n = __shfl_up_sync(0xffffffffu, incl, o);
      if ((t & 31) >= o) incl += n;
    }
    int excl = incl - s;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      sm.cnt[4 * t + q] = excl;
      excl += v[q];
    }
  }
  __syncthreads();
  const int myOff = sm.cnt[t];
  // Total = offset of the last thread + its own count.
  __shared__ int sTotal;
  if (t == TILE - 1) sTotal = myOff + myCnt;
  {
    int o = myOff;
    for (int k = 0; k < TILE; ++k) {
      const int jl = (t + k) & (TILE - 1);
      if (pmask[jl >> 5] & (1u << (jl & 31))) sm.plist[o++] = (uint16_t)((t << 8) | jl);
    }
  }
  __syncthreads();
  const int nPar = sTotal;
  D3 fjp3 = {0, 0, 0}, fjp4 = {0, 0, 0};  // near-parallel forces on j = t
  unsigned long long nCore = 0;
  for (int base = 0; base < nPar; base += CHUNK) {
    const int e = base + t;
    if (e < nPar) {
      const int il = sm.plist[e] >> 8, jl = sm.plist[e] & 0xff;
      SegF64 a, b;
      if (MODE == 0) {
        a = load_seg_global(soa, npad, I * TILE + il);
      } else {
        a = load_seg_global(soa, npad, rows[I * TILE + il]);
      }
      b = load_seg_smem(sm, jl);
      double c = dot(a.t, b.t);
      D3 F1, F2, F3 = {0, 0, 0}, F4 = {0, 0, 0};
      if (MODE == 0)
        nCore += parallel_pair<true>(K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
      else
        nCore += parallel_pair<false>(K, a.b, a.n1, a.n2, a.t, a.tN, b.b, b.n1, b.n2, b.t, b.tN, c, F1, F2, F3, F4);
      sm.cf[t][0] = F1.x; sm.cf[t][1] = F1.y; sm.cf[t][2] = F1.z;
      sm.cf[t][3] = F2.x; sm.cf[t][4] = F2.y; sm.cf[t][5] = F2.z;
      sm.cf[t][6] = F3.x; sm.cf[t][7] = F3.y; sm.cf[t][8] = F3.z;
      sm.cf[t][9] = F4.x; sm.cf[t][10] = F4.y; sm.cf[t][11] = F4.z;
    }
    __syncthreads();
    const int lim = min(CHUNK, nPar - base);
    // i-side: this thread's entries are contiguous in the list.
    int lo = max(myOff, base), hi = min(myOff + myCnt, base + lim);
    for (int e2 = lo; e2 < hi; ++e2) {
      const double* f = sm.cf[e2 - base];
      fi1 = fi1 + D3{f[0], f[1], f[2]};
      fi2 = fi2 + D3{f[3], f[4], f[5]};
    }
    if (MODE == 0) {
      // j-side: scan the chunk for entries whose j is this thread's slot.
      for (int q = 0; q < lim; ++q) {
        if ((sm.plist[base + q] & 0xff) == t) {
          const double* f = sm.cf[q];
          fjp3 = fjp3 + D3{f[6], f[7], f[8]};
          fjp4 = fjp4 + D3{f[9], f[10], f[11]};
        }
      }
    }
    __syncthreads();
  }

  // ---- Write partials: [block][side][6][TILE], side 0 = row tile, 1 = col tile. ----
  double* p = partial + (int64_t)blockIdx.x * (MODE == 0 ? 12 : 6) * TILE;
  p[0 * TILE + t] = fi1.x;
  p[1 * TILE + t] = fi1.y;
  p[2 * TILE + t] = fi1.z;
  p[3 * TILE + t] = fi2.x;
  p[4 * TILE + t] = fi2.y;
  p[5 * TILE + t] = fi2.z;
  if (MODE == 0) {
    double acc[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      double s = sm.fj[0][c][t];
#pragma unroll
      for (int w = 1; w < NWARP; ++w) s += sm.fj[w][c][t];
      acc[c] = s;
    }
    acc[0] += fjp3.x;
    acc[1] += fjp3.y;
    acc[2] += fjp3.z;
    acc[3] += fjp4.x;
    acc[4] += fjp4.y;
    acc[5] += fjp4.z;
#pragma unroll
    for (int c = 0; c < 6; ++c) p[(6 + c) * TILE + t] = acc[c];
  }

  // Branch statistics: pairs on the general path, pairs on the near-parallel
  // path, near-parallel sides that needed the two core-correction evaluations.
  if (counters) {
    unsigned long long g = nGeneral, cc = nCore;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      g += __shfl_down_sync(0xffffffffu, g, o);
      cc += __shfl_down_sync(0xffffffffu, cc, o);
    }
    if ((t & 31) == 0) {
      atomicAdd(&counters[0], g);
      atomicAdd(&counters[2], cc);
    }
    if (t == 0) atomicAdd(&counters[1], (unsigned long long)nPar);
  }
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

static bool g_attr_set[2] = {false, false};

template <int MODE>
static cudaError_t set_attr() {
  if (!g_attr_set[MODE]) {
    cudaError_t e = cudaFuncSetAttribute(segseg_tile_f64<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TileSmem));
    if (e != cudaSuccess) return e;
    g_attr_set[MODE] = true;
  }
  return cudaSuccess;
}

cudaError_t launch_reduce_all(const double* partial, int64_t npad, int64_t numSeg, double* out, cudaStream_t st) {
  segseg_reduce_all<<<(unsigned)((numSeg + 127) / 128), 128, 0, st>>>(partial, npad / TILE, numSeg, out);
  return cudaGetLastError();
}

cudaError_t launch_reduce_rows(const double* partial, int64_t npad, int64_t nRows, double* out, cudaStream_t st) {
  segseg_reduce_rows<<<(unsigned)((nRows + 127) / 128), 128, 0, st>>>(partial, npad / TILE, nRows, out);
  return cudaGetLastError();
}

cudaError_t launch_segseg_all_f64(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                  double* partial, double* out, int64_t numSeg, unsigned long long* counters,
                                  cudaStream_t st) {
  cudaError_t e = set_attr<0>();
  if (e != cudaSuccess) return e;
  const int64_t nt = npad / TILE;
  const int64_t nb = nt * (nt + 1) / 2;
  segseg_tile_f64<0><<<(unsigned)nb, TILE, sizeof(TileSmem), st>>>(K, soa, skip, npad, nullptr, 0, 0, partial,
                                                                    counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  segseg_reduce_all<<<(unsigned)((numSeg + 127) / 128), 128, 0, st>>>(partial, nt, numSeg, out);
  return cudaGetLastError();
}

cudaError_t launch_segseg_rows_f64(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                   const int64_t* rows, int64_t nRows, double* partial, double* out,
                                   unsigned long long* counters, cudaStream_t st) {
  cudaError_t e = set_attr<1>();
  if (e != cudaSuccess) return e;
  const int64_t nJt = npad / TILE;
  const int64_t nrt = (nRows + TILE - 1) / TILE;
  segseg_tile_f64<1><<<(unsigned)(nrt * nJt), TILE, sizeof(TileSmem), st>>>(K, soa, skip, npad, rows, nRows, nJt,
                                                                             partial, counters);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  segseg_reduce_rows<<<(unsigned)((nRows + 127) / 128), 128, 0, st>>>(partial, nJt, nRows, out);
  return cudaGetLastError();
}

}  // namespace DDD_VARIANT
}  // namespace ddd
