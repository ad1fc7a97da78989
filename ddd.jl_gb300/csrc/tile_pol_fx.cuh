// Tile-body policy of the fast FP64 form (DDD_MODE_FP64_FAST): the strict FP64
// policy (segment data, branch decision, near-parallel branch, accumulation)
// with the general branch of pair_f64fast.cuh, its logarithms and arctangents on
// the integer pipes (intmath_f64.cuh).  Used by the all-pairs and
// index-list kernels (segseg_f64fast.cu) and by the surrogate path's exact
// passes (surrogate_force.cu); both translation units compile without
// contraction, so the fused operations are exactly pair_f64fast.cuh's.
#pragma once
#include "pair_f64.cuh"
#include "pair_f64fast.cuh"
#include "tile_body.cuh"

namespace ddd {

__device__ __forceinline__ fx::X3 fx_x3(const D3& v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ D3 fx_d3(const fx::X3& v) { return {v.x, v.y, v.z}; }

struct PolF64Fast : PolF64 {
  template <bool BOTH>
  static __device__ __forceinline__ void general(const Consts&, const TileArgs& A, const Seg& a, const Seg& b,
                                                 double c, D3& F1, D3& F2, D3& F3, D3& F4) {
    const fx::KFast K{A.K.aSq, A.K.mu4pi, A.K.mu8pi, A.K.mu4pinu, A.K.mu8piaSq, A.K.mu4pinuaSq};
    fx::X3 G1, G2, G3, G4;
    fx::general_pair<true, BOTH, fx::kMathInt>(K, fx_x3(a.b), fx_x3(a.n1), fx_x3(a.n2), fx_x3(a.t), a.tN, fx_x3(b.b),
                                       fx_x3(b.n1), fx_x3(b.n2), fx_x3(b.t), b.tN, c, G1, G2, G3, G4);
    F1 = fx_d3(G1);
    F2 = fx_d3(G2);
    if (BOTH) {
      F3 = fx_d3(G3);
      F4 = fx_d3(G4);
    }
  }
  static __device__ __forceinline__ void dense_general(const Consts& KP, const TileArgs& A, int64_t gi, int64_t gj,
                                                       D3& F1, D3& F2, D3& F3, D3& F4) {
    const SegF64 a = tb_load_seg64(A.soa, A.npad, gi), b = tb_load_seg64(A.soa, A.npad, gj);
    general<true>(KP, A, a, b, dot(a.t, b.t), F1, F2, F3, F4);
  }
};

}  // namespace ddd
