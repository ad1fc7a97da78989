// Self force and PK force of each segment (calcSelfForce / calcPKForce,
// DislocationForces.jl:216-300, 320-455), strict FP64 (compiled with
// --fmad=false: every multiply and add rounded as in the reference).
//
// One thread per entry k of the segment list (rows of segIdx, 0-based; all
// segments when rows is NULL).  Outputs, 3 × n each:
//   S  = the self force on node 2 (_calcSelfForce; node 1 gets -S);
//   PK = (σ̂ b) × (n2 - n1) from the caller's stress at each segment's midpoint
//        (sigmaHat 6 × n: xx, yy, zz, xy, xz, yz), or skipped when sigmaHat is NULL.
// Entry k is skipped (zeros) when ext[k] is set: the reference reads the
// external flag at the position in its index list, not at the segment.
#include <cuda_runtime.h>

#include "ddd_internal.h"
#include "pair_f64.cuh"

namespace ddd {
namespace {

__global__ void self_pk_f64(SelfK K, const double* __restrict__ coord, const double* __restrict__ bVec,
                            const int64_t* __restrict__ segIdx, int64_t ld, const uint8_t* __restrict__ ext,
                            int64_t nExt, const int64_t* __restrict__ rows, int64_t n,
                            const double* __restrict__ sigmaHat, double* __restrict__ S, double* __restrict__ PK) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  D3 s = {0, 0, 0}, pk = {0, 0, 0};
  if (!(ext && q < nExt && ext[q])) {
    const int64_t i = rows ? rows[q] : q;
    const int64_t l = segIdx[i] - 1, a = segIdx[i + ld] - 1, c = segIdx[i + 2 * ld] - 1;
    const D3 n1 = {coord[3 * a], coord[3 * a + 1], coord[3 * a + 2]};
    const D3 n2 = {coord[3 * c], coord[3 * c + 1], coord[3 * c + 2]};
    const D3 b = {bVec[3 * l], bVec[3 * l + 1], bVec[3 * l + 2]};
    const D3 tVec = n2 - n1;
    // _calcSelfForce (:414-455).
    const double tVecSq = dot(tVec, tVec);
    const double L = sqrt(tVecSq);
    const double Linv = 1.0 / L;
    const D3 t = tVec * Linv;
    const double La = sqrt(tVecSq + K.aSq);
    const double bScrew = dot(t, b);
    const D3 bEdge = b - bScrew * t;
    const double bEdgeSq = dot(bEdge, bEdge);
    const double LaMa = La - K.a;
    const double tor =
        K.mu4pi * bScrew * (K.nuOmNuInv * (log((La + L) / K.a) - 2.0 * LaMa * Linv) - LaMa * LaMa / (2.0 * La * L));
    const double torCore = 2.0 * K.Ec * K.nuOmNuInv * bScrew;
    const double torTot = tor + torCore;
    const double lonCore = (bScrew * bScrew + bEdgeSq * K.omNuInv) * K.Ec;
    s = torTot * bEdge - lonCore * t;
    if (sigmaHat) {
      // _calcPKForce (:292-300): (σ̂ b) × t, t not normalised.
      const double* g = sigmaHat + 6 * q;
      const D3 sb = {g[0] * b.x + g[3] * b.y + g[4] * b.z, g[3] * b.x + g[1] * b.y + g[5] * b.z,
                     g[4] * b.x + g[5] * b.y + g[2] * b.z};
      pk = cross(sb, tVec);
    }
  }
  S[3 * q] = s.x;
  S[3 * q + 1] = s.y;
  S[3 * q + 2] = s.z;
  if (PK) {
    PK[3 * q] = pk.x;
    PK[3 * q + 1] = pk.y;
    PK[3 * q + 2] = pk.z;
  }
}

}  // namespace

cudaError_t launch_self_pk(const SelfK& K, const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld,
                           const uint8_t* ext, int64_t nExt, const int64_t* rows, int64_t n, const double* sigmaHat,
                           double* S, double* PK, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  self_pk_f64<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(K, coord, bVec, segIdx, ld, ext, nExt, rows, n, sigmaHat,
                                                          S, PK);
  return cudaGetLastError();
}

}  // namespace ddd
