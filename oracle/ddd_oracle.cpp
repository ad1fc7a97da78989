// CPU ORACLE — test infrastructure only (see ddd_oracle.hpp).  C entry points
// over the templated restatement, for ctypes (oracle/oracle.py).
//
// Network layout (Julia column-major, 1-based indices, as DislocationNetwork
// stores it: src/Type/DislocationType.jl:324-340):
//   coord   double[3 * coordCols]       coord[3*(node-1) + k]
//   bVec    double[3 * bVecCols]        bVec[3*(link-1) + k]
//   segIdx  int64[ldSegIdx * 3]          segIdx[(i-1) + ldSegIdx*c] = (link, node1, node2)
//   extSeg  uint8[numSeg]                Julia Vector{Bool}
//   forces  double[3 * 2 * n]            F[k + 3*(node + 2*s)]  (segForce layout)
//   sigma   double[6 * M]                (xx, yy, zz, xy, xz, yz) per point
#include "ddd_oracle.hpp"

#include <omp.h>

#include <atomic>
#include <cstring>
#include <vector>

using namespace ddd_oracle;

namespace {

struct Seg {
  V3<double> b, n1, n2;
};

Consts<double> make_consts(const double* k5) {
  // k5 = (aSq, μ4π, μ8π, μ4πν, νμ4πν)
  Consts<double> K;
  K.aSq = k5[0];
  K.mu4pi = k5[1];
  K.mu8pi = k5[2];
  K.mu4pinu = k5[3];
  K.nuMu4pinu = k5[4];
  K.mu8piaSq = K.aSq * K.mu8pi;      // DislocationForces.jl:681
  K.mu4pinuaSq = K.aSq * K.mu4pinu;  // DislocationForces.jl:682
  return K;
}

inline V3<double> col3(const double* a, int64_t col1) {
  const double* p = a + 3 * (col1 - 1);
  return {p[0], p[1], p[2]};
}

// segSegForceUnroll's gathers (DislocationForces.jl:692-697).
std::vector<Seg> gather(const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld, int64_t numSeg) {
  std::vector<Seg> s(numSeg);
  for (int64_t i = 0; i < numSeg; ++i) {
    s[i].b = col3(bVec, segIdx[i]);
    s[i].n1 = col3(coord, segIdx[i + ld]);
    s[i].n2 = col3(coord, segIdx[i + 2 * ld]);
  }
  return s;
}

inline void add3(double* dst, const V3<double>& v) {
  dst[0] = dst[0] + v.x;
  dst[1] = dst[1] + v.y;
  dst[2] = dst[2] + v.z;
}

}  // namespace

extern "C" {

// One pair: F[12] = (Fnode1, Fnode2, Fnode3, Fnode4).  DislocationForces.jl:879.
void oracle_segseg_pair(const double* k5, const double* b1, const double* n11, const double* n12, const double* b2,
                        const double* n21, const double* n22, double* F) {
  Consts<double> K = make_consts(k5);
  V3<double> out[4];
  seg_seg_force<double>(K, {b1[0], b1[1], b1[2]}, {n11[0], n11[1], n11[2]}, {n12[0], n12[1], n12[2]},
                        {b2[0], b2[1], b2[2]}, {n21[0], n21[1], n21[2]}, {n22[0], n22[1], n22[2]}, out);
  for (int q = 0; q < 4; ++q) {
    F[3 * q + 0] = out[q].x;
    F[3 * q + 1] = out[q].y;
    F[3 * q + 2] = out[q].z;
  }
}

// One pair by Gauss quadrature of the σ̃ field (not a reference function: the
// restatement of a far-field form planned for the GPU, kept as its checker).
// Segment 1's nodal forces are the integrals over s in [0, 1] of
// N_k(s) (σ̃_2(x(s)) b1) × (n12 - n11), N_1 = 1 - s, N_2 = s, x(s) = n11 +
// s (n12 - n11), where σ̃_2 is segment 2's non-singular stress (the reference's
// formula, DislocationFEM.jl:86-303) and (σ b) × (n2 - n1) the force per unit
// parameter (DislocationForces.jl:292-300).  nq-point Gauss-Legendre rule on
// [0, 1], nq = 1..4.  Segment 2's nodal forces the same way with the roles
// exchanged.  F[12] as oracle_segseg_pair.
void oracle_segseg_pair_quad(const double* k5, const double* b1, const double* n11, const double* n12,
                             const double* b2, const double* n21, const double* n22, int nq, double* F) {
  static const double X[4][4] = {{0.0}, {-0.5773502691896257, 0.5773502691896257},
                                 {-0.7745966692414834, 0.0, 0.7745966692414834},
                                 {-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526}};
  static const double W[4][4] = {{2.0}, {1.0, 1.0}, {0.5555555555555556, 0.8888888888888888, 0.5555555555555556},
                                 {0.3478548451374538, 0.6521451548625461, 0.6521451548625461, 0.3478548451374538}};
  for (int k = 0; k < 12; ++k) F[k] = 0.0;
  if (nq < 1 || nq > 4) return;
  const Consts<double> K = make_consts(k5);
  const V3<double> B[2] = {{b1[0], b1[1], b1[2]}, {b2[0], b2[1], b2[2]}};
  const V3<double> A[2] = {{n11[0], n11[1], n11[2]}, {n21[0], n21[1], n21[2]}};
  const V3<double> E[2] = {{n12[0], n12[1], n12[2]}, {n22[0], n22[1], n22[2]}};
  for (int side = 0; side < 2; ++side) {
    const int o = 1 - side;  // the segment whose field acts
    const V3<double> to = normalize(E[o] - A[o]);
    const V3<double> l = E[side] - A[side];
    V3<double> Fa = {0, 0, 0}, Fb = {0, 0, 0};
    for (int q = 0; q < nq; ++q) {
      const double sq = 0.5 * (1.0 + X[nq - 1][q]), wq = 0.5 * W[nq - 1][q];
      const V3<double> x = A[side] + sq * l;
      double sig[6] = {0, 0, 0, 0, 0, 0};
      sigma_tilde_point<double>(K, B[o], A[o], E[o], to, x, sig);
      const V3<double> f = pk_force<double>(sig, B[side], l);
      Fa = Fa + (wq * (1.0 - sq)) * f;
      Fb = Fb + (wq * sq) * f;
    }
    const V3<double> out[2] = {Fa, Fb};
    for (int k = 0; k < 2; ++k) {
      F[6 * side + 3 * k + 0] = out[k].x;
      F[6 * side + 3 * k + 1] = out[k].y;
      F[6 * side + 3 * k + 2] = out[k].z;
    }
  }
}

// Same pair in single precision (for the reduced-precision error studies).
void oracle_segseg_pair_f32(const double* k5, const double* b1, const double* n11, const double* n12,
                            const double* b2, const double* n21, const double* n22, double* F) {
  Consts<float> K;
  K.aSq = (float)k5[0];
  K.mu4pi = (float)k5[1];
  K.mu8pi = (float)k5[2];
  K.mu4pinu = (float)k5[3];
  K.nuMu4pinu = (float)k5[4];
  K.mu8piaSq = K.aSq * K.mu8pi;
  K.mu4pinuaSq = K.aSq * K.mu4pinu;
  auto f = [](const double* p) { return V3<float>{(float)p[0], (float)p[1], (float)p[2]}; };
  V3<float> out[4];
  seg_seg_force<float>(K, f(b1), f(n11), f(n12), f(b2), f(n21), f(n22), out);
  for (int q = 0; q < 4; ++q) {
    F[3 * q + 0] = out[q].x;
    F[3 * q + 1] = out[q].y;
    F[3 * q + 2] = out[q].z;
  }
}

// calcSegSegForceSer! (DislocationForces.jl:778-829): accumulates into F
// (3×2×numSeg), which the caller zeroes for the non-mutating form.
void oracle_segseg_ser(const double* k5, const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld,
                       const uint8_t* extSeg, int64_t numSeg, double* F) {
  Consts<double> K = make_consts(k5);
  std::vector<Seg> s = gather(coord, bVec, segIdx, ld, numSeg);
  V3<double> out[4];
  for (int64_t i = 0; i < numSeg; ++i) {
    if (extSeg[i]) continue;
    for (int64_t j = i + 1; j < numSeg; ++j) {
      if (extSeg[j]) continue;
      seg_seg_force<double>(K, s[i].b, s[i].n1, s[i].n2, s[j].b, s[j].n1, s[j].n2, out);
      add3(F + 6 * i, out[0]);
      add3(F + 6 * i + 3, out[1]);
      add3(F + 6 * j, out[2]);
      add3(F + 6 * j + 3, out[3]);
    }
  }
}

// calcSegSegForcePar (DislocationForces.jl:719-777): contiguous i-chunks
// start = 1 + ((tid-1)·N)÷T, stop = (tid·N)÷T per thread, j > i, one atomic
// add per output component.  Overwrites F (3×2×numSeg).
void oracle_segseg_par_atomic(const double* k5, const double* coord, const double* bVec, const int64_t* segIdx,
                              int64_t ld, const uint8_t* extSeg, int64_t numSeg, double* F, int nthreads) {
  Consts<double> K = make_consts(k5);
  std::vector<Seg> s = gather(coord, bVec, segIdx, ld, numSeg);
  std::vector<std::atomic<double>> acc(6 * numSeg);
  for (auto& a : acc) a.store(0.0, std::memory_order_relaxed);
#pragma omp parallel num_threads(nthreads)
  {
    const int64_t T = omp_get_num_threads();
    const int64_t tid = omp_get_thread_num() + 1;
    const int64_t start = 1 + ((tid - 1) * numSeg) / T;
    const int64_t stop = (tid * numSeg) / T;
    V3<double> out[4];
    for (int64_t i1 = start; i1 <= stop; ++i1) {
      const int64_t i = i1 - 1;
      if (extSeg[i]) continue;
      for (int64_t j = i + 1; j < numSeg; ++j) {
        if (extSeg[j]) continue;
        seg_seg_force<double>(K, s[i].b, s[i].n1, s[i].n2, s[j].b, s[j].n1, s[j].n2, out);
        const double* o = &out[0].x;
        (void)o;
        const V3<double>* q = out;
        acc[6 * i + 0].fetch_add(q[0].x, std::memory_order_relaxed);
        acc[6 * i + 1].fetch_add(q[0].y, std::memory_order_relaxed);
        acc[6 * i + 2].fetch_add(q[0].z, std::memory_order_relaxed);
        acc[6 * i + 3].fetch_add(q[1].x, std::memory_order_relaxed);
        acc[6 * i + 4].fetch_add(q[1].y, std::memory_order_relaxed);
        acc[6 * i + 5].fetch_add(q[1].z, std::memory_order_relaxed);
        acc[6 * j + 0].fetch_add(q[2].x, std::memory_order_relaxed);
        acc[6 * j + 1].fetch_add(q[2].y, std::memory_order_relaxed);
        acc[6 * j + 2].fetch_add(q[2].z, std::memory_order_relaxed);
        acc[6 * j + 3].fetch_add(q[3].x, std::memory_order_relaxed);
        acc[6 * j + 4].fetch_add(q[3].y, std::memory_order_relaxed);
        acc[6 * j + 5].fetch_add(q[3].z, std::memory_order_relaxed);
      }
    }
  }
  for (int64_t k = 0; k < 6 * numSeg; ++k) F[k] = acc[k].load(std::memory_order_relaxed);
}

// The best-effort CPU form of the same all-pairs sum (not a reference code
// path): rows handed out dynamically, every thread accumulating into its own
// 3×2×numSeg array, the arrays summed at the end.  No atomics, balanced load;
// the result differs from Ser / Par only by summation order.
void oracle_segseg_par_private(const double* k5, const double* coord, const double* bVec, const int64_t* segIdx,
                               int64_t ld, const uint8_t* extSeg, int64_t numSeg, double* F, int nthreads) {
  Consts<double> K = make_consts(k5);
  std::vector<Seg> s = gather(coord, bVec, segIdx, ld, numSeg);
  const int T = nthreads > 0 ? nthreads : 1;
  std::vector<double> priv((size_t)T * 6 * numSeg, 0.0);
#pragma omp parallel num_threads(T)
  {
    double* acc = priv.data() + (size_t)omp_get_thread_num() * 6 * numSeg;
    V3<double> out[4];
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < numSeg; ++i) {
      if (extSeg[i]) continue;
      for (int64_t j = i + 1; j < numSeg; ++j) {
        if (extSeg[j]) continue;
        seg_seg_force<double>(K, s[i].b, s[i].n1, s[i].n2, s[j].b, s[j].n1, s[j].n2, out);
        add3(acc + 6 * i, out[0]);
        add3(acc + 6 * i + 3, out[1]);
        add3(acc + 6 * j, out[2]);
        add3(acc + 6 * j + 3, out[3]);
      }
    }
  }
  for (int64_t k = 0; k < 6 * numSeg; ++k) {
    double v = 0.0;
    for (int t = 0; t < T; ++t) v += priv[(size_t)t * 6 * numSeg + k];
    F[k] = v;
  }
}

// Rows of the all-pairs (Ser) result for the segments in rows[] (0-based):
// F_s = Σ_{j<s} Fnode3,4(j, s) + Σ_{j>s} Fnode1,2(s, j), added in that order,
// which is exactly the order calcSegSegForceSer! adds into column s.  Used to
// check large networks on sampled segments.  Overwrites F (3×2×nRows).
void oracle_segseg_rows(const double* k5, const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld,
                        const uint8_t* extSeg, int64_t numSeg, const int64_t* rows, int64_t nRows, double* F,
                        int nthreads) {
  Consts<double> K = make_consts(k5);
  std::vector<Seg> s = gather(coord, bVec, segIdx, ld, numSeg);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int64_t r = 0; r < nRows; ++r) {
    const int64_t i = rows[r];
    double* dst = F + 6 * r;
    for (int k = 0; k < 6; ++k) dst[k] = 0.0;
    if (extSeg[i]) continue;
    V3<double> out[4];
    for (int64_t j = 0; j < i; ++j) {
      if (extSeg[j]) continue;
      seg_seg_force<double>(K, s[j].b, s[j].n1, s[j].n2, s[i].b, s[i].n1, s[i].n2, out);
      add3(dst, out[2]);
      add3(dst + 3, out[3]);
    }
    for (int64_t j = i + 1; j < numSeg; ++j) {
      if (extSeg[j]) continue;
      seg_seg_force<double>(K, s[i].b, s[i].n1, s[i].n2, s[j].b, s[j].n1, s[j].n2, out);
      add3(dst, out[0]);
      add3(dst + 3, out[1]);
    }
  }
}

// Index-list form (DislocationForces.jl:528-557 and calcSegSegForceIdx! :831-877):
// for k, i = idx[k] (1-based), skip ext i; F[:,:,k] += Σ_{j≠i, !ext j} Fnode1,2(i, j).
// F is 3×2×nIdx and accumulated into (the caller zeroes it for the fresh form).
void oracle_segseg_idx(const double* k5, const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld,
                       const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx, double* F,
                       int nthreads) {
  Consts<double> K = make_consts(k5);
  std::vector<Seg> s = gather(coord, bVec, segIdx, ld, numSeg);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int64_t k = 0; k < nIdx; ++k) {
    const int64_t i = idx[k] - 1;
    if (extSeg[i]) continue;
    double* dst = F + 6 * k;
    V3<double> out[4];
    for (int64_t j = 0; j < numSeg; ++j) {
      if (i == j || extSeg[j]) continue;
      seg_seg_force<double>(K, s[i].b, s[i].n1, s[i].n2, s[j].b, s[j].n1, s[j].n2, out);
      add3(dst, out[0]);
      add3(dst + 3, out[1]);
    }
  }
}

// _calc_σTilde! (DislocationFEM.jl:86-303) for an array of points x0 (3×M).
// calcSelfForce (DislocationForces.jl:320-353): for each k (idx[k], 1-based
// rows of segIdx, or 1:numSeg when idx is NULL) the node forces F1 = -s,
// F2 = s (3 × n each, overwritten).  As in the reference, the external flag
// read for entry k is extSeg[k] (the position in idx, not the segment).
// sc = (coreRad, coreEnergy, ν) and k5[1] = μ4π.
void oracle_self_force(const double* k5, const double* sc, const double* coord, const double* bVec,
                       const int64_t* segIdx, int64_t ld, const uint8_t* extSeg, int64_t numSeg, const int64_t* idx,
                       int64_t nIdx, double* F1, double* F2) {
  SelfConsts<double> K;
  K.a = sc[0];
  K.aSq = sc[0] * sc[0];  // DislocationConstructor.jl:83
  K.mu4pi = k5[1];
  K.omNuInv = 1.0 / (1.0 - sc[2]);  // MaterialConstructor.jl
  K.nuOmNuInv = sc[2] * K.omNuInv;
  K.Ec = sc[1];
  const int64_t n = idx ? nIdx : numSeg;
  for (int64_t q = 0; q < n; ++q) {
    for (int c = 0; c < 3; ++c) F1[3 * q + c] = F2[3 * q + c] = 0.0;
    if (extSeg[q]) continue;
    const int64_t i = idx ? idx[q] - 1 : q;
    const V3<double> n1 = col3(coord, segIdx[i + ld]), n2 = col3(coord, segIdx[i + 2 * ld]);
    const V3<double> s = self_force_node2(K, n2 - n1, col3(bVec, segIdx[i]));
    F1[3 * q] = -s.x;
    F1[3 * q + 1] = -s.y;
    F1[3 * q + 2] = -s.z;
    F2[3 * q] = s.x;
    F2[3 * q + 1] = s.y;
    F2[3 * q + 2] = s.z;
  }
}

// dlnMobility for a BCC material (DislocationMobility.jl:16-178): node forces
// and velocities (3 × n each) of the nodes in idx (1-based) or 1:numNode.
// mp = (σPN, edge, screw, climb, line drag).
void oracle_mobility_bcc(const double* mp, const double* coord, const double* bVec, const int64_t* links,
                         const int64_t* conn, int64_t ldConn, const double* segForce, int64_t numNode,
                         const int64_t* idx, int64_t nIdx, double* nodeForce, double* nodeVel) {
  const MobParams P{mp[0], mp[1], mp[2], mp[3], mp[4]};
  const int64_t n = idx ? nIdx : numNode;
  for (int64_t q = 0; q < n; ++q) {
    const int64_t node = idx ? idx[q] - 1 : q;
    V3<double> f, v;
    mobility_bcc_node<double>(P, coord, bVec, links, conn, ldConn, segForce, node, f, v);
    nodeForce[3 * q] = f.x;
    nodeForce[3 * q + 1] = f.y;
    nodeForce[3 * q + 2] = f.z;
    nodeVel[3 * q] = v.x;
    nodeVel[3 * q + 1] = v.y;
    nodeVel[3 * q + 2] = v.z;
  }
}

// minimumDistance (Misc.jl:314-367) for n segment pairs: pts is 3 × 8 × n
// (x0, x1, y0, y1, vx0, vx1, vy0, vy1 per pair), out 4 × n (distSq,
// dDistSqDt, L1, L2).
void oracle_minimum_distance(const double* pts, int64_t n, double* out) {
  for (int64_t q = 0; q < n; ++q) {
    V3<double> v[8];
    for (int k = 0; k < 8; ++k) v[k] = {pts[24 * q + 3 * k], pts[24 * q + 3 * k + 1], pts[24 * q + 3 * k + 2]};
    const MinDist<double> m = minimum_distance(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7]);
    out[4 * q] = m.distSq;
    out[4 * q + 1] = m.dDistSqDt;
    out[4 * q + 2] = m.L1;
    out[4 * q + 3] = m.L2;
  }
}

// detectCollision (DislocationTopologyCollision.jl:1-221).  iout (8): collision,
// type (0 null, 1 hinge, 2 twoLine), n1s1, n2s1, n1s2, n2s2, s1, s2; dout (5):
// L1, L2 (the reference's return values), pairDistSq, pairL1, pairL2.  skip holds
// nSkip (s1, s2) link pairs.
void oracle_detect_collision(double collisionDistSq, const double* coord, const double* nodeVel, const int32_t* label,
                             const int64_t* links, const double* bVec, const int64_t* conn, int64_t ldConn,
                             int64_t numNode, int64_t numSeg, const int64_t* skip, int64_t nSkip, int64_t* iout,
                             double* dout) {
  const Collision r = detect_collision<double>(collisionDistSq, coord, nodeVel, label, links, bVec, conn, ldConn,
                                               numNode, numSeg, skip, nSkip);
  const int64_t iv[8] = {r.collision, r.type, r.n1s1, r.n2s1, r.n1s2, r.n2s2, r.s1, r.s2};
  const double dv[5] = {r.L1, r.L2, r.pairDistSq, r.pairL1, r.pairL2};
  for (int k = 0; k < 8; ++k) iout[k] = iv[k];
  for (int k = 0; k < 5; ++k) dout[k] = dv[k];
}

// calc_uTilde (DislocationFEM.jl:355-581) at numPoints points (3 × M): u (3 × M)
// summed over the triangles in the reference's order for each point.  k2 =
// (omνInv8π, om2νomνInv8π); box = (lo xyz, hi xyz); C the closure point.  Points
// are split over nthreads (each point's sum keeps its order).  Returns the
// number of triangles.
int64_t oracle_u_tilde(const double* k2, const double* C, const double* faceNorm, const double* faceMidPt,
                       int64_t nF, const double* normals, int64_t nN, const double* box, double tol,
                       const double* points, int64_t M, const double* coord, const int32_t* label,
                       const int64_t* links, const double* bVec, int64_t numNode, int64_t numSeg, double* u,
                       int nthreads) {
  const UMesh<double> m{faceNorm, faceMidPt, nF, normals, nN, {box[0], box[1], box[2]}, {box[3], box[4], box[5]},
                        {C[0], C[1], C[2]}, tol};
  const std::vector<UTri<double>> tris = u_tilde_triangles<double>(m, coord, label, links, bVec, numNode, numSeg);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
  for (int64_t p = 0; p < M; ++p) {
    const V3<double> P = {points[3 * p], points[3 * p + 1], points[3 * p + 2]};
    V3<double> acc = {0.0, 0.0, 0.0};
    for (const auto& t : tris) acc = acc + tri_u(t, k2[0], k2[1], P);
    u[3 * p] = acc.x;
    u[3 * p + 1] = acc.y;
    u[3 * p + 2] = acc.z;
  }
  return (int64_t)tris.size();
}

// The triangle list of calc_uTilde (13 doubles each: A, B, C, b, full), for
// tests that look at single triangles.  Returns the count; writes at most cap.
int64_t oracle_u_tilde_tris(const double* C, const double* faceNorm, const double* faceMidPt, int64_t nF,
                            const double* normals, int64_t nN, const double* box, double tol, const double* coord,
                            const int32_t* label, const int64_t* links, const double* bVec, int64_t numNode,
                            int64_t numSeg, double* out, int64_t cap) {
  const UMesh<double> m{faceNorm, faceMidPt, nF, normals, nN, {box[0], box[1], box[2]}, {box[3], box[4], box[5]},
                        {C[0], C[1], C[2]}, tol};
  const std::vector<UTri<double>> tris = u_tilde_triangles<double>(m, coord, label, links, bVec, numNode, numSeg);
  for (int64_t t = 0; t < (int64_t)tris.size() && t < cap; ++t) {
    const UTri<double>& q = tris[t];
    const double r[13] = {q.A.x, q.A.y, q.A.z, q.B.x, q.B.y, q.B.z, q.C.x, q.C.y, q.C.z, q.b.x, q.b.y, q.b.z,
                          q.full ? 1.0 : 0.0};
    for (int k = 0; k < 13; ++k) out[13 * t + k] = r[k];
  }
  return (int64_t)tris.size();
}

// The same triangles (built in double, as the reference builds them) summed in
// long double: the reference arithmetic's own error at each point is
// |oracle_u_tilde - this|.
int64_t oracle_u_tilde_ld(const double* k2, const double* C, const double* faceNorm, const double* faceMidPt,
                          int64_t nF, const double* normals, int64_t nN, const double* box, double tol,
                          const double* points, int64_t M, const double* coord, const int32_t* label,
                          const int64_t* links, const double* bVec, int64_t numNode, int64_t numSeg, double* u,
                          int nthreads) {
  using LD = long double;
  const UMesh<double> m{faceNorm, faceMidPt, nF, normals, nN, {box[0], box[1], box[2]}, {box[3], box[4], box[5]},
                        {C[0], C[1], C[2]}, tol};
  const std::vector<UTri<double>> tris = u_tilde_triangles<double>(m, coord, label, links, bVec, numNode, numSeg);
  std::vector<UTri<LD>> tl;
  auto up = [](const V3<double>& v) { return V3<LD>{(LD)v.x, (LD)v.y, (LD)v.z}; };
  for (const auto& t : tris) tl.push_back(make_tri(up(t.A), up(t.B), up(t.C), up(t.b), t.full));
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
  for (int64_t p = 0; p < M; ++p) {
    const V3<LD> P = {(LD)points[3 * p], (LD)points[3 * p + 1], (LD)points[3 * p + 2]};
    V3<LD> acc = {0, 0, 0};
    for (const auto& t : tl) acc = acc + tri_u(t, (LD)k2[0], (LD)k2[1], P);
    u[3 * p] = (double)acc.x;
    u[3 * p + 1] = (double)acc.y;
    u[3 * p + 2] = (double)acc.z;
  }
  return (int64_t)tris.size();
}

// PK forces (σ̂ b) × (n2 - n1) of the segments in idx (or 1:numSeg) from the
// stresses sigmaHat (6 × n, one per entry, at the segment midpoints): PK
// (3 × n, overwritten; 0 where extSeg[k]).
void oracle_pk_force(const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld,
                     const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx, const double* sigmaHat,
                     double* PK) {
  const int64_t n = idx ? nIdx : numSeg;
  for (int64_t q = 0; q < n; ++q) {
    for (int c = 0; c < 3; ++c) PK[3 * q + c] = 0.0;
    if (extSeg[q]) continue;
    const int64_t i = idx ? idx[q] - 1 : q;
    const V3<double> t = col3(coord, segIdx[i + 2 * ld]) - col3(coord, segIdx[i + ld]);
    const V3<double> f = pk_force(sigmaHat + 6 * q, col3(bVec, segIdx[i]), t);
    PK[3 * q] = f.x;
    PK[3 * q + 1] = f.y;
    PK[3 * q + 2] = f.z;
  }
}

// idx (1-based rows of segIdx) selects segments, NULL = 1:numSeg.  Overwrites
// sigma (6×M).  The reference loops segments outside and points inside; each
// point's sum is taken over segments in order either way, so the threaded
// form (points split over threads) returns bitwise the same values.
void oracle_sigma_tilde(const double* k5, const double* x0, int64_t M, const double* coord, const double* bVec,
                        const int64_t* segIdx, int64_t ld, int64_t numSeg, const int64_t* idx, int64_t nIdx,
                        double* sigma, int nthreads) {
  Consts<double> K = make_consts(k5);
  int64_t nS = idx ? nIdx : numSeg;
  std::vector<Seg> s(nS);
  std::vector<V3<double>> t(nS);
  for (int64_t q = 0; q < nS; ++q) {
    int64_t i = idx ? idx[q] - 1 : q;
    s[q].b = col3(bVec, segIdx[i]);
    s[q].n1 = col3(coord, segIdx[i + ld]);
    s[q].n2 = col3(coord, segIdx[i + 2 * ld]);
    t[q] = normalize(s[q].n2 - s[q].n1);
  }
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t j = 0; j < M; ++j) {
    double sig[6] = {0, 0, 0, 0, 0, 0};
    V3<double> x = {x0[3 * j], x0[3 * j + 1], x0[3 * j + 2]};
    for (int64_t q = 0; q < nS; ++q) sigma_tilde_point<double>(K, s[q].b, s[q].n1, s[q].n2, t[q], x, sig);
    for (int k = 0; k < 6; ++k) sigma[6 * j + k] = sig[k];
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Operation counting.  The same templates instantiated with a scalar that
// counts every arithmetic operation give the algorithmic work of one pair or
// one (segment, point) evaluation.  Convention: add/sub/mul each 1; div, sqrt,
// log, atan counted separately; sign flips free.  Since the reference never
// fuses, the FLOP count is add + mul + div + sqrt + log + atan.
namespace {
struct OpCounts {
  long long add, mul, div, sqrt, log, atan, cmp;
};
thread_local OpCounts g_ops;

struct OD {
  double v;
  OD() = default;
  constexpr OD(double x) : v(x) {}
};
inline OD operator+(OD a, OD b) { ++g_ops.add; return OD(a.v + b.v); }
inline OD operator-(OD a, OD b) { ++g_ops.add; return OD(a.v - b.v); }
inline OD operator-(OD a) { return OD(-a.v); }
inline OD operator*(OD a, OD b) { ++g_ops.mul; return OD(a.v * b.v); }
inline OD operator/(OD a, OD b) { ++g_ops.div; return OD(a.v / b.v); }
inline bool operator>(OD a, OD b) { ++g_ops.cmp; return a.v > b.v; }
inline bool operator<(OD a, OD b) { ++g_ops.cmp; return a.v < b.v; }
inline OD sqrt(OD a) { ++g_ops.sqrt; return OD(std::sqrt(a.v)); }
inline OD log(OD a) { ++g_ops.log; return OD(std::log(a.v)); }
inline OD atan(OD a) { ++g_ops.atan; return OD(std::atan(a.v)); }

Consts<OD> make_consts_od(const double* k5) {
  Consts<OD> K;
  K.aSq = k5[0];
  K.mu4pi = k5[1];
  K.mu8pi = k5[2];
  K.mu4pinu = k5[3];
  K.nuMu4pinu = k5[4];
  K.mu8piaSq = k5[0] * k5[2];
  K.mu4pinuaSq = k5[0] * k5[3];
  return K;
}
inline V3<OD> v3od(const double* p) { return {OD(p[0]), OD(p[1]), OD(p[2])}; }
void store_counts(long long* c) {
  c[0] = g_ops.add;
  c[1] = g_ops.mul;
  c[2] = g_ops.div;
  c[3] = g_ops.sqrt;
  c[4] = g_ops.log;
  c[5] = g_ops.atan;
  c[6] = g_ops.cmp;
}
}  // namespace

extern "C" {
// counts[7] = (add/sub, mul, div, sqrt, log, atan, compare) for one pair; F[12] out.
void oracle_opcount_pair(const double* k5, const double* b1, const double* n11, const double* n12, const double* b2,
                         const double* n21, const double* n22, long long* counts, double* F) {
  g_ops = OpCounts{0, 0, 0, 0, 0, 0, 0};
  Consts<OD> K = make_consts_od(k5);
  V3<OD> out[4];
  seg_seg_force<OD>(K, v3od(b1), v3od(n11), v3od(n12), v3od(b2), v3od(n21), v3od(n22), out);
  store_counts(counts);
  for (int q = 0; q < 4; ++q) {
    F[3 * q + 0] = out[q].x.v;
    F[3 * q + 1] = out[q].y.v;
    F[3 * q + 2] = out[q].z.v;
  }
}

// counts[7] for one (segment, point) σ̃ evaluation, excluding the per-segment
// normalisation of t (done once per segment in the reference).
void oracle_opcount_sigma(const double* k5, const double* b, const double* n1, const double* n2, const double* x,
                          long long* counts, double* sig6) {
  Consts<OD> K = make_consts_od(k5);
  V3<OD> bb = v3od(b), a1 = v3od(n1), a2 = v3od(n2), xx = v3od(x);
  V3<OD> t = normalize(a2 - a1);
  OD sig[6] = {0, 0, 0, 0, 0, 0};
  g_ops = OpCounts{0, 0, 0, 0, 0, 0, 0};
  sigma_tilde_point<OD>(K, bb, a1, a2, t, xx, sig);
  store_counts(counts);
  for (int k = 0; k < 6; ++k) sig6[k] = sig[k].v;
}
}  // extern "C"

// ---------------------------------------------------------------------------
// σ̃ with every operation in long double (rounded to double at the end): its
// distance from the Float64 result is the reference arithmetic's own error
// (_calc_σTilde!, DislocationFEM.jl:129-299, as oracle_sigma_tilde).
extern "C" void oracle_sigma_tilde_ld(const double* k5, const double* x0, int64_t M, const double* coord,
                                      const double* bVec, const int64_t* segIdx, int64_t ld, int64_t numSeg,
                                      double* sigma, int nthreads) {
  typedef long double L;
  Consts<L> K;
  K.aSq = k5[0];
  K.mu4pi = k5[1];
  K.mu8pi = k5[2];
  K.mu4pinu = k5[3];
  K.nuMu4pinu = k5[4];
  K.mu8piaSq = (L)k5[0] * (L)k5[2];
  K.mu4pinuaSq = (L)k5[0] * (L)k5[3];
  std::vector<Seg> s = gather(coord, bVec, segIdx, ld, numSeg);
  auto cv = [](const V3<double>& v) { return V3<L>{(L)v.x, (L)v.y, (L)v.z}; };
  std::vector<V3<L>> t(numSeg);
  for (int64_t q = 0; q < numSeg; ++q) t[q] = normalize(cv(s[q].n2) - cv(s[q].n1));
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t j = 0; j < M; ++j) {
    L sig[6] = {0, 0, 0, 0, 0, 0};
    const V3<L> x = {(L)x0[3 * j], (L)x0[3 * j + 1], (L)x0[3 * j + 2]};
    for (int64_t q = 0; q < numSeg; ++q) sigma_tilde_point<L>(K, cv(s[q].b), cv(s[q].n1), cv(s[q].n2), t[q], x, sig);
    for (int k = 0; k < 6; ++k) sigma[6 * j + k] = (double)sig[k];
  }
}

// Extended-precision all-pairs (long double), to measure the rounding noise of
// the Float64 algorithm itself: |F_f64 - F_ld| is the reference's own error.
// rows (0-based, may be NULL = all) selects the segments returned; F is 3×2×nRows.
extern "C" void oracle_segseg_ser_ld(const double* k5, const double* coord, const double* bVec, const int64_t* segIdx,
                                     int64_t ld, const uint8_t* extSeg, int64_t numSeg, const int64_t* rows,
                                     int64_t nRows, double* F, int nthreads) {
  typedef long double L;
  Consts<L> K;
  K.aSq = k5[0];
  K.mu4pi = k5[1];
  K.mu8pi = k5[2];
  K.mu4pinu = k5[3];
  K.nuMu4pinu = k5[4];
  K.mu8piaSq = (L)k5[0] * (L)k5[2];
  K.mu4pinuaSq = (L)k5[0] * (L)k5[3];
  std::vector<Seg> s = gather(coord, bVec, segIdx, ld, numSeg);
  auto cv = [](const V3<double>& v) { return V3<L>{(L)v.x, (L)v.y, (L)v.z}; };
  const int64_t nOut = rows ? nRows : numSeg;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int64_t r = 0; r < nOut; ++r) {
    const int64_t i = rows ? rows[r] : r;
    L acc[6] = {0, 0, 0, 0, 0, 0};
    if (!extSeg[i]) {
      V3<L> out[4];
      for (int64_t j = 0; j < numSeg; ++j) {
        if (j == i || extSeg[j]) continue;
        const int64_t a = i < j ? i : j, b = i < j ? j : i;
        seg_seg_force<L>(K, cv(s[a].b), cv(s[a].n1), cv(s[a].n2), cv(s[b].b), cv(s[b].n1), cv(s[b].n2), out);
        const V3<L>* q = (i < j) ? out : out + 2;
        acc[0] += q[0].x; acc[1] += q[0].y; acc[2] += q[0].z;
        acc[3] += q[1].x; acc[4] += q[1].y; acc[5] += q[1].z;
      }
    }
    for (int c = 0; c < 6; ++c) F[6 * r + c] = (double)acc[c];
  }
}
