// Internal declarations shared by the kernel files and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <vector>

struct ddd_ctx;

namespace ddd {

// An NVTX range for the life of a C-ABI call: profilers (Nsight Systems, ncu's
// NVTX filters) show each entry point's span on the host timeline.  NVTX is
// header-only and costs a function-pointer check when no tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define DDD_NVTX(name) ::ddd::NvtxRange ddd_nvtx_range_(name)

struct KConsts;

// Raise a kernel's dynamic shared-memory limit on the current device, once per
// device: the attribute lives in each device's context, so `done` keeps one bit
// per device (devices past 63 set it on every call).  The bits are atomic, so
// contexts on several host threads may race here; setting it twice is harmless.
template <typename Kernel>
cudaError_t set_smem_once(Kernel* kernel, int bytes, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = dev < 64 ? (uint64_t)1 << dev : 0;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_release);
  return e;
}

// All-pairs partial sums: one slot (12 x TILE doubles) per tile pair I <= J,
// slot J(J+1)/2 + I.  The all-pairs launchers take the partial buffer's size
// in slots; when it is below nt(nt+1)/2 they run bands of J columns (each band
// at most capSlots slots, at least one column, so capSlots >= nt is required).
//
// segseg_f64.cu and sigma_f64.cu, each compiled as two variants:
//   strict: --fmad=false, every operation rounded as in the reference;
//   fast:   FMA contraction.
#define DDD_F64_DECLS \
  int64_t segseg_npad(int64_t numSeg); \
  size_t segseg_soa_bytes(int64_t npad); \
  size_t segseg_partial_bytes_all(int64_t npad); \
  size_t segseg_partial_bytes_rows(int64_t nRows, int64_t npad); \
  cudaError_t launch_prep_segments(const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld, \
                                   const uint8_t* extSeg, int64_t numSeg, int64_t npad, double* soa, uint8_t* skip, \
                                   cudaStream_t st); \
  cudaError_t launch_prep_segments_packed(const double* in, int64_t ldIn, const uint8_t* extSeg, int64_t numSeg, \
                                          int64_t npad, double* soa, uint8_t* skip, cudaStream_t st); \
  int64_t segseg_band_end(int64_t J0, int64_t nt, int64_t capSlots); \
  cudaError_t launch_segseg_all_f64(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad, \
                                    double* partial, double* out, int64_t numSeg, unsigned long long* counters, \
                                    cudaStream_t st, int64_t capSlots); \
  cudaError_t launch_segseg_rows_f64(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad, \
                                     const int64_t* rows, int64_t nRows, double* partial, double* out, \
                                     unsigned long long* counters, cudaStream_t st); \
  cudaError_t launch_sigma_f64(const KConsts& K, const double* soa, int64_t npad, int64_t nSeg, const double* x0, \
                               int64_t M, double* sigma, cudaStream_t st); \
  cudaError_t launch_reduce_all(const double* partial, int64_t npad, int64_t numSeg, double* out, cudaStream_t st); \
  cudaError_t launch_reduce_band(const double* partial, int64_t J0, int64_t J1, int64_t numSeg, double* out, \
                                 cudaStream_t st); \
  cudaError_t launch_reduce_rows(const double* partial, int64_t npad, int64_t nRows, double* out, cudaStream_t st); \
  cudaError_t preload_all_f64();

namespace strict {
DDD_F64_DECLS
}
namespace fast {
DDD_F64_DECLS
}

// segseg_df.cu: the general branch in df64 (pairs of FP32) on the FP32 pipes
// (form 0), or df64 corner integrals with FP32 assembly (form 1, mixed);
// near-parallel pairs and the cross-tile reduction in FP64 (strict).
size_t segseg_df_soa_bytes(int64_t npad);
cudaError_t launch_prep_df(const double* soa, int64_t npad, float* soadf, cudaStream_t st);
cudaError_t launch_segseg_all_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                 int64_t npad, double* partial, double* out, int64_t numSeg,
                                 unsigned long long* counters, cudaStream_t st, int form, int64_t capSlots);
cudaError_t launch_segseg_rows_df(const KConsts& K, const double* soa, const float* soadf, const uint8_t* skip,
                                  int64_t npad, const int64_t* rows, int64_t nRows, double* partial, double* out,
                                  unsigned long long* counters, cudaStream_t st, int form);
// σ̃ in the mixed form: geometry and endpoint differences in df64, assembly in FP32.
cudaError_t launch_sigma_mixed(const KConsts& K, const float* soadf, int64_t npad, int64_t nSeg, const double* x0,
                               int64_t M, double* sigma, cudaStream_t st);

// segseg_f64fast.cu: the FP64 tile kernels with the fast general branch
// (pair_f64fast.cuh: fewer divisions, table-driven log/atan, explicit FMAs);
// near-parallel branch, segment preparation and reductions strict.
// The fast FP64 form of σ̃ (sigma_fx.cu).
cudaError_t launch_sigma_fx(const KConsts& K, const double* soa, int64_t npad, int64_t nSeg, const double* x0,
                            int64_t M, double* sigma, cudaStream_t st);
cudaError_t launch_segseg_all_fx(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                 double* partial, double* out, int64_t numSeg, unsigned long long* counters,
                                 cudaStream_t st, int64_t capSlots);
cudaError_t launch_segseg_rows_fx(const KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                                  const int64_t* rows, int64_t nRows, double* partial, double* out,
                                  unsigned long long* counters, cudaStream_t st);

// tc_gemm.cu: tcgen05 GEMM, D = A * B^T (both K-major), A and B both BF16 or both F16.
size_t tc_gemm_smem_bytes(int N);
cudaError_t launch_tc_gemm_bf16(int M, int N, int K, const void* A, const void* B, float* D, int* err,
                                cudaStream_t st);
cudaError_t launch_tc_gemm_f16(int M, int N, int K, const void* A, const void* B, float* D, int* err,
                               cudaStream_t st);
// One warp waiting (bounded by max_clocks) on an mbarrier that receives its
// arrival only when `arrive` != 0; *err = 1 when the wait ran out.
cudaError_t launch_bounded_wait_probe(long long max_clocks, int arrive, int* err, cudaStream_t st);

// surrogate_data.cu: features and exact scaled targets of a pair list.
cudaError_t launch_pair_data(const KConsts& K, const double* soa, int64_t npad, const int32_t* pairs, int64_t P,
                             void* X, float* Bp, float* T, double* F, cudaStream_t st);

// self_force.cu: per-segment self force (node 2) and PK force, strict FP64.
struct SelfK {
  double a, aSq, mu4pi, nuOmNuInv, omNuInv, Ec;
};
cudaError_t launch_self_pk(const SelfK& K, const double* coord, const double* bVec, const int64_t* segIdx, int64_t ld,
                           const uint8_t* ext, int64_t nExt, const int64_t* rows, int64_t n, const double* sigmaHat,
                           double* S, double* PK, cudaStream_t st);

// mobility.cu: BCC node velocities, strict FP64.
struct MobK {
  double sigmaPN, edge, screw, climb, line;
};
cudaError_t launch_mobility_bcc(const MobK& P, const double* coord, const double* bVec, const int64_t* links,
                                const int64_t* conn, int64_t ldConn, const double* segForce, const int64_t* rows,
                                int64_t n, double* nodeForce, double* nodeVel, cudaStream_t st);

// collision.cu: detectCollision and minimumDistance, strict FP64.  type: 0
// none, 1 hinge, 2 two-line; indices 1-based; L1, L2 as the reference returns
// them (its last evaluated pair), pair* of the reported pair.
struct CollisionOut {
  int32_t collision, type;
  int64_t n1s1, n2s1, n1s2, n2s2, s1, s2;
  double L1, L2, pairDistSq, pairL1, pairL2;
};
struct CollisionPlan;
CollisionPlan* collision_plan_create();
void collision_plan_destroy(CollisionPlan* p);
// Device arrays in the network's layout (coord / vel / bVec 3 x n, links 2 x n
// and conn ldConn x n 1-based); skip: nSkip canonical (a <= b), sorted pairs;
// box: min xyz, max xyz of the node coordinates; maxAbs: max |coordinate|.
// Writes *out (host) and synchronises st.
cudaError_t collision_detect(CollisionPlan* P, double cd2, const double* coord, const double* vel, const int32_t* label,
                             const int64_t* links, const double* bVec, const int64_t* conn, int64_t ldConn,
                             int64_t numNode, int64_t numSeg, const int64_t* skip, int64_t nSkip, const double box[6],
                             double maxAbs, CollisionOut* out, cudaEvent_t e0, cudaEvent_t e1, cudaStream_t st);
// pts: 3 x 8 x n (x0, x1, y0, y1, vx0, vx1, vy0, vy1), out 4 x n.
cudaError_t launch_minimum_distance(const double* pts, int64_t n, double* out, cudaStream_t st);

// Grow-only device buffer (12.5 % headroom on growth), freed on release() or
// destruction; used by every file that keeps device scratch between calls.
struct GrowBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    release();
    const size_t want = bytes + bytes / 8 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class X> X* as() const { return reinterpret_cast<X*>(p); }
  GrowBuf() = default;
  GrowBuf(const GrowBuf&) = delete;
  GrowBuf& operator=(const GrowBuf&) = delete;
  ~GrowBuf() { release(); }
};

// u_tilde.cu: calc_uTilde's displacements at numPoints points (u: host, 3 x
// numPoints).  The host arrays drive the segment pass; the *Dev copies feed the
// kernels.  Mesh: closure point C, volume box [lo, hi] widened by tol, face
// normals / midpoints (3 x numFaces), projection directions (3 x numNormals).
// Doubles per triangle in the field kernels' table (u_tilde.cu lays it out).
constexpr int kUTriRows = 32;
struct UTildeArgs {
  double omNuInv8pi, om2NuOmNuInv8pi;
  bool fast;  // the reformulated FP64 kernel (u_tilde_fast.cu) instead of the reference's formulas
  double C[3], lo[3], hi[3], tol;
  const double* faceNorm;
  const double* faceMidPt;
  int64_t numFaces;
  const double* normals;
  int64_t numNormals;
  const double* coord;
  const int32_t* label;
  const int64_t* links;
  const double* bVec;
  int64_t numNode, numSeg, numPoints;
  const double* coordDev;
  const int64_t* linksDev;
  const double* bVecDev;
  const double* pointsDev;
};
struct UTildeScratch {
  std::vector<int64_t> order;
  std::vector<double> explicitTri;
  GrowBuf order_d, ex_d, tri_d, u_d, part_d;
  int64_t lastTriangles = 0, lastChunks = 0;
  int sms = 0, occStrict = 0, occFast = 0;
};
cudaError_t u_tilde_compute(const UTildeArgs& a, double* u, cudaEvent_t e0, cudaEvent_t e1, cudaStream_t st,
                            UTildeScratch& S);
int u_field_fast_blocks_per_sm();
// Partial sums part[k][p] over triangle chunk k (K chunks of `chunk`).
cudaError_t launch_u_field_fast(const double* tri, int64_t nTri, int64_t chunk, int64_t K, const double* points,
                                int64_t M, double omNuInv8pi, double om2NuOmNuInv8pi, const double C[3], double* part,
                                cudaStream_t st);

// ddd_api.cu: context accessors for the other C-ABI files.
int ctx_device(const ddd_ctx* c);

// probes.cu
cudaError_t launch_fp64_peak_probe(double* sink, int iters, int blocks, int threads, cudaStream_t st);
cudaError_t launch_fp32_peak_probe(float* sink, int iters, int blocks, int threads, cudaStream_t st);

}  // namespace ddd
