// Batched seg-seg force: many independent networks of uneven sizes in one
// persistent launch, replayed from a captured CUDA graph, with the tile size and
// the work order chosen by a small autotuner.
//
// Layout.  The caller passes all networks concatenated: a packed 9 × totalSeg
// device array (n1, n2, b per segment), network n occupying columns
// [outOff_n, outOff_n + N_n), and gets the forces in the same order
// (3 × 2 × totalSeg).  Internally each network is padded to whole tiles of T
// segments; its tile pairs (I <= J) become work items.  A persistent grid
// (resident CTAs on every SM) takes items from a global counter (one atomicAdd
// per item, no waiting), runs the shared tile body on each and writes the
// item's partial forces to its own slot; a reduction sums each segment's slots
// in a fixed order.  Results are deterministic and equal, bit for bit, to the
// per-network launches with the same tile size and arithmetic.
//
// Arithmetic: DDD_MODE_FP64 (strict), DDD_MODE_FP64_FAST (tile_pol_fx.cuh),
// DDD_MODE_DF64, DDD_MODE_F32C.  The file is compiled with --fmad=false (strict
// FP64 rounding, the fast form's explicit fused operations only, exact df64
// transforms).
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/ddd_gb300.h"
#include "ddd_internal.h"
#include "pair_df.cuh"
#include "pair_f64.cuh"
#include "tile_body.cuh"
#include "tile_pol_df.cuh"
#include "tile_pol_fx.cuh"

namespace ddd {
namespace batch {

template <int FORM>
using PolDFb = PolDF<FORM>;  // tile_pol_df.cuh

// The precision forms read the df64 SoA as well.
bool uses_df(int mode) { return mode == DDD_MODE_DF64 || mode == DDD_MODE_F32C; }

// Padded SoA from the caller's packed 9 × ld array; src[g] = source column or -1.
__global__ void prep_batched(const double* __restrict__ in, int64_t ldIn, const uint8_t* __restrict__ ext,
                             const int32_t* __restrict__ src, int64_t ntot, double* __restrict__ soa,
                             uint8_t* __restrict__ skip) {
  int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= ntot) return;
  const int32_t i = src[g];
  double v[13];
  uint8_t sk = 1;
  if (i >= 0) {
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
    sk = ext ? (ext[i] ? 1 : 0) : 0;
  } else {
#pragma unroll
    for (int k = 0; k < 13; ++k) v[k] = 0.0;
    v[3] = 1.0;
    v[9] = 1.0;
    v[12] = 1.0;
  }
#pragma unroll
  for (int k = 0; k < 13; ++k) soa[k * ntot + g] = v[k];
  skip[g] = sk;
}

// Work item: (slot, first row segment, first column segment, diagonal flag).
template <int T, class P>
__global__ void __launch_bounds__(T, 256 / T)
persistent_tiles(TileArgs A, typename P::Consts KP, const int4* __restrict__ items, int32_t nItems,
                 int32_t* __restrict__ next, double* __restrict__ partial, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& sm = *reinterpret_cast<TileSmemT<T, P>*>(smem_raw);
  __shared__ int32_t s_item;
  for (;;) {
    __syncthreads();  // the previous item's shared memory is no longer read
    if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int32_t w = s_item;
    if (w >= nItems) break;
    const int4 it = items[w];
    tile_body<T, 0, P>(A, KP, sm, it.y, it.z, it.w != 0, nullptr, 0, partial + (int64_t)it.x * 12 * T, counters);
  }
}

// Per segment (unpadded, caller order): sum of its row and column slots in a
// fixed order, as segseg_reduce_all does for one network.
template <int T>
__global__ void reduce_batched(const double* __restrict__ partial, const int32_t* __restrict__ segNet,
                               const int64_t* __restrict__ netTab, int64_t nNet, int64_t totalSeg,
                               double* __restrict__ out) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= totalSeg) return;
  const int32_t n = segNet[s];
  const int64_t outOff = netTab[n], slotBase = netTab[nNet + n], nt = netTab[2 * nNet + n];
  const int64_t loc = s - outOff;
  const int64_t Ab = loc / T;
  const int t = (int)(loc % T);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t Jt = Ab; Jt < nt; ++Jt) {
    const double* p = partial + (slotBase + Jt * (Jt + 1) / 2 + Ab) * 12 * T;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[c * T + t];
  }
  for (int64_t It = 0; It <= Ab; ++It) {
    const double* p = partial + (slotBase + Ab * (Ab + 1) / 2 + It) * 12 * T;
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] += p[(6 + c) * T + t];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) out[6 * s + c] = acc[c];
}

}  // namespace batch
}  // namespace ddd

// ---------------------------------------------------------------------------
// Host side.
namespace {

using namespace ddd;
using namespace ddd::batch;

using DBuf = GrowBuf;

// One (tile size, work order) layout of a batch.
struct Layout {
  int T = 0;
  int order = 0;  // 0 = network order, 1 = networks with the most tiles first
  int64_t ntot = 0, nItems = 0;
  unsigned grid = 0;  // persistent CTAs (resident blocks per SM x SMs, capped by the item count)
  DBuf soa, skip, soadf, partial, items, src, segNet, netTab;
  bool built = false;
  void release() {
    for (DBuf* b : {&soa, &skip, &soadf, &partial, &items, &src, &segNet, &netTab}) b->release();
  }
};

struct Config {
  int T, order;
};

std::mutex g_tune_mu;
std::map<std::string, Config> g_tuned;  // (mode, sizes) -> chosen configuration

}  // namespace

struct ddd_batch {
  int device = 0;
  int mode = DDD_MODE_FP64;
  cudaStream_t own = nullptr;
  std::vector<int64_t> numSeg;
  int64_t totalSeg = 0;
  Layout lay[2][2];  // [T == 64 ? 0 : 1][order]
  Config chosen{128, 1};
  bool tuned = false, tune = false;
  std::vector<double> tuneMs;  // per candidate, in candidate order
  DBuf next, counters;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // Arguments baked into the graph.
  ddd_consts gk{};
  const double* gsegs = nullptr;
  const uint8_t* gext = nullptr;
  double* gforce = nullptr;
  cudaStream_t gstream = nullptr;
  int graphLaunches = 0;
  std::string err;
};

namespace {

cudaError_t prepare(ddd_batch* b, Layout& L);

cudaError_t build_layout(ddd_batch* b, Layout& L, int T, int order) {
  if (L.built) return cudaSuccess;
  L.T = T;
  L.order = order;
  const int64_t nNet = (int64_t)b->numSeg.size();
  std::vector<int64_t> padOff(nNet), outOff(nNet), slotBase(nNet), nt(nNet);
  int64_t ntot = 0, out = 0, slots = 0;
  for (int64_t n = 0; n < nNet; ++n) {
    const int64_t N = b->numSeg[n];
    nt[n] = (N + T - 1) / T;
    padOff[n] = ntot;
    outOff[n] = out;
    slotBase[n] = slots;
    ntot += nt[n] * T;
    out += N;
    slots += nt[n] * (nt[n] + 1) / 2;
  }
  L.ntot = ntot;
  L.nItems = slots;
  std::vector<int32_t> src((size_t)ntot, -1), segNet((size_t)out);
  for (int64_t n = 0; n < nNet; ++n) {
    for (int64_t s = 0; s < b->numSeg[n]; ++s) {
      src[padOff[n] + s] = (int32_t)(outOff[n] + s);
      segNet[outOff[n] + s] = (int32_t)n;
    }
  }
  std::vector<int64_t> netOrder(nNet);
  std::iota(netOrder.begin(), netOrder.end(), 0);
  if (order == 1) std::stable_sort(netOrder.begin(), netOrder.end(), [&](int64_t a, int64_t c) { return nt[a] > nt[c]; });
  std::vector<int4> items;
  items.reserve((size_t)slots);
  for (int64_t n : netOrder) {
    for (int64_t J = 0; J < nt[n]; ++J)
      for (int64_t I = 0; I <= J; ++I)
        items.push_back(make_int4((int)(slotBase[n] + J * (J + 1) / 2 + I), (int)(padOff[n] + I * T),
                                  (int)(padOff[n] + J * T), I == J ? 1 : 0));
  }
  std::vector<int64_t> tab((size_t)(3 * nNet));
  for (int64_t n = 0; n < nNet; ++n) {
    tab[n] = outOff[n];
    tab[nNet + n] = slotBase[n];
    tab[2 * nNet + n] = nt[n];
  }
  cudaError_t e;
  if ((e = L.soa.ensure((size_t)ntot * 13 * sizeof(double))) != cudaSuccess) return e;
  if ((e = L.skip.ensure((size_t)ntot)) != cudaSuccess) return e;
  if (uses_df(b->mode) && (e = L.soadf.ensure((size_t)ntot * 26 * sizeof(float))) != cudaSuccess) return e;
  if ((e = L.partial.ensure((size_t)slots * 12 * T * sizeof(double))) != cudaSuccess) return e;
  if ((e = L.items.ensure(items.size() * sizeof(int4))) != cudaSuccess) return e;
  if ((e = L.src.ensure(src.size() * sizeof(int32_t))) != cudaSuccess) return e;
  if ((e = L.segNet.ensure(segNet.size() * sizeof(int32_t) + 4)) != cudaSuccess) return e;
  if ((e = L.netTab.ensure(tab.size() * sizeof(int64_t) + 8)) != cudaSuccess) return e;
  if (!items.empty() && (e = cudaMemcpy(L.items.p, items.data(), items.size() * sizeof(int4),
                                        cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  if (!src.empty() &&
      (e = cudaMemcpy(L.src.p, src.data(), src.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  if (!segNet.empty() && (e = cudaMemcpy(L.segNet.p, segNet.data(), segNet.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  if (!tab.empty() &&
      (e = cudaMemcpy(L.netTab.p, tab.data(), tab.size() * sizeof(int64_t), cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  if ((e = prepare(b, L)) != cudaSuccess) return e;
  L.built = true;
  return cudaSuccess;
}

KConsts kconsts(const ddd_consts* k) {
  KConsts K;
  K.aSq = k->aSq;
  K.mu4pi = k->mu4pi;
  K.mu8pi = k->mu8pi;
  K.mu4pinu = k->mu4pinu;
  K.nuMu4pinu = k->nuMu4pinu;
  K.mu8piaSq = k->aSq * k->mu8pi;
  K.mu4pinuaSq = k->aSq * k->mu4pinu;
  return K;
}

// Shared-memory attribute and grid size of the persistent kernel, set up outside
// any stream capture.
template <int T, class P>
cudaError_t prepare_persistent(int device, Layout& L) {
  static std::atomic<uint64_t> attr{0};
  const int smem = (int)sizeof(TileSmemT<T, P>);
  cudaError_t e = set_smem_once(persistent_tiles<T, P>, smem, attr);
  if (e != cudaSuccess) return e;
  int sms = 0, per = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, persistent_tiles<T, P>, T, smem);
  if (e != cudaSuccess) return e;
  if (per < 1) per = 1;
  const int64_t want = (int64_t)sms * per;
  L.grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, L.nItems));
  return cudaSuccess;
}

template <int T, class P>
cudaError_t launch_persistent(const TileArgs& A, const typename P::Consts& KP, const Layout& L, int32_t* next,
                              unsigned long long* counters, cudaStream_t st) {
  persistent_tiles<T, P><<<L.grid, T, sizeof(TileSmemT<T, P>), st>>>(A, KP, (const int4*)L.items.p, (int32_t)L.nItems,
                                                                     next, (double*)L.partial.p, counters);
  return cudaGetLastError();
}

// The whole batch on stream st with layout L: counter reset, prep, tiles, reduction.
cudaError_t enqueue(ddd_batch* b, Layout& L, const ddd_consts* k, const double* segs, const uint8_t* ext,
                    double* force, unsigned long long* counters, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(b->next.p, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  const int64_t ntot = L.ntot;
  if (ntot == 0) return cudaSuccess;
  prep_batched<<<(unsigned)((ntot + 255) / 256), 256, 0, st>>>(segs, b->totalSeg, ext, (const int32_t*)L.src.p, ntot,
                                                               (double*)L.soa.p, (uint8_t*)L.skip.p);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (uses_df(b->mode)) {
    if ((e = launch_prep_df((const double*)L.soa.p, ntot, (float*)L.soadf.p, st)) != cudaSuccess) return e;
  }
  const KConsts K = kconsts(k);
  const TileArgs A{K, (const double*)L.soa.p, (const uint8_t*)L.skip.p, ntot, (const float*)L.soadf.p, nullptr};
  int32_t* next = (int32_t*)b->next.p;
  if (b->mode == DDD_MODE_FP64) {
    e = L.T == 64 ? launch_persistent<64, PolF64>(A, PolF64::Consts{}, L, next, counters, st)
                  : launch_persistent<128, PolF64>(A, PolF64::Consts{}, L, next, counters, st);
  } else if (b->mode == DDD_MODE_FP64_FAST) {
    e = L.T == 64 ? launch_persistent<64, PolF64Fast>(A, PolF64Fast::Consts{}, L, next, counters, st)
                  : launch_persistent<128, PolF64Fast>(A, PolF64Fast::Consts{}, L, next, counters, st);
  } else if (b->mode == DDD_MODE_DF64) {
    const PolDFb<0>::Consts KP{kconsts_df(K), kconsts_f(K)};
    e = L.T == 64 ? launch_persistent<64, PolDFb<0>>(A, KP, L, next, counters, st)
                  : launch_persistent<128, PolDFb<0>>(A, KP, L, next, counters, st);
  } else {
    const PolDFb<1>::Consts KP{kconsts_df(K), kconsts_f(K)};
    e = L.T == 64 ? launch_persistent<64, PolDFb<1>>(A, KP, L, next, counters, st)
                  : launch_persistent<128, PolDFb<1>>(A, KP, L, next, counters, st);
  }
  if (e != cudaSuccess) return e;
  const int64_t nNet = (int64_t)b->numSeg.size();
  if (b->totalSeg > 0) {
    if (L.T == 64)
      reduce_batched<64><<<(unsigned)((b->totalSeg + 127) / 128), 128, 0, st>>>(
          (const double*)L.partial.p, (const int32_t*)L.segNet.p, (const int64_t*)L.netTab.p, nNet, b->totalSeg, force);
    else
      reduce_batched<128><<<(unsigned)((b->totalSeg + 127) / 128), 128, 0, st>>>(
          (const double*)L.partial.p, (const int32_t*)L.segNet.p, (const int64_t*)L.netTab.p, nNet, b->totalSeg, force);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

Layout& layout_of(ddd_batch* b, const Config& c) { return b->lay[c.T == 64 ? 0 : 1][c.order]; }

cudaError_t prepare(ddd_batch* b, Layout& L) {
  if (b->mode == DDD_MODE_FP64) return L.T == 64 ? prepare_persistent<64, PolF64>(b->device, L)
                                                 : prepare_persistent<128, PolF64>(b->device, L);
  if (b->mode == DDD_MODE_FP64_FAST) return L.T == 64 ? prepare_persistent<64, PolF64Fast>(b->device, L)
                                                      : prepare_persistent<128, PolF64Fast>(b->device, L);
  if (b->mode == DDD_MODE_DF64) return L.T == 64 ? prepare_persistent<64, PolDFb<0>>(b->device, L)
                                                 : prepare_persistent<128, PolDFb<0>>(b->device, L);
  return L.T == 64 ? prepare_persistent<64, PolDFb<1>>(b->device, L)
                   : prepare_persistent<128, PolDFb<1>>(b->device, L);
}

std::string tune_key(const ddd_batch* b) {
  std::string k = std::to_string(b->mode) + ":";
  for (int64_t n : b->numSeg) k += std::to_string(n) + ",";
  return k;
}

int fail(ddd_batch* b, int code, const std::string& m) {
  b->err = m;
  return code;
}

}  // namespace

extern "C" {

ddd_batch* ddd_batch_create(ddd_ctx* ctx, int64_t nNet, const int64_t* numSeg, int mode, int tune) {
  DDD_NVTX("ddd_batch_create");
  if (!ctx || nNet < 0 || (nNet > 0 && !numSeg)) return nullptr;
  if (mode != DDD_MODE_FP64 && mode != DDD_MODE_FP64_FAST && mode != DDD_MODE_DF64 && mode != DDD_MODE_F32C)
    return nullptr;
  ddd_batch* b = new ddd_batch();
  b->device = ddd::ctx_device(ctx);
  b->mode = mode;
  b->tune = tune != 0;
  b->numSeg.assign(numSeg, numSeg + nNet);
  for (int64_t n : b->numSeg) {
    if (n < 0 || n > (int64_t)1 << 24) {
      delete b;
      return nullptr;
    }
    b->totalSeg += n;
  }
  if (cudaSetDevice(b->device) != cudaSuccess || cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess ||
      b->next.ensure(sizeof(int32_t)) != cudaSuccess || b->counters.ensure(3 * sizeof(unsigned long long)) != cudaSuccess) {
    ddd_batch_destroy(b);
    return nullptr;
  }
  std::lock_guard<std::mutex> g(g_tune_mu);
  auto it = g_tuned.find(tune_key(b));
  if (it != g_tuned.end()) {
    b->chosen = it->second;
    b->tuned = true;
  } else if (!b->tune) {
    b->chosen = Config{128, 1};
    b->tuned = true;
  }
  return b;
}

void ddd_batch_destroy(ddd_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->own) cudaStreamSynchronize(b->own);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto& row : b->lay)
    for (auto& L : row) L.release();
  b->next.release();
  b->counters.release();
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
}

const char* ddd_batch_last_error(const ddd_batch* b) { return b ? b->err.c_str() : "null batch"; }

int ddd_batch_run(ddd_batch* b, const ddd_consts* k, const double* segs, const uint8_t* ext, double* force,
                  void* stream) {
  DDD_NVTX("ddd_batch_run");
  if (!b || !k) return DDD_EINVAL;
  if (b->totalSeg > 0 && (!segs || !force)) return fail(b, DDD_EINVAL, "segs or force is NULL");
  if (!(k->aSq > 0.0)) return fail(b, DDD_EINVAL, "aSq must be > 0");
  cudaError_t e = cudaSetDevice(b->device);
  if (e != cudaSuccess) return fail(b, DDD_EDEVICE, cudaGetErrorString(e));
  cudaStream_t st = stream ? (cudaStream_t)stream : b->own;
  if (b->totalSeg == 0) return DDD_OK;

  // Autotune: each (tile size, work order) timed twice on these inputs.
  if (!b->tuned) {
    const Config cands[4] = {{128, 1}, {128, 0}, {64, 1}, {64, 0}};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    b->tuneMs.clear();
    for (const Config& c : cands) {
      Layout& L = layout_of(b, c);
      if ((e = build_layout(b, L, c.T, c.order)) != cudaSuccess) break;
      float ms = 1e30f;
      for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
        cudaEventRecord(e0, st);
        e = enqueue(b, L, k, segs, ext, force, nullptr, st);
        cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float m = 0;
        cudaEventElapsedTime(&m, e0, e1);
        if (r > 0) ms = std::min(ms, m);
      }
      if (e != cudaSuccess) break;
      b->tuneMs.push_back(ms);
      if (ms < best) {
        best = ms;
        b->chosen = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return fail(b, e == cudaErrorMemoryAllocation ? DDD_ENOMEM : DDD_EDEVICE,
                                      std::string("autotune: ") + cudaGetErrorString(e));
    b->tuned = true;
    {
      std::lock_guard<std::mutex> g(g_tune_mu);
      g_tuned[tune_key(b)] = b->chosen;
    }
    for (int i = 0; i < 2; ++i)
      for (int o = 0; o < 2; ++o)
        if (&b->lay[i][o] != &layout_of(b, b->chosen)) {
          b->lay[i][o].release();
          b->lay[i][o].built = false;
        }
  }

  Layout& L = layout_of(b, b->chosen);
  if ((e = build_layout(b, L, b->chosen.T, b->chosen.order)) != cudaSuccess)
    return fail(b, e == cudaErrorMemoryAllocation ? DDD_ENOMEM : DDD_EDEVICE, cudaGetErrorString(e));

  // Capture the batch once per (arguments, stream); replay afterwards.
  const bool same = b->exec && b->gsegs == segs && b->gext == ext && b->gforce == force && b->gstream == st &&
                    b->gk.aSq == k->aSq && b->gk.mu4pi == k->mu4pi && b->gk.mu8pi == k->mu8pi &&
                    b->gk.mu4pinu == k->mu4pinu && b->gk.nuMu4pinu == k->nuMu4pinu;
  if (!same) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(b, DDD_EDEVICE, std::string("begin capture: ") + cudaGetErrorString(e));
    cudaError_t eq = enqueue(b, L, k, segs, ext, force, nullptr, st);
    e = cudaStreamEndCapture(st, &b->graph);
    if (eq != cudaSuccess) return fail(b, DDD_EDEVICE, std::string("capture: ") + cudaGetErrorString(eq));
    if (e != cudaSuccess) return fail(b, DDD_EDEVICE, std::string("end capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) return fail(b, DDD_EDEVICE, std::string("instantiate: ") + cudaGetErrorString(e));
    b->gk = *k;
    b->gsegs = segs;
    b->gext = ext;
    b->gforce = force;
    b->gstream = st;
  }
  e = cudaGraphLaunch(b->exec, st);
  if (e != cudaSuccess) return fail(b, DDD_EDEVICE, std::string("graph launch: ") + cudaGetErrorString(e));
  ++b->graphLaunches;
  return DDD_OK;
}

int ddd_batch_info(const ddd_batch* b, ddd_batch_info_t* out) {
  if (!b || !out) return DDD_EINVAL;
  out->tile = b->chosen.T;
  out->order = b->chosen.order;
  out->work_items = 0;
  const Layout& L = const_cast<ddd_batch*>(b)->lay[b->chosen.T == 64 ? 0 : 1][b->chosen.order];
  out->work_items = L.nItems;
  out->total_segments = b->totalSeg;
  out->graph_launches = b->graphLaunches;
  for (int i = 0; i < 4; ++i) out->tune_ms[i] = i < (int)b->tuneMs.size() ? b->tuneMs[i] : -1.0;
  return DDD_OK;
}

}  // extern "C"
