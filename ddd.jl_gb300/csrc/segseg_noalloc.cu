// Allocation-free entry point: the all-pairs FP64 seg-seg force of
// ddd_segseg_force_device, with its scratch (packed segments, skip flags,
// per-tile partial forces) in a fixed, file-scope device array instead of
// context-owned cudaMalloc'd buffers.
//
// Who needs it: callers that must not allocate device memory from inside this
// library — an application whose device memory is owned by its own pool
// allocator (a framework's caching allocator that has reserved the GPU), or a
// time-stepping loop that cannot afford the device-wide synchronisation that
// cudaMalloc/cudaFree imply.  They pass device inputs and outputs; this entry
// point calls no cudaMalloc, cudaFree or other allocating routine.
//
// Limits and sharing:
//   * at most DDD_NOALLOC_MAX_SEGMENTS segments (larger sizes are rejected);
//   * the scratch array (about 6.9 MB) is device memory that the CUDA driver
//     reserves when it loads this file's module on a device, and the force
//     kernels' code is loaded the same way.  Under CUDA's default lazy module
//     loading that happens inside the first call on that device (the
//     cudaGetSymbolAddress and kernel look-ups below), not when the library
//     loads; with CUDA_MODULE_LOADING=EAGER it happens when the device's
//     context is created.  The memory stays reserved until the process exits.
//     A caller whose pool reserves the GPU should therefore make one call on
//     each device during set-up, before the pool reserves its memory: a call
//     with numSeg = 0 does only that set-up (module loads, kernel attribute,
//     address lookup) and launches nothing;
//   * every call shares the array and it keeps the last call's contents; every
//     scratch element this call reads is written earlier in the same call, so
//     nothing needs clearing, and calls that overlap on the GPU (two streams,
//     or two host threads) race on it: serialise them;
//   * the first call on a device looks up the array's device address (once per
//     device, that device current); make that first call before any stream
//     capture that contains later calls.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/ddd_gb300.h"
#include "ddd_internal.h"
#include "pair_f64.cuh"

namespace {

constexpr int64_t kTile = 128;                            // tile of the all-pairs kernel
constexpr int64_t kMaxSeg = DDD_NOALLOC_MAX_SEGMENTS;     // 4096
constexpr int64_t kMaxTiles = kMaxSeg / kTile;            // 32
constexpr size_t kSoaBytes = (size_t)kMaxSeg * 13 * sizeof(double);
constexpr size_t kSkipBytes = ((size_t)kMaxSeg + 255) / 256 * 256;
constexpr size_t kPartialBytes = (size_t)(kMaxTiles * (kMaxTiles + 1) / 2) * 12 * kTile * sizeof(double);
constexpr size_t kScratchBytes = kSoaBytes + kSkipBytes + kPartialBytes;

// The scratch.  In host code this name is only a host-side stand-in: its device
// address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_mu;

// Device address of g_scratch on the current device (looked up once per device,
// with that device current), the force kernels loaded there.
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DDD_EDEVICE;
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) return DDD_EDEVICE;
    if (ddd::strict::preload_all_f64() != cudaSuccess) return DDD_EDEVICE;
    g_scratch_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[dev]);
  return DDD_OK;
}

}  // namespace

extern "C" {

int ddd_segseg_force_device_noalloc(const ddd_consts* k, const double* segs, int64_t ldSegs, const uint8_t* ext,
                                    int64_t numSeg, double* force, void* stream) {
  if (!k || numSeg < 0 || ldSegs < numSeg) return DDD_EINVAL;
  if (numSeg > kMaxSeg) return DDD_ETOOBIG;
  if (numSeg > 0 && (!segs || !force)) return DDD_EINVAL;
  const double v[5] = {k->aSq, k->mu4pi, k->mu8pi, k->mu4pinu, k->nuMu4pinu};
  for (double x : v)
    if (!std::isfinite(x)) return DDD_ENONFINITE;
  if (!(k->aSq > 0.0)) return DDD_EINVAL;
  // Per-device set-up first, so that a numSeg = 0 call loads the scratch.
  unsigned char* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  if (numSeg == 0) return DDD_OK;
  ddd::KConsts K;
  K.aSq = k->aSq;
  K.mu4pi = k->mu4pi;
  K.mu8pi = k->mu8pi;
  K.mu4pinu = k->mu4pinu;
  K.nuMu4pinu = k->nuMu4pinu;
  K.mu8piaSq = k->aSq * k->mu8pi;
  K.mu4pinuaSq = k->aSq * k->mu4pinu;

  double* soa = reinterpret_cast<double*>(base);
  uint8_t* skip = base + kSoaBytes;
  double* partial = reinterpret_cast<double*>(base + kSoaBytes + kSkipBytes);

  const int64_t npad = ddd::strict::segseg_npad(numSeg);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = ddd::strict::launch_prep_segments_packed(segs, ldSegs, ext, numSeg, npad, soa, skip, st);
  if (e == cudaSuccess)
    e = ddd::strict::launch_segseg_all_f64(K, soa, skip, npad, partial, force, numSeg, nullptr, st, INT64_MAX);
  return e == cudaSuccess ? DDD_OK : DDD_EDEVICE;
}

}  // extern "C"
