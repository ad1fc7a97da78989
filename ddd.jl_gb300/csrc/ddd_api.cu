// C-ABI layer of libddd_gb300.so: validation, device buffers, copies, launch
// sequencing.  Declared in include/ddd_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ddd_gb300.h"
#include "ddd_internal.h"
#include "net_check.h"
#include "pair_f64.cuh"

namespace {

std::string g_create_error;
std::mutex g_create_mu;

using DevBuf = ddd::GrowBuf;

}  // namespace

struct ddd_ctx {
  int device = 0;
  int mode = DDD_MODE_FP64;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::mutex mu;
  std::string err;
  DevBuf coord, bvec, segidx, ext, soa, soadf, skip, partial, out, rows, x0, sigma, counters, probe, errflag;
  DevBuf links, conn, segforce;  // mobility inputs
  DevBuf vel, label, skippairs;  // collision inputs
  ddd::CollisionPlan* coll = nullptr;
  DevBuf upoints;  // calc_uTilde evaluation points
  ddd::UTildeScratch* ut = nullptr;
  std::vector<double> hostTmp;
  double lastKernelMs = 0.0;  // device time of the last self-force / mobility kernel
  int64_t partialLimit = 0;   // bytes of all-pairs partial sums; 0: kDefaultPartialLimit
};

int ddd::ctx_device(const ddd_ctx* c) { return c->device; }

namespace {

int fail(ddd_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(ddd_ctx* c, cudaError_t e, const char* where) {
  std::string m = std::string(where) + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e);
  return fail(c, e == cudaErrorMemoryAllocation ? DDD_ENOMEM : DDD_EDEVICE, m);
}

#define CK(call, where)                              \
  do {                                               \
    cudaError_t _e = (call);                         \
    if (_e != cudaSuccess) return cuda_fail(ctx, _e, where); \
  } while (0)

// FP64 kernel variant of the context's mode.  Segment preparation (direction
// and inverse length) always uses the strict build, so t and 1/|l| are the
// reference's values in both modes.
bool use_fma(const ddd_ctx* c) { return c->mode == DDD_MODE_FP64_FMA; }
bool use_fx(const ddd_ctx* c) { return c->mode == DDD_MODE_FP64_FAST; }
bool use_df(const ddd_ctx* c) { return c->mode == DDD_MODE_DF64 || c->mode == DDD_MODE_F32C; }
int df_form(const ddd_ctx* c) { return c->mode == DDD_MODE_F32C ? 1 : 0; }

// For the df64 / f32c modes the df64 copy of the segment SoA is built first (ctx->soadf).
cudaError_t prep_df_if_needed(ddd_ctx* c, int64_t npad, cudaStream_t st) {
  if (!use_df(c)) return cudaSuccess;
  cudaError_t e = c->soadf.ensure(ddd::segseg_df_soa_bytes(npad));
  if (e != cudaSuccess) return e;
  return ddd::launch_prep_df(c->soa.as<double>(), npad, c->soadf.as<float>(), st);
}

// All-pairs partial sums: 16 GiB by default.  Below that every tile pair has
// its slot (one tile launch, one reduction); above it the launchers run bands
// of tile columns through a buffer of the limit's size.
constexpr int64_t kDefaultPartialLimit = (int64_t)16 << 30;

// Slots to allocate for npad segments: all nt(nt+1)/2 when they fit in the
// context's limit, else as many as the limit holds, at least one column (nt).
int64_t partial_slots(const ddd_ctx* c, int64_t npad) {
  const int64_t tile = ddd::strict::segseg_npad(1);
  const int64_t slotBytes = (int64_t)ddd::strict::segseg_partial_bytes_all(tile);
  const int64_t nt = npad / tile, all = nt * (nt + 1) / 2;
  const int64_t cap = (c->partialLimit ? c->partialLimit : kDefaultPartialLimit) / slotBytes;
  return cap >= all ? all : (cap < nt ? nt : cap);
}

size_t partial_bytes(const ddd_ctx* c, int64_t npad) {
  return (size_t)partial_slots(c, npad) * ddd::strict::segseg_partial_bytes_all(ddd::strict::segseg_npad(1));
}

cudaError_t run_segseg_all(ddd_ctx* c, const ddd::KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                           double* partial, double* out, int64_t numSeg, unsigned long long* cnt, cudaStream_t st) {
  const int64_t cap = partial_slots(c, npad);
  if (use_df(c)) {
    cudaError_t e = prep_df_if_needed(c, npad, st);
    if (e != cudaSuccess) return e;
    return ddd::launch_segseg_all_df(K, soa, c->soadf.as<float>(), skip, npad, partial, out, numSeg, cnt, st,
                                     df_form(c), cap);
  }
  if (use_fx(c)) return ddd::launch_segseg_all_fx(K, soa, skip, npad, partial, out, numSeg, cnt, st, cap);
  return use_fma(c) ? ddd::fast::launch_segseg_all_f64(K, soa, skip, npad, partial, out, numSeg, cnt, st, cap)
                    : ddd::strict::launch_segseg_all_f64(K, soa, skip, npad, partial, out, numSeg, cnt, st, cap);
}

// Index rows per launch: all of them when their partial sums (one block of
// 6 x TILE doubles per row tile and column tile) fit in the context's limit,
// else whole row tiles up to the limit, at least one.  Rows are independent,
// so chunking changes no bit of the result.
int64_t rows_per_chunk(const ddd_ctx* c, int64_t npad, int64_t nRows) {
  const int64_t tile = ddd::strict::segseg_npad(1);
  const int64_t perTile = (int64_t)ddd::strict::segseg_partial_bytes_rows(tile, npad);  // one row tile
  const int64_t limit = c->partialLimit ? c->partialLimit : kDefaultPartialLimit;
  const int64_t tiles = limit / perTile;
  const int64_t chunk = (tiles < 1 ? 1 : tiles) * tile;
  return chunk < nRows ? chunk : nRows;
}

cudaError_t run_segseg_rows(ddd_ctx* c, const ddd::KConsts& K, const double* soa, const uint8_t* skip, int64_t npad,
                            const int64_t* rows, int64_t nRows, double* partial, double* out,
                            unsigned long long* cnt, cudaStream_t st) {
  if (use_df(c)) {
    cudaError_t e = prep_df_if_needed(c, npad, st);
    if (e != cudaSuccess) return e;
  }
  const int64_t chunk = rows_per_chunk(c, npad, nRows);
  for (int64_t r0 = 0; r0 < nRows; r0 += chunk) {
    const int64_t n = nRows - r0 < chunk ? nRows - r0 : chunk;
    const cudaError_t e =
        use_df(c) ? ddd::launch_segseg_rows_df(K, soa, c->soadf.as<float>(), skip, npad, rows + r0, n, partial,
                                               out + 6 * r0, cnt, st, df_form(c))
        : use_fx(c)  ? ddd::launch_segseg_rows_fx(K, soa, skip, npad, rows + r0, n, partial, out + 6 * r0, cnt, st)
        : use_fma(c) ? ddd::fast::launch_segseg_rows_f64(K, soa, skip, npad, rows + r0, n, partial, out + 6 * r0, cnt,
                                                         st)
                     : ddd::strict::launch_segseg_rows_f64(K, soa, skip, npad, rows + r0, n, partial, out + 6 * r0,
                                                           cnt, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t run_sigma(ddd_ctx* c, const ddd::KConsts& K, const double* soa, int64_t npad, int64_t nSeg,
                      const double* x0, int64_t M, double* sigma, cudaStream_t st) {
  if (use_df(c)) {  // both precision modes: the mixed σ̃ form
    cudaError_t e = prep_df_if_needed(c, npad, st);
    if (e != cudaSuccess) return e;
    return ddd::launch_sigma_mixed(K, c->soadf.as<float>(), npad, nSeg, x0, M, sigma, st);
  }
  if (use_fx(c)) return ddd::launch_sigma_fx(K, soa, npad, nSeg, x0, M, sigma, st);
  return use_fma(c) ? ddd::fast::launch_sigma_f64(K, soa, npad, nSeg, x0, M, sigma, st)
                    : ddd::strict::launch_sigma_f64(K, soa, npad, nSeg, x0, M, sigma, st);
}


int check_consts(ddd_ctx* ctx, const ddd_consts* k, ddd::KConsts& K) {
  if (!k) return fail(ctx, DDD_EINVAL, "consts is NULL");
  const double v[5] = {k->aSq, k->mu4pi, k->mu8pi, k->mu4pinu, k->nuMu4pinu};
  for (double x : v)
    if (!std::isfinite(x)) return fail(ctx, DDD_ENONFINITE, "non-finite material/core constant");
  if (!(k->aSq > 0.0)) return fail(ctx, DDD_EINVAL, "aSq (coreRadSq) must be > 0");
  K.aSq = k->aSq;
  K.mu4pi = k->mu4pi;
  K.mu8pi = k->mu8pi;
  K.mu4pinu = k->mu4pinu;
  K.nuMu4pinu = k->nuMu4pinu;
  K.mu8piaSq = k->aSq * k->mu8pi;      // DislocationForces.jl:681
  K.mu4pinuaSq = k->aSq * k->mu4pinu;  // DislocationForces.jl:682
  return DDD_OK;
}

// Checks one segIdx row (0-based row r): net_check.h.
int check_row(ddd_ctx* ctx, const double* coord, int64_t coordCols, const double* bVec, int64_t bVecCols,
              const int64_t* segIdx, int64_t ld, int64_t r) {
  std::string msg;
  const int rc = ddd::check_segment_row(coord, coordCols, bVec, bVecCols, segIdx, ld, r, msg);
  return rc ? fail(ctx, rc, msg) : DDD_OK;
}

int check_network(ddd_ctx* ctx, const double* coord, int64_t coordCols, const double* bVec, int64_t bVecCols,
                  const int64_t* segIdx, int64_t ld, int64_t numSeg) {
  if (numSeg < 0 || coordCols < 0 || bVecCols < 0 || ld < 0) return fail(ctx, DDD_EINVAL, "negative size");
  if (numSeg > ld) return fail(ctx, DDD_EINVAL, "numSeg exceeds the rows of segIdx (ldSegIdx)");
  if (numSeg > 0 && (!coord || !bVec || !segIdx)) return fail(ctx, DDD_EINVAL, "network array is NULL");
  for (int64_t r = 0; r < numSeg; ++r) {
    int rc = check_row(ctx, coord, coordCols, bVec, bVecCols, segIdx, ld, r);
    if (rc) return rc;
  }
  return DDD_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// Uploads the network and builds the packed SoA; returns npad.
int upload_network(ddd_ctx* ctx, const double* coord, int64_t coordCols, const double* bVec, int64_t bVecCols,
                   const int64_t* segIdx, int64_t ld, const uint8_t* extSeg, int64_t numSeg, int64_t& npad,
                   int64_t& h2d) {
  npad = ddd::strict::segseg_npad(numSeg);
  const size_t cB = (size_t)coordCols * 3 * sizeof(double), bB = (size_t)bVecCols * 3 * sizeof(double);
  const size_t sB = (size_t)ld * 3 * sizeof(int64_t), eB = extSeg ? (size_t)numSeg : 0;
  CK(ctx->coord.ensure(cB), "alloc coord");
  CK(ctx->bvec.ensure(bB), "alloc bVec");
  CK(ctx->segidx.ensure(sB), "alloc segIdx");
  if (eB) CK(ctx->ext.ensure(eB), "alloc extSeg");
  CK(ctx->soa.ensure(ddd::strict::segseg_soa_bytes(npad)), "alloc segment SoA");
  CK(ctx->skip.ensure((size_t)npad), "alloc skip flags");
  CK(cudaMemcpyAsync(ctx->coord.p, coord, cB, cudaMemcpyHostToDevice, ctx->stream), "copy coord");
  CK(cudaMemcpyAsync(ctx->bvec.p, bVec, bB, cudaMemcpyHostToDevice, ctx->stream), "copy bVec");
  CK(cudaMemcpyAsync(ctx->segidx.p, segIdx, sB, cudaMemcpyHostToDevice, ctx->stream), "copy segIdx");
  if (eB) CK(cudaMemcpyAsync(ctx->ext.p, extSeg, eB, cudaMemcpyHostToDevice, ctx->stream), "copy extSeg");
  h2d += (int64_t)(cB + bB + sB + eB);
  CK(ddd::strict::launch_prep_segments(ctx->coord.as<double>(), ctx->bvec.as<double>(), ctx->segidx.as<int64_t>(), ld,
                               eB ? ctx->ext.as<uint8_t>() : nullptr, numSeg, npad, ctx->soa.as<double>(),
                               ctx->skip.as<uint8_t>(), ctx->stream),
     "prep_segments");
  return DDD_OK;
}

// Shared body of ddd_segseg_force / _inplace: computes into ctx->hostTmp
// (6 × (numSeg or nIdx)).
int segseg_compute(ddd_ctx* ctx, const ddd_consts* k, const double* coord, int64_t coordCols, const double* bVec,
                   int64_t bVecCols, const int64_t* segIdx, int64_t ld, const uint8_t* extSeg, int64_t numSeg,
                   const int64_t* idx, int64_t nIdx, ddd_report* rep) {
  ddd::KConsts K;
  int rc = check_consts(ctx, k, K);
  if (rc) return rc;
  rc = check_network(ctx, coord, coordCols, bVec, bVecCols, segIdx, ld, numSeg);
  if (rc) return rc;
  const bool rowsMode = idx != nullptr;
  if (rowsMode) {
    if (nIdx < 0) return fail(ctx, DDD_EINVAL, "nIdx < 0");
    for (int64_t q = 0; q < nIdx; ++q)
      if (idx[q] < 1 || idx[q] > numSeg) {
        char buf[96];
        snprintf(buf, sizeof buf, "idx[%lld] = %lld outside 1..numSeg=%lld", (long long)q, (long long)idx[q],
                 (long long)numSeg);
        return fail(ctx, DDD_ERANGE, buf);
      }
  }
  const int64_t nOut = rowsMode ? nIdx : numSeg;
  ctx->hostTmp.assign((size_t)nOut * 6, 0.0);
  if (rep) memset(rep, 0, sizeof *rep);
  if (nOut == 0 || numSeg == 0) return DDD_OK;

  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  int64_t h2d = 0, npad = 0;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  rc = upload_network(ctx, coord, coordCols, bVec, bVecCols, segIdx, ld, extSeg, numSeg, npad, h2d);
  if (rc) return rc;
  CK(ctx->counters.ensure(3 * sizeof(unsigned long long)), "alloc counters");
  CK(cudaMemsetAsync(ctx->counters.p, 0, 3 * sizeof(unsigned long long), ctx->stream), "memset counters");
  CK(ctx->out.ensure((size_t)nOut * 6 * sizeof(double)), "alloc output");
  if (!rowsMode) {
    CK(ctx->partial.ensure(partial_bytes(ctx, npad)), "alloc partial sums");
    CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
    CK(run_segseg_all(ctx, K, ctx->soa.as<double>(), ctx->skip.as<uint8_t>(), npad, ctx->partial.as<double>(),
                                  ctx->out.as<double>(), numSeg, ctx->counters.as<unsigned long long>(), ctx->stream),
       "segseg_all_f64");
  } else {
    std::vector<int64_t> rows0((size_t)nIdx);
    for (int64_t q = 0; q < nIdx; ++q) rows0[q] = idx[q] - 1;
    CK(ctx->rows.ensure((size_t)nIdx * sizeof(int64_t)), "alloc rows");
    CK(cudaMemcpyAsync(ctx->rows.p, rows0.data(), (size_t)nIdx * sizeof(int64_t), cudaMemcpyHostToDevice,
                       ctx->stream),
       "copy idx");
    h2d += nIdx * (int64_t)sizeof(int64_t);
    const int64_t chunkRows = rows_per_chunk(ctx, npad, nIdx);
    CK(ctx->partial.ensure(ddd::strict::segseg_partial_bytes_rows(chunkRows, npad)), "alloc partial sums");
    CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
    CK(run_segseg_rows(ctx, K, ctx->soa.as<double>(), ctx->skip.as<uint8_t>(), npad, ctx->rows.as<int64_t>(),
                                   nIdx, ctx->partial.as<double>(), ctx->out.as<double>(),
                                   ctx->counters.as<unsigned long long>(), ctx->stream),
       "segseg_rows_f64");
  }
  CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
  unsigned long long cnt[3] = {0, 0, 0};
  CK(cudaMemcpyAsync(ctx->hostTmp.data(), ctx->out.p, (size_t)nOut * 6 * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream),
     "copy forces");
  CK(cudaMemcpyAsync(cnt, ctx->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, ctx->stream), "copy counters");
  CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
  CK(cudaStreamSynchronize(ctx->stream), "segseg_force");
  if (rep) {
    rep->pairs_general = (int64_t)cnt[0];
    rep->pairs_parallel = (int64_t)cnt[1];
    rep->core_sides = (int64_t)cnt[2];
    rep->kernel_ms = elapsed(ctx->ev[1], ctx->ev[2]);
    rep->total_ms = elapsed(ctx->ev[0], ctx->ev[3]);
    rep->h2d_bytes = h2d;
    rep->d2h_bytes = nOut * 6 * (int64_t)sizeof(double);
  }
  return DDD_OK;
}

}  // namespace

extern "C" {

int ddd_version(void) { return 100; }

ddd_ctx* ddd_create(int device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  auto bad = [&](const std::string& m) -> ddd_ctx* {
    std::lock_guard<std::mutex> g(g_create_mu);
    g_create_error = m;
    return nullptr;
  };
  if (e != cudaSuccess) return bad(std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
  if (device < 0 || device >= n) return bad("no CUDA device " + std::to_string(device));
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return bad(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  ddd_ctx* c = new ddd_ctx();
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
  if (e != cudaSuccess) {
    ddd_destroy(c);
    return bad(std::string("stream/event creation: ") + cudaGetErrorString(e));
  }
  return c;
}

void ddd_destroy(ddd_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (DevBuf* b : {&c->links, &c->conn, &c->segforce, &c->vel, &c->label, &c->skippairs}) b->release();
  if (c->coll) ddd::collision_plan_destroy(c->coll);
  delete c->ut;
  c->upoints.release();
  for (DevBuf* b : {&c->coord, &c->bvec, &c->segidx, &c->ext, &c->soa, &c->soadf, &c->skip, &c->partial, &c->out, &c->rows,
                    &c->x0, &c->sigma, &c->counters, &c->probe, &c->errflag})
    b->release();
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* ddd_last_error(const ddd_ctx* c) {
  if (!c) return g_create_error.c_str();
  return c->err.c_str();
}

double ddd_last_kernel_ms(const ddd_ctx* c) { return c ? c->lastKernelMs : 0.0; }

int ddd_segseg_force(ddd_ctx* ctx, const ddd_consts* k, const double* coord, int64_t coordCols, const double* bVec,
                     int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx, const uint8_t* extSeg,
                     int64_t numSeg, const int64_t* idx, int64_t nIdx, double* force, ddd_report* rep) {
  DDD_NVTX("ddd_segseg_force");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  const int64_t nOut = idx ? nIdx : numSeg;
  if (nOut > 0 && !force) return fail(ctx, DDD_EINVAL, "force is NULL");
  int rc = segseg_compute(ctx, k, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx, rep);
  if (rc) return rc;
  if (nOut > 0) memcpy(force, ctx->hostTmp.data(), (size_t)nOut * 6 * sizeof(double));
  return DDD_OK;
}

}  // extern "C"

namespace {

// Adds the seg-seg result in ctx->hostTmp into segForce the way
// calcSegSegForce! does.
void add_segseg_inplace(ddd_ctx* ctx, const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx,
                        double* segForce) {
  const double* F = ctx->hostTmp.data();
  if (!idx) {
    for (int64_t q = 0; q < 6 * numSeg; ++q) segForce[q] += F[q];
  } else {
    // calcSegSegForce!'s idx loop (DislocationForces.jl:640-667): skip external,
    // add into column idx[k]; a repeated index adds again.
    for (int64_t q = 0; q < nIdx; ++q) {
      const int64_t i = idx[q] - 1;
      if (extSeg && extSeg[i]) continue;
      for (int c = 0; c < 6; ++c) segForce[6 * i + c] += F[6 * q + c];
    }
  }
}

// Self force on node 2 (S) and, with sigmaHat, the PK force of each entry of
// idx (or of every segment), on the GPU (self_force.cu), into S and PK (3 × n
// each; PK left empty without sigmaHat).
int self_pk_compute(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                    int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ld,
                    const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx, const double* sigmaHat,
                    std::vector<double>& S, std::vector<double>& PK) {
  ddd::KConsts K;
  int rc = check_consts(ctx, k, K);
  if (rc) return rc;
  if (!sp) return fail(ctx, DDD_EINVAL, "self-force parameters are NULL");
  if (!std::isfinite(sp->coreRad) || !std::isfinite(sp->coreEnergy) || !std::isfinite(sp->nu))
    return fail(ctx, DDD_ENONFINITE, "non-finite self-force parameter");
  if (!(sp->coreRad > 0.0) || !(sp->nu < 1.0)) return fail(ctx, DDD_EINVAL, "coreRad must be > 0 and nu < 1");
  rc = check_network(ctx, coord, coordCols, bVec, bVecCols, segIdx, ld, numSeg);
  if (rc) return rc;
  if (idx) {
    if (nIdx < 0) return fail(ctx, DDD_EINVAL, "nIdx < 0");
    for (int64_t q = 0; q < nIdx; ++q)
      if (idx[q] < 1 || idx[q] > numSeg) {
        char buf[96];
        snprintf(buf, sizeof buf, "idx[%lld] = %lld outside 1..numSeg=%lld", (long long)q, (long long)idx[q],
                 (long long)numSeg);
        return fail(ctx, DDD_ERANGE, buf);
      }
  }
  const int64_t n = idx ? nIdx : numSeg;
  S.assign((size_t)n * 3, 0.0);
  PK.assign(sigmaHat ? (size_t)n * 3 : 0, 0.0);
  if (n == 0) return DDD_OK;
  if (sigmaHat)
    for (int64_t q = 0; q < 6 * n; ++q)
      if (!std::isfinite(sigmaHat[q])) return fail(ctx, DDD_ENONFINITE, "non-finite sigmaHat");
  ddd::SelfK SK;
  SK.a = sp->coreRad;
  SK.aSq = k->aSq;                    // dlnParams.coreRadSq
  SK.mu4pi = k->mu4pi;
  SK.omNuInv = 1.0 / (1.0 - sp->nu);  // MaterialConstructor.jl:20
  SK.nuOmNuInv = sp->nu * SK.omNuInv;  // MaterialConstructor.jl:22
  SK.Ec = sp->coreEnergy;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  int64_t npad = 0, h2d = 0;
  rc = upload_network(ctx, coord, coordCols, bVec, bVecCols, segIdx, ld, extSeg, numSeg, npad, h2d);
  if (rc) return rc;
  if (idx) {
    std::vector<int64_t> rows0((size_t)n);
    for (int64_t q = 0; q < n; ++q) rows0[q] = idx[q] - 1;
    CK(ctx->rows.ensure((size_t)n * sizeof(int64_t)), "alloc rows");
    CK(cudaMemcpyAsync(ctx->rows.p, rows0.data(), (size_t)n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream),
       "copy idx");
  }
  if (sigmaHat) {
    CK(ctx->sigma.ensure((size_t)n * 6 * sizeof(double)), "alloc sigmaHat");
    CK(cudaMemcpyAsync(ctx->sigma.p, sigmaHat, (size_t)n * 6 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
       "copy sigmaHat");
  }
  CK(ctx->out.ensure((size_t)n * 6 * sizeof(double)), "alloc output");
  double* dS = ctx->out.as<double>();
  CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
  CK(ddd::launch_self_pk(SK, ctx->coord.as<double>(), ctx->bvec.as<double>(), ctx->segidx.as<int64_t>(), ld,
                         extSeg ? ctx->ext.as<uint8_t>() : nullptr, numSeg, idx ? ctx->rows.as<int64_t>() : nullptr,
                         n, sigmaHat ? ctx->sigma.as<double>() : nullptr, dS, sigmaHat ? dS + 3 * n : nullptr,
                         ctx->stream),
     "self_pk_f64");
  CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
  CK(cudaMemcpyAsync(S.data(), dS, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "copy S");
  if (sigmaHat)
    CK(cudaMemcpyAsync(PK.data(), dS + 3 * n, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
       "copy PK");
  CK(cudaStreamSynchronize(ctx->stream), "self force");
  ctx->lastKernelMs = elapsed(ctx->ev[1], ctx->ev[2]);
  return DDD_OK;
}

// The reference skips entry q of its index list when extSeg[q] is set (the
// position, DislocationForces.jl:338,376); positions past numSeg hold no
// segment flag here and are treated as internal.
inline bool ext_at(const uint8_t* extSeg, int64_t numSeg, int64_t q) { return extSeg && q < numSeg && extSeg[q]; }

}  // namespace

extern "C" {

int ddd_self_force(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                   int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                   const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx, double* F1, double* F2) {
  DDD_NVTX("ddd_self_force");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  const int64_t n = idx ? nIdx : numSeg;
  if (n > 0 && (!F1 || !F2)) return fail(ctx, DDD_EINVAL, "F1 or F2 is NULL");
  std::vector<double> S, PK;
  int rc = self_pk_compute(ctx, k, sp, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx,
                           nullptr, S, PK);
  if (rc) return rc;
  for (int64_t q = 0; q < 3 * n; ++q) {
    F1[q] = -S[q];  // selfForceNode1 = -selfForceNode2 (:350)
    F2[q] = S[q];
  }
  return DDD_OK;
}

int ddd_self_force_inplace(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                           int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx,
                           int64_t ldSegIdx, const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx,
                           double* segForce, int64_t segForceCols) {
  DDD_NVTX("ddd_self_force_inplace");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (segForceCols < numSeg) return fail(ctx, DDD_EINVAL, "segForce has fewer columns than numSeg");
  const int64_t n = idx ? nIdx : numSeg;
  if (n > 0 && !segForce) return fail(ctx, DDD_EINVAL, "segForce is NULL");
  std::vector<double> S, PK;
  int rc = self_pk_compute(ctx, k, sp, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx,
                           nullptr, S, PK);
  if (rc) return rc;
  for (int64_t q = 0; q < n; ++q) {  // calcSelfForce! (:354-387)
    if (ext_at(extSeg, numSeg, q)) continue;
    const int64_t i = idx ? idx[q] - 1 : q;
    for (int c = 0; c < 3; ++c) {
      segForce[6 * i + c] -= S[3 * q + c];
      segForce[6 * i + 3 + c] += S[3 * q + c];
    }
  }
  return DDD_OK;
}

int ddd_seg_force(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                  int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                  const uint8_t* extSeg, int64_t numSeg, const double* sigmaHat, const int64_t* idx, int64_t nIdx,
                  double* force, ddd_report* rep) {
  DDD_NVTX("ddd_seg_force");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  const int64_t n = idx ? nIdx : numSeg;
  if (n > 0 && !force) return fail(ctx, DDD_EINVAL, "force is NULL");
  std::vector<double> S, PK;
  int rc = self_pk_compute(ctx, k, sp, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx,
                           sigmaHat, S, PK);
  if (rc) return rc;
  rc = segseg_compute(ctx, k, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx, rep);
  if (rc) return rc;
  // calcSegForce (:23-46): segForce[k, j, i] += selfForce[j][k, i] + 0.5 * PKForce[k, i].
  const double* F = ctx->hostTmp.data();
  for (int64_t q = 0; q < n; ++q)
    for (int c = 0; c < 3; ++c) {
      const double pk = sigmaHat ? PK[3 * q + c] : 0.0;
      force[6 * q + c] = F[6 * q + c] + (-S[3 * q + c] + 0.5 * pk);
      force[6 * q + 3 + c] = F[6 * q + 3 + c] + (S[3 * q + c] + 0.5 * pk);
    }
  return DDD_OK;
}

int ddd_seg_force_inplace(ddd_ctx* ctx, const ddd_consts* k, const ddd_self_params* sp, const double* coord,
                          int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx,
                          int64_t ldSegIdx, const uint8_t* extSeg, int64_t numSeg, const double* sigmaHat,
                          const int64_t* idx, int64_t nIdx, double* segForce, int64_t segForceCols, ddd_report* rep) {
  DDD_NVTX("ddd_seg_force_inplace");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (segForceCols < numSeg) return fail(ctx, DDD_EINVAL, "segForce has fewer columns than numSeg");
  const int64_t n = idx ? nIdx : numSeg;
  if (n > 0 && !segForce) return fail(ctx, DDD_EINVAL, "segForce is NULL");
  std::vector<double> S, PK;
  int rc = self_pk_compute(ctx, k, sp, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx,
                           sigmaHat, S, PK);
  if (rc) return rc;
  rc = segseg_compute(ctx, k, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx, rep);
  if (rc) return rc;
  // calcSegForce! (:48-72): zero the range, then calcPKForce!, calcSelfForce!,
  // calcSegSegForce!, each adding in turn.
  for (int64_t q = 0; q < n; ++q) {
    const int64_t i = idx ? idx[q] - 1 : q;
    for (int c = 0; c < 6; ++c) segForce[6 * i + c] = 0.0;
  }
  if (sigmaHat)
    for (int64_t q = 0; q < n; ++q) {  // calcPKForce! (:244-272)
      if (ext_at(extSeg, numSeg, q)) continue;
      const int64_t i = idx ? idx[q] - 1 : q;
      for (int c = 0; c < 3; ++c) {
        segForce[6 * i + c] += PK[3 * q + c] / 2;
        segForce[6 * i + 3 + c] += PK[3 * q + c] / 2;
      }
    }
  for (int64_t q = 0; q < n; ++q) {  // calcSelfForce! (:354-387)
    if (ext_at(extSeg, numSeg, q)) continue;
    const int64_t i = idx ? idx[q] - 1 : q;
    for (int c = 0; c < 3; ++c) {
      segForce[6 * i + c] -= S[3 * q + c];
      segForce[6 * i + 3 + c] += S[3 * q + c];
    }
  }
  add_segseg_inplace(ctx, extSeg, numSeg, idx, nIdx, segForce);
  return DDD_OK;
}

}  // extern "C"

namespace {

// dlnMobility (BCC) on the GPU for the nodes of idx (or 1:numNode) into
// ctx->hostTmp: [nodeForce 3n | nodeVel 3n].  All indices are checked on the
// host first.
int mobility_compute(ddd_ctx* ctx, const ddd_mob_params* mp, const double* coord, int64_t coordCols,
                     const double* bVec, int64_t bVecCols, const int64_t* links, int64_t linkCols,
                     const int64_t* connectivity, int64_t ldConn, int64_t connCols, const double* segForce,
                     int64_t segForceCols, int64_t numNode, const int64_t* idx, int64_t nIdx) {
  if (!mp) return fail(ctx, DDD_EINVAL, "mobility parameters are NULL");
  const double pv[5] = {mp->sigmaPN, mp->edgeDrag, mp->screwDrag, mp->climbDrag, mp->lineDrag};
  for (double v : pv)
    if (!std::isfinite(v)) return fail(ctx, DDD_ENONFINITE, "non-finite mobility parameter");
  if (numNode < 0 || coordCols < 0 || bVecCols < 0 || linkCols < 0 || connCols < 0 || segForceCols < 0 ||
      (idx && nIdx < 0))
    return fail(ctx, DDD_EINVAL, "negative size");
  if (ldConn < 1 || ldConn % 2 == 0) return fail(ctx, DDD_EINVAL, "connectivity must have 1 + 2 maxConnect rows");
  if (numNode > connCols || numNode > coordCols) return fail(ctx, DDD_EINVAL, "numNode exceeds coord / connectivity");
  if (linkCols > bVecCols || linkCols > segForceCols)
    return fail(ctx, DDD_EINVAL, "links has more columns than bVec or segForce");
  const int64_t n = idx ? nIdx : numNode;
  ctx->hostTmp.assign((size_t)n * 6, 0.0);
  if (n == 0) return DDD_OK;
  if (!coord || !bVec || !links || !connectivity || !segForce) return fail(ctx, DDD_EINVAL, "network array is NULL");
  char buf[160];
  for (int64_t q = 0; q < n; ++q) {
    const int64_t node = idx ? idx[q] : q + 1;
    if (node < 1 || node > numNode) {
      snprintf(buf, sizeof buf, "idx[%lld] = %lld outside 1..numNode=%lld", (long long)q, (long long)node,
               (long long)numNode);
      return fail(ctx, DDD_ERANGE, buf);
    }
    const int64_t* cn = connectivity + ldConn * (node - 1);
    if (cn[0] < 0 || 2 * cn[0] + 1 > ldConn) {
      snprintf(buf, sizeof buf, "node %lld: %lld connections exceed the connectivity rows", (long long)node,
               (long long)cn[0]);
      return fail(ctx, DDD_ERANGE, buf);
    }
    for (int64_t c = 1; c <= cn[0]; ++c) {
      const int64_t link = cn[2 * c - 1], col = cn[2 * c];
      if (link < 1 || link > linkCols || (col != 1 && col != 2)) {
        snprintf(buf, sizeof buf, "node %lld: connection %lld = (link %lld, column %lld) out of range",
                 (long long)node, (long long)c, (long long)link, (long long)col);
        return fail(ctx, DDD_ERANGE, buf);
      }
      const int64_t other = links[2 * (link - 1) + (2 - col)];
      if (other < 1 || other > coordCols) {
        snprintf(buf, sizeof buf, "link %lld: node %lld outside 1..%lld", (long long)link, (long long)other,
                 (long long)coordCols);
        return fail(ctx, DDD_ERANGE, buf);
      }
    }
  }
  ddd::MobK P{mp->sigmaPN, mp->edgeDrag, mp->screwDrag, mp->climbDrag, mp->lineDrag};
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = ctx->stream;
  const size_t cB = (size_t)coordCols * 3 * 8, bB = (size_t)linkCols * 3 * 8, lB = (size_t)linkCols * 2 * 8;
  const size_t nB = (size_t)ldConn * numNode * 8, fB = (size_t)linkCols * 6 * 8;
  CK(ctx->coord.ensure(cB), "alloc coord");
  CK(ctx->bvec.ensure(bB), "alloc bVec");
  CK(ctx->links.ensure(lB), "alloc links");
  CK(ctx->conn.ensure(nB), "alloc connectivity");
  CK(ctx->segforce.ensure(fB), "alloc segForce");
  CK(ctx->out.ensure((size_t)n * 6 * sizeof(double)), "alloc output");
  CK(cudaMemcpyAsync(ctx->coord.p, coord, cB, cudaMemcpyHostToDevice, st), "copy coord");
  CK(cudaMemcpyAsync(ctx->bvec.p, bVec, bB, cudaMemcpyHostToDevice, st), "copy bVec");
  CK(cudaMemcpyAsync(ctx->links.p, links, lB, cudaMemcpyHostToDevice, st), "copy links");
  CK(cudaMemcpyAsync(ctx->conn.p, connectivity, nB, cudaMemcpyHostToDevice, st), "copy connectivity");
  CK(cudaMemcpyAsync(ctx->segforce.p, segForce, fB, cudaMemcpyHostToDevice, st), "copy segForce");
  if (idx) {
    std::vector<int64_t> rows0((size_t)n);
    for (int64_t q = 0; q < n; ++q) rows0[q] = idx[q] - 1;
    CK(ctx->rows.ensure((size_t)n * sizeof(int64_t)), "alloc rows");
    CK(cudaMemcpyAsync(ctx->rows.p, rows0.data(), (size_t)n * sizeof(int64_t), cudaMemcpyHostToDevice, st),
       "copy idx");
  }
  double* dOut = ctx->out.as<double>();
  CK(cudaEventRecord(ctx->ev[1], st), "event");
  CK(ddd::launch_mobility_bcc(P, ctx->coord.as<double>(), ctx->bvec.as<double>(), ctx->links.as<int64_t>(),
                              ctx->conn.as<int64_t>(), ldConn, ctx->segforce.as<double>(),
                              idx ? ctx->rows.as<int64_t>() : nullptr, n, dOut, dOut + 3 * n, st),
     "mobility_bcc_f64");
  CK(cudaEventRecord(ctx->ev[2], st), "event");
  CK(cudaMemcpyAsync(ctx->hostTmp.data(), dOut, (size_t)n * 6 * sizeof(double), cudaMemcpyDeviceToHost, st),
     "copy node forces and velocities");
  CK(cudaStreamSynchronize(st), "mobility");
  ctx->lastKernelMs = elapsed(ctx->ev[1], ctx->ev[2]);
  return DDD_OK;
}

}  // namespace

extern "C" {

int ddd_mobility_bcc(ddd_ctx* ctx, const ddd_mob_params* mp, const double* coord, int64_t coordCols,
                     const double* bVec, int64_t bVecCols, const int64_t* links, int64_t linkCols,
                     const int64_t* connectivity, int64_t ldConn, int64_t connCols, const double* segForce,
                     int64_t segForceCols, int64_t numNode, const int64_t* idx, int64_t nIdx, double* nodeForce,
                     double* nodeVel) {
  DDD_NVTX("ddd_mobility_bcc");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  const int64_t n = idx ? nIdx : numNode;
  if (n > 0 && (!nodeForce || !nodeVel)) return fail(ctx, DDD_EINVAL, "nodeForce or nodeVel is NULL");
  int rc = mobility_compute(ctx, mp, coord, coordCols, bVec, bVecCols, links, linkCols, connectivity, ldConn, connCols,
                            segForce, segForceCols, numNode, idx, nIdx);
  if (rc || n == 0) return rc;
  std::memcpy(nodeForce, ctx->hostTmp.data(), (size_t)n * 3 * sizeof(double));
  std::memcpy(nodeVel, ctx->hostTmp.data() + 3 * n, (size_t)n * 3 * sizeof(double));
  return DDD_OK;
}

int ddd_mobility_bcc_inplace(ddd_ctx* ctx, const ddd_mob_params* mp, const double* coord, int64_t coordCols,
                             const double* bVec, int64_t bVecCols, const int64_t* links, int64_t linkCols,
                             const int64_t* connectivity, int64_t ldConn, int64_t connCols, const double* segForce,
                             int64_t segForceCols, int64_t numNode, const int64_t* idx, int64_t nIdx,
                             double* nodeForce, double* nodeVel, int64_t nodeCols) {
  DDD_NVTX("ddd_mobility_bcc_inplace");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  const int64_t n = idx ? nIdx : numNode;
  if (nodeCols < numNode) return fail(ctx, DDD_EINVAL, "nodeForce / nodeVel have fewer columns than numNode");
  if (n > 0 && (!nodeForce || !nodeVel)) return fail(ctx, DDD_EINVAL, "nodeForce or nodeVel is NULL");
  int rc = mobility_compute(ctx, mp, coord, coordCols, bVec, bVecCols, links, linkCols, connectivity, ldConn, connCols,
                            segForce, segForceCols, numNode, idx, nIdx);
  if (rc) return rc;
  const double* H = ctx->hostTmp.data();
  for (int64_t q = 0; q < n; ++q) {  // nodeForce[:, node1] = ...; nodeVel[:, node1] = ... (:338-339)
    const int64_t node = idx ? idx[q] - 1 : q;
    for (int c = 0; c < 3; ++c) {
      nodeForce[3 * node + c] = H[3 * q + c];
      nodeVel[3 * node + c] = H[3 * n + 3 * q + c];
    }
  }
  return DDD_OK;
}

int ddd_segseg_force_inplace(ddd_ctx* ctx, const ddd_consts* k, const double* coord, int64_t coordCols,
                             const double* bVec, int64_t bVecCols, const int64_t* segIdx, int64_t ldSegIdx,
                             const uint8_t* extSeg, int64_t numSeg, const int64_t* idx, int64_t nIdx,
                             double* segForce, int64_t segForceCols, ddd_report* rep) {
  DDD_NVTX("ddd_segseg_force_inplace");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (segForceCols < numSeg) return fail(ctx, DDD_EINVAL, "segForce has fewer columns than numSeg");
  const int64_t nOut = idx ? nIdx : numSeg;
  if (nOut > 0 && !segForce) return fail(ctx, DDD_EINVAL, "segForce is NULL");
  int rc = segseg_compute(ctx, k, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, extSeg, numSeg, idx, nIdx, rep);
  if (rc) return rc;
  add_segseg_inplace(ctx, extSeg, numSeg, idx, nIdx, segForce);
  return DDD_OK;
}

int ddd_sigma_tilde(ddd_ctx* ctx, const ddd_consts* k, const double* x0, int64_t numPoints, const double* coord,
                    int64_t coordCols, const double* bVec, int64_t bVecCols, const int64_t* segIdx,
                    int64_t ldSegIdx, int64_t numSeg, const int64_t* idx, int64_t nIdx, double* sigma,
                    ddd_report* rep) {
  DDD_NVTX("ddd_sigma_tilde");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  ddd::KConsts K;
  int rc = check_consts(ctx, k, K);
  if (rc) return rc;
  if (numPoints < 0 || numSeg < 0 || ldSegIdx < 0 || (idx && nIdx < 0))
    return fail(ctx, DDD_EINVAL, "negative size");
  if (numPoints > 0 && (!x0 || !sigma)) return fail(ctx, DDD_EINVAL, "x0 or sigma is NULL");
  if (numSeg > ldSegIdx) return fail(ctx, DDD_EINVAL, "numSeg exceeds the rows of segIdx (ldSegIdx)");
  const int64_t nSel = idx ? nIdx : numSeg;
  if (nSel > 0 && (!coord || !bVec || !segIdx)) return fail(ctx, DDD_EINVAL, "network array is NULL");
  // Selected rows, gathered into a compact nSel × 3 segIdx (DislocationFEM.jl:108-118).
  std::vector<int64_t> sel((size_t)nSel * 3);
  for (int64_t q = 0; q < nSel; ++q) {
    int64_t r = q;
    if (idx) {
      if (idx[q] < 1 || idx[q] > ldSegIdx) {
        char buf[96];
        snprintf(buf, sizeof buf, "idx[%lld] = %lld outside 1..%lld", (long long)q, (long long)idx[q],
                 (long long)ldSegIdx);
        return fail(ctx, DDD_ERANGE, buf);
      }
      r = idx[q] - 1;
    }
    rc = check_row(ctx, coord, coordCols, bVec, bVecCols, segIdx, ldSegIdx, r);
    if (rc) return rc;
    sel[q] = segIdx[r];
    sel[q + nSel] = segIdx[r + ldSegIdx];
    sel[q + 2 * nSel] = segIdx[r + 2 * ldSegIdx];
  }
  for (int64_t j = 0; j < numPoints; ++j)
    if (!ddd::finite3(x0 + 3 * j)) return fail(ctx, DDD_ENONFINITE, "non-finite field point");
  if (rep) memset(rep, 0, sizeof *rep);
  if (numPoints == 0) return DDD_OK;
  if (nSel == 0) {
    memset(sigma, 0, (size_t)numPoints * 6 * sizeof(double));
    return DDD_OK;
  }
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  int64_t h2d = 0, npad = 0;
  CK(cudaEventRecord(ctx->ev[0], ctx->stream), "event");
  rc = upload_network(ctx, coord, coordCols, bVec, bVecCols, sel.data(), nSel, nullptr, nSel, npad, h2d);
  if (rc) return rc;
  const size_t xB = (size_t)numPoints * 3 * sizeof(double), sB = (size_t)numPoints * 6 * sizeof(double);
  CK(ctx->x0.ensure(xB), "alloc points");
  CK(ctx->sigma.ensure(sB), "alloc sigma");
  CK(cudaMemcpyAsync(ctx->x0.p, x0, xB, cudaMemcpyHostToDevice, ctx->stream), "copy points");
  h2d += (int64_t)xB;
  CK(cudaEventRecord(ctx->ev[1], ctx->stream), "event");
  CK(run_sigma(ctx, K, ctx->soa.as<double>(), npad, nSel, ctx->x0.as<double>(), numPoints,
                           ctx->sigma.as<double>(), ctx->stream),
     "sigma_tilde_f64");
  CK(cudaEventRecord(ctx->ev[2], ctx->stream), "event");
  CK(cudaMemcpyAsync(sigma, ctx->sigma.p, sB, cudaMemcpyDeviceToHost, ctx->stream), "copy sigma");
  CK(cudaEventRecord(ctx->ev[3], ctx->stream), "event");
  CK(cudaStreamSynchronize(ctx->stream), "sigma_tilde");
  if (rep) {
    rep->kernel_ms = elapsed(ctx->ev[1], ctx->ev[2]);
    rep->total_ms = elapsed(ctx->ev[0], ctx->ev[3]);
    rep->h2d_bytes = h2d;
    rep->d2h_bytes = (int64_t)sB;
  }
  return DDD_OK;
}

int ddd_segseg_force_device(ddd_ctx* ctx, const ddd_consts* k, const double* segs, int64_t ldSegs,
                            const uint8_t* ext, int64_t numSeg, double* force, void* stream, ddd_report* rep) {
  DDD_NVTX("ddd_segseg_force_device");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  ddd::KConsts K;
  int rc = check_consts(ctx, k, K);
  if (rc) return rc;
  if (numSeg < 0 || ldSegs < numSeg) return fail(ctx, DDD_EINVAL, "bad numSeg / ldSegs");
  if (numSeg > 0 && (!segs || !force)) return fail(ctx, DDD_EINVAL, "segs or force is NULL");
  if (rep) memset(rep, 0, sizeof *rep);
  if (numSeg == 0) return DDD_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  const int64_t npad = ddd::strict::segseg_npad(numSeg);
  CK(ctx->soa.ensure(ddd::strict::segseg_soa_bytes(npad)), "alloc segment SoA");
  CK(ctx->skip.ensure((size_t)npad), "alloc skip flags");
  CK(ctx->partial.ensure(partial_bytes(ctx, npad)), "alloc partial sums");
  CK(ctx->counters.ensure(3 * sizeof(unsigned long long)), "alloc counters");
  if (rep) CK(cudaMemsetAsync(ctx->counters.p, 0, 3 * sizeof(unsigned long long), st), "memset counters");
  if (rep) CK(cudaEventRecord(ctx->ev[1], st), "event");
  CK(ddd::strict::launch_prep_segments_packed(segs, ldSegs, ext, numSeg, npad, ctx->soa.as<double>(),
                                      ctx->skip.as<uint8_t>(), st),
     "prep_segments_packed");
  CK(run_segseg_all(ctx, K, ctx->soa.as<double>(), ctx->skip.as<uint8_t>(), npad, ctx->partial.as<double>(),
                                force, numSeg, rep ? ctx->counters.as<unsigned long long>() : nullptr, st),
     "segseg_all_f64");
  if (rep) {
    unsigned long long cnt[3] = {0, 0, 0};
    CK(cudaEventRecord(ctx->ev[2], st), "event");
    CK(cudaMemcpyAsync(cnt, ctx->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, st), "copy counters");
    CK(cudaStreamSynchronize(st), "segseg_force_device");
    rep->pairs_general = (int64_t)cnt[0];
    rep->pairs_parallel = (int64_t)cnt[1];
    rep->core_sides = (int64_t)cnt[2];
    rep->kernel_ms = elapsed(ctx->ev[1], ctx->ev[2]);
    rep->total_ms = rep->kernel_ms;
  }
  return DDD_OK;
}

int ddd_sigma_tilde_device(ddd_ctx* ctx, const ddd_consts* k, const double* x0, int64_t numPoints,
                           const double* segs, int64_t ldSegs, int64_t numSeg, double* sigma, void* stream,
                           ddd_report* rep) {
  DDD_NVTX("ddd_sigma_tilde_device");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  ddd::KConsts K;
  int rc = check_consts(ctx, k, K);
  if (rc) return rc;
  if (numSeg < 0 || ldSegs < numSeg || numPoints < 0) return fail(ctx, DDD_EINVAL, "bad sizes");
  if (numPoints > 0 && (!x0 || !sigma)) return fail(ctx, DDD_EINVAL, "x0 or sigma is NULL");
  if (numSeg > 0 && !segs) return fail(ctx, DDD_EINVAL, "segs is NULL");
  if (rep) memset(rep, 0, sizeof *rep);
  if (numPoints == 0) return DDD_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (numSeg == 0) {
    CK(cudaMemsetAsync(sigma, 0, (size_t)numPoints * 6 * sizeof(double), st), "memset sigma");
    return DDD_OK;
  }
  const int64_t npad = ddd::strict::segseg_npad(numSeg);
  CK(ctx->soa.ensure(ddd::strict::segseg_soa_bytes(npad)), "alloc segment SoA");
  CK(ctx->skip.ensure((size_t)npad), "alloc skip flags");
  if (rep) CK(cudaEventRecord(ctx->ev[1], st), "event");
  CK(ddd::strict::launch_prep_segments_packed(segs, ldSegs, nullptr, numSeg, npad, ctx->soa.as<double>(),
                                      ctx->skip.as<uint8_t>(), st),
     "prep_segments_packed");
  CK(run_sigma(ctx, K, ctx->soa.as<double>(), npad, numSeg, x0, numPoints, sigma, st), "sigma_tilde_f64");
  if (rep) {
    CK(cudaEventRecord(ctx->ev[2], st), "event");
    CK(cudaStreamSynchronize(st), "sigma_tilde_device");
    rep->kernel_ms = elapsed(ctx->ev[1], ctx->ev[2]);
    rep->total_ms = rep->kernel_ms;
  }
  return DDD_OK;
}

int ddd_set_mode(ddd_ctx* ctx, int mode) {
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (mode != DDD_MODE_FP64 && mode != DDD_MODE_FP64_FMA && mode != DDD_MODE_DF64 && mode != DDD_MODE_F32C &&
      mode != DDD_MODE_FP64_FAST)
    return fail(ctx, DDD_EINVAL, "unknown mode");
  ctx->mode = mode;
  return DDD_OK;
}

int ddd_get_mode(const ddd_ctx* ctx) { return ctx ? ctx->mode : DDD_EINVAL; }

int ddd_set_partial_limit(ddd_ctx* ctx, int64_t bytes) {
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (bytes < 0) return fail(ctx, DDD_EINVAL, "negative partial-sum limit");
  ctx->partialLimit = bytes;
  return DDD_OK;
}

int64_t ddd_get_partial_limit(const ddd_ctx* ctx) {
  return ctx ? (ctx->partialLimit ? ctx->partialLimit : kDefaultPartialLimit) : DDD_EINVAL;
}

int ddd_surrogate_make_data(ddd_ctx* ctx, const ddd_consts* k, const double* segs, int64_t n, const int32_t* pairs,
                            int64_t P, void* X, float* Bp, float* T, double* F) {
  DDD_NVTX("ddd_surrogate_make_data");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  ddd::KConsts K;
  int rc = check_consts(ctx, k, K);
  if (rc) return rc;
  if (n <= 0 || P < 0 || !segs || (P > 0 && (!pairs || !X || !Bp || !T))) return fail(ctx, DDD_EINVAL, "bad arguments");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  CK(cudaDeviceSynchronize(), "wait for the caller's device inputs");
  const int64_t npad = ddd::strict::segseg_npad(n);
  CK(ctx->soa.ensure(ddd::strict::segseg_soa_bytes(npad)), "alloc segment SoA");
  CK(ctx->skip.ensure((size_t)npad), "alloc skip flags");
  CK(ddd::strict::launch_prep_segments_packed(segs, n, nullptr, n, npad, ctx->soa.as<double>(),
                                              ctx->skip.as<uint8_t>(), ctx->stream),
     "prep_segments_packed");
  CK(ddd::launch_pair_data(K, ctx->soa.as<double>(), npad, pairs, P, X, Bp, T, F, ctx->stream), "pair_data");
  CK(cudaStreamSynchronize(ctx->stream), "surrogate_make_data");
  return DDD_OK;
}

int ddd_tc_gemm_bf16(ddd_ctx* ctx, int M, int N, int K, const void* A, const void* B, float* D, void* stream) {
  DDD_NVTX("ddd_tc_gemm_bf16");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (M <= 0 || M % 128 || N < 16 || N > 256 || N % 16 || K <= 0 || K % 16)
    return fail(ctx, DDD_EINVAL, "shape must be M % 128 == 0, N in [16, 256] multiple of 16, K multiple of 16");
  if (!A || !B || !D) return fail(ctx, DDD_EINVAL, "null pointer");
  if (((uintptr_t)A | (uintptr_t)B) & 15) return fail(ctx, DDD_EINVAL, "A and B must be 16-byte aligned");
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  CK(ctx->errflag.ensure(sizeof(int)), "alloc error flag");
  CK(cudaMemsetAsync(ctx->errflag.p, 0, sizeof(int), st), "memset");
  CK(ddd::launch_tc_gemm_bf16(M, N, K, A, B, D, ctx->errflag.as<int>(), st), "tc_gemm_bf16");
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, ctx->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st), "copy flag");
  CK(cudaStreamSynchronize(st), "tc_gemm_bf16");
  if (flag) return fail(ctx, DDD_ETIMEOUT, "tensor-core GEMM: mbarrier wait timed out");
  return DDD_OK;
}

int ddd_selftest_bounded_wait(ddd_ctx* ctx, long long max_clocks, int arrive) {
  DDD_NVTX("ddd_selftest_bounded_wait");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (max_clocks < 1 || max_clocks > 2000000000LL)
    return fail(ctx, DDD_EINVAL, "max_clocks must be in [1, 2e9] (about a second at most)");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  CK(ctx->errflag.ensure(sizeof(int)), "alloc error flag");
  CK(cudaMemsetAsync(ctx->errflag.p, 0, sizeof(int), ctx->stream), "memset");
  CK(ddd::launch_bounded_wait_probe(max_clocks, arrive, ctx->errflag.as<int>(), ctx->stream), "bounded_wait_probe");
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, ctx->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "copy flag");
  CK(cudaStreamSynchronize(ctx->stream), "bounded_wait_probe");
  if (flag) return fail(ctx, DDD_ETIMEOUT, "bounded mbarrier wait timed out (self-test)");
  return DDD_OK;
}

int ddd_probe_fma_peak(ddd_ctx* ctx, int precision, double* flops_per_s) {
  DDD_NVTX("ddd_probe_fma_peak");
  if (!ctx || !flops_per_s) return DDD_EINVAL;
  if (precision != 64 && precision != 32) return fail(ctx, DDD_EINVAL, "precision must be 64 or 32");
  std::lock_guard<std::mutex> g(ctx->mu);
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "attr");
  const int threads = 256, blocks = sms * 8;
  CK(ctx->probe.ensure((size_t)blocks * threads * sizeof(double)), "alloc probe");
  auto run = [&](int iters, float* ms) -> cudaError_t {
    cudaError_t e = cudaEventRecord(ctx->ev[0], ctx->stream);
    if (e == cudaSuccess)
      e = precision == 64 ? ddd::launch_fp64_peak_probe(ctx->probe.as<double>(), iters, blocks, threads, ctx->stream)
                          : ddd::launch_fp32_peak_probe(ctx->probe.as<float>(), iters, blocks, threads, ctx->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[1], ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) *ms = elapsed(ctx->ev[0], ctx->ev[1]);
    return e;
  };
  // Calibrate the chain length so one timed run lasts about a second.
  int iters = precision == 64 ? 4096 : 65536;
  float ms = 0.0f;
  CK(run(iters, &ms), "probe");
  CK(run(iters, &ms), "probe");
  const double want = (double)iters * 1100.0 / (ms > 1e-3f ? ms : 1e-3f);
  iters = (int)std::min(want, 1.0e9);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    CK(run(iters, &ms), "probe");
    if (ms < best) best = ms;
  }
  *flops_per_s = 2.0 * 8.0 * (double)iters * (double)threads * (double)blocks / (best * 1e-3);
  return DDD_OK;
}

}  // extern "C"

extern "C" {

int ddd_detect_collision(ddd_ctx* ctx, double collisionDistSq, const double* coord, int64_t coordCols,
                         const double* nodeVel, int64_t nodeVelCols, const int32_t* label, int64_t labelLen,
                         const int64_t* links, int64_t linkCols, const double* bVec, int64_t bVecCols,
                         const int64_t* connectivity, int64_t ldConn, int64_t connCols, int64_t numNode,
                         int64_t numSeg, const int64_t* skipSegs, int64_t nSkip, ddd_collision* out) {
  DDD_NVTX("ddd_detect_collision");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (!out) return fail(ctx, DDD_EINVAL, "out is NULL");
  *out = ddd_collision{};
  if (numNode < 0 || numSeg < 0 || coordCols < 0 || nodeVelCols < 0 || labelLen < 0 || linkCols < 0 ||
      bVecCols < 0 || connCols < 0 || nSkip < 0)
    return fail(ctx, DDD_EINVAL, "negative size");
  if (numNode > coordCols || numNode > nodeVelCols || numNode > labelLen || numNode > connCols)
    return fail(ctx, DDD_EINVAL, "numNode exceeds coord / nodeVel / label / connectivity");
  if (numSeg > linkCols || numSeg > bVecCols) return fail(ctx, DDD_EINVAL, "numSeg exceeds links / bVec");
  if (ldConn < 1 || ldConn % 2 == 0) return fail(ctx, DDD_EINVAL, "connectivity must have 1 + 2 maxConnect rows");
  if (numNode >= INT32_MAX || numSeg >= INT32_MAX) return fail(ctx, DDD_ETOOBIG, "more than 2^31 - 1 nodes or links");
  if (numNode == 0) return DDD_OK;
  if (!coord || !nodeVel || !label || !links || !connectivity || (numSeg > 0 && !bVec) || (nSkip > 0 && !skipSegs))
    return fail(ctx, DDD_EINVAL, "network array is NULL");
  char buf[160];
  // Nodes: finite coordinates and velocities, their box; connections of the
  // mobile nodes (the ones the hinge loop reads) in range.
  double box[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  double maxAbs = 0.0;
  for (int64_t i = 0; i < numNode; ++i) {
    for (int k = 0; k < 3; ++k) {
      const double x = coord[3 * i + k], v = nodeVel[3 * i + k];
      if (!std::isfinite(x) || !std::isfinite(v)) {
        snprintf(buf, sizeof buf, "node %lld: non-finite coordinate or velocity", (long long)(i + 1));
        return fail(ctx, DDD_ENONFINITE, buf);
      }
      box[k] = std::min(box[k], x);
      box[3 + k] = std::max(box[3 + k], x);
      maxAbs = std::max(maxAbs, std::fabs(x));
    }
    if (label[i] != 1 && label[i] != 3) continue;
    const int64_t* cn = connectivity + ldConn * i;
    if (cn[0] < 0 || 2 * cn[0] + 1 > ldConn) {
      snprintf(buf, sizeof buf, "node %lld: %lld connections exceed the connectivity rows", (long long)(i + 1),
               (long long)cn[0]);
      return fail(ctx, DDD_ERANGE, buf);
    }
    for (int64_t c = 1; c <= cn[0]; ++c) {
      const int64_t link = cn[2 * c - 1], col = cn[2 * c];
      if (link < 1 || link > linkCols || (col != 1 && col != 2)) {
        snprintf(buf, sizeof buf, "node %lld: connection %lld = (link %lld, column %lld) out of range",
                 (long long)(i + 1), (long long)c, (long long)link, (long long)col);
        return fail(ctx, DDD_ERANGE, buf);
      }
      const int64_t other = links[2 * (link - 1) + (2 - col)];
      if (other < 1 || other > numNode) {
        snprintf(buf, sizeof buf, "link %lld: node %lld outside 1..numNode=%lld", (long long)link, (long long)other,
                 (long long)numNode);
        return fail(ctx, DDD_ERANGE, buf);
      }
    }
  }
  for (int64_t i = 0; i < numSeg; ++i)
    for (int k = 0; k < 2; ++k)
      if (links[2 * i + k] < 1 || links[2 * i + k] > numNode) {
        snprintf(buf, sizeof buf, "links[%d, %lld] = %lld outside 1..numNode=%lld", k + 1, (long long)(i + 1),
                 (long long)links[2 * i + k], (long long)numNode);
        return fail(ctx, DDD_ERANGE, buf);
      }
  // skipSegs as canonical (a <= b) sorted pairs: the reference matches either order.
  std::vector<std::pair<int64_t, int64_t>> sk((size_t)nSkip);
  for (int64_t q = 0; q < nSkip; ++q)
    sk[q] = {std::min(skipSegs[2 * q], skipSegs[2 * q + 1]), std::max(skipSegs[2 * q], skipSegs[2 * q + 1])};
  std::sort(sk.begin(), sk.end());
  sk.erase(std::unique(sk.begin(), sk.end()), sk.end());
  std::vector<int64_t> skFlat(2 * sk.size() + 2);
  for (size_t q = 0; q < sk.size(); ++q) skFlat[2 * q] = sk[q].first, skFlat[2 * q + 1] = sk[q].second;

  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (!ctx->coll) ctx->coll = ddd::collision_plan_create();
  cudaStream_t st = ctx->stream;
  const size_t cB = (size_t)numNode * 3 * 8, lB = (size_t)linkCols * 2 * 8, bB = (size_t)std::max<int64_t>(numSeg, 1) * 3 * 8;
  const size_t nB = (size_t)ldConn * numNode * 8, kB = skFlat.size() * 8;
  CK(ctx->coord.ensure(cB), "alloc coord");
  CK(ctx->vel.ensure(cB), "alloc nodeVel");
  CK(ctx->label.ensure((size_t)numNode * 4), "alloc label");
  CK(ctx->links.ensure(lB), "alloc links");
  CK(ctx->bvec.ensure(bB), "alloc bVec");
  CK(ctx->conn.ensure(nB), "alloc connectivity");
  CK(ctx->skippairs.ensure(kB), "alloc skipSegs");
  CK(cudaMemcpyAsync(ctx->coord.p, coord, cB, cudaMemcpyHostToDevice, st), "copy coord");
  CK(cudaMemcpyAsync(ctx->vel.p, nodeVel, cB, cudaMemcpyHostToDevice, st), "copy nodeVel");
  CK(cudaMemcpyAsync(ctx->label.p, label, (size_t)numNode * 4, cudaMemcpyHostToDevice, st), "copy label");
  CK(cudaMemcpyAsync(ctx->links.p, links, lB, cudaMemcpyHostToDevice, st), "copy links");
  if (numSeg > 0) CK(cudaMemcpyAsync(ctx->bvec.p, bVec, (size_t)numSeg * 3 * 8, cudaMemcpyHostToDevice, st), "copy bVec");
  CK(cudaMemcpyAsync(ctx->conn.p, connectivity, nB, cudaMemcpyHostToDevice, st), "copy connectivity");
  CK(cudaMemcpyAsync(ctx->skippairs.p, skFlat.data(), kB, cudaMemcpyHostToDevice, st), "copy skipSegs");
  ddd::CollisionOut r{};
  CK(ddd::collision_detect(ctx->coll, collisionDistSq, ctx->coord.as<double>(), ctx->vel.as<double>(),
                           ctx->label.as<int32_t>(), ctx->links.as<int64_t>(), ctx->bvec.as<double>(),
                           ctx->conn.as<int64_t>(), ldConn, numNode, numSeg, ctx->skippairs.as<int64_t>(),
                           (int64_t)sk.size(), box, maxAbs, &r, ctx->ev[1], ctx->ev[2], st),
     "detect_collision");
  ctx->lastKernelMs = elapsed(ctx->ev[1], ctx->ev[2]);
  out->collision = r.collision;
  out->type = r.type;
  out->n1s1 = r.n1s1, out->n2s1 = r.n2s1, out->n1s2 = r.n1s2, out->n2s2 = r.n2s2, out->s1 = r.s1, out->s2 = r.s2;
  out->L1 = r.L1, out->L2 = r.L2;
  out->pairDistSq = r.pairDistSq, out->pairL1 = r.pairL1, out->pairL2 = r.pairL2;
  return DDD_OK;
}

int ddd_minimum_distance(ddd_ctx* ctx, const double* pts, int64_t n, double* out) {
  DDD_NVTX("ddd_minimum_distance");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (n < 0) return fail(ctx, DDD_EINVAL, "negative size");
  if (n == 0) return DDD_OK;
  if (!pts || !out) return fail(ctx, DDD_EINVAL, "array is NULL");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = ctx->stream;
  CK(ctx->x0.ensure((size_t)n * 24 * 8), "alloc points");
  CK(ctx->out.ensure((size_t)n * 4 * 8), "alloc output");
  CK(cudaMemcpyAsync(ctx->x0.p, pts, (size_t)n * 24 * 8, cudaMemcpyHostToDevice, st), "copy points");
  CK(ddd::launch_minimum_distance(ctx->x0.as<double>(), n, ctx->out.as<double>(), st), "minimum_distance");
  CK(cudaMemcpyAsync(out, ctx->out.p, (size_t)n * 4 * 8, cudaMemcpyDeviceToHost, st), "copy output");
  CK(cudaStreamSynchronize(st), "minimum_distance");
  return DDD_OK;
}

int ddd_u_tilde(ddd_ctx* ctx, double omNuInv8pi, double om2NuOmNuInv8pi, const ddd_u_mesh* mesh,
                const double* points, int64_t numPoints, const double* coord, int64_t coordCols, const int32_t* label,
                int64_t labelLen, const int64_t* links, int64_t linkCols, const double* bVec, int64_t bVecCols,
                int64_t numNode, int64_t numSeg, const int64_t* uDofs, double* uTilde, int64_t uLen) {
  DDD_NVTX("ddd_u_tilde");
  if (!ctx) return DDD_EINVAL;
  std::lock_guard<std::mutex> g(ctx->mu);
  if (!mesh) return fail(ctx, DDD_EINVAL, "mesh is NULL");
  if (numPoints < 0 || coordCols < 0 || labelLen < 0 || linkCols < 0 || bVecCols < 0 || numNode < 0 || numSeg < 0 ||
      uLen < 0 || mesh->numFaces < 0 || mesh->numNormals < 0)
    return fail(ctx, DDD_EINVAL, "negative size");
  if (numNode > coordCols || numNode > labelLen) return fail(ctx, DDD_EINVAL, "numNode exceeds coord / label");
  if (numSeg > linkCols || numSeg > bVecCols) return fail(ctx, DDD_EINVAL, "numSeg exceeds links / bVec");
  if (!uDofs && uLen < 3 * numPoints) return fail(ctx, DDD_EINVAL, "uTilde shorter than 3 numPoints");
  if (numPoints == 0) return DDD_OK;
  if (!points || !uTilde || (numNode > 0 && (!coord || !label)) || (numSeg > 0 && (!links || !bVec)) ||
      (mesh->numFaces > 0 && (!mesh->faceNorm || !mesh->faceMidPt)) || (mesh->numNormals > 0 && !mesh->normals))
    return fail(ctx, DDD_EINVAL, "array is NULL");
  char buf[160];
  for (int64_t i = 0; i < numSeg; ++i)
    for (int k = 0; k < 2; ++k)
      if (links[2 * i + k] < 1 || links[2 * i + k] > numNode) {
        snprintf(buf, sizeof buf, "links[%d, %lld] = %lld outside 1..numNode=%lld", k + 1, (long long)(i + 1),
                 (long long)links[2 * i + k], (long long)numNode);
        return fail(ctx, DDD_ERANGE, buf);
      }
  if (uDofs)
    for (int64_t q = 0; q < 3 * numPoints; ++q)
      if (uDofs[q] < 1 || uDofs[q] > uLen) {
        snprintf(buf, sizeof buf, "uDofs[%lld] = %lld outside 1..%lld", (long long)(q + 1), (long long)uDofs[q],
                 (long long)uLen);
        return fail(ctx, DDD_ERANGE, buf);
      }
  for (int64_t q = 0; q < 3 * numPoints; ++q)
    if (!std::isfinite(points[q])) return fail(ctx, DDD_ENONFINITE, "non-finite evaluation point");
  for (int64_t q = 0; q < 3 * numNode; ++q)
    if (!std::isfinite(coord[q])) return fail(ctx, DDD_ENONFINITE, "non-finite node coordinate");
  ddd::UTildeArgs a{};
  a.fast = ctx->mode != DDD_MODE_FP64;
  a.omNuInv8pi = omNuInv8pi;
  a.om2NuOmNuInv8pi = om2NuOmNuInv8pi;
  double ext = 0.0;
  for (int k = 0; k < 3; ++k) {
    a.C[k] = mesh->C[k];
    a.lo[k] = mesh->lo[k];
    a.hi[k] = mesh->hi[k];
    ext = std::max(ext, mesh->hi[k] - mesh->lo[k]);
  }
  a.tol = mesh->tol > 0.0 ? mesh->tol : 1e-10 * ext;
  a.faceNorm = mesh->faceNorm;
  a.faceMidPt = mesh->faceMidPt;
  a.numFaces = mesh->numFaces;
  a.normals = mesh->normals;
  a.numNormals = mesh->numNormals;
  a.coord = coord;
  a.label = label;
  a.links = links;
  a.bVec = bVec;
  a.numNode = numNode;
  a.numSeg = numSeg;
  a.numPoints = numPoints;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (!ctx->ut) ctx->ut = new ddd::UTildeScratch();
  cudaStream_t st = ctx->stream;
  const size_t cB = (size_t)std::max<int64_t>(numNode, 1) * 24, lB = (size_t)std::max<int64_t>(numSeg, 1) * 16;
  const size_t bB = (size_t)std::max<int64_t>(numSeg, 1) * 24, pB = (size_t)numPoints * 24;
  CK(ctx->coord.ensure(cB), "alloc coord");
  CK(ctx->links.ensure(lB), "alloc links");
  CK(ctx->bvec.ensure(bB), "alloc bVec");
  CK(ctx->upoints.ensure(pB), "alloc points");
  if (numNode > 0) CK(cudaMemcpyAsync(ctx->coord.p, coord, (size_t)numNode * 24, cudaMemcpyHostToDevice, st), "copy coord");
  if (numSeg > 0) {
    CK(cudaMemcpyAsync(ctx->links.p, links, (size_t)numSeg * 16, cudaMemcpyHostToDevice, st), "copy links");
    CK(cudaMemcpyAsync(ctx->bvec.p, bVec, (size_t)numSeg * 24, cudaMemcpyHostToDevice, st), "copy bVec");
  }
  CK(cudaMemcpyAsync(ctx->upoints.p, points, pB, cudaMemcpyHostToDevice, st), "copy points");
  a.coordDev = ctx->coord.as<double>();
  a.linksDev = ctx->links.as<int64_t>();
  a.bVecDev = ctx->bvec.as<double>();
  a.pointsDev = ctx->upoints.as<double>();
  ctx->hostTmp.assign((size_t)numPoints * 3, 0.0);
  CK(ddd::u_tilde_compute(a, ctx->hostTmp.data(), ctx->ev[1], ctx->ev[2], st, *ctx->ut), "u_tilde");
  ctx->lastKernelMs = elapsed(ctx->ev[1], ctx->ev[2]);
  for (int64_t q = 0; q < 3 * numPoints; ++q) uTilde[uDofs ? uDofs[q] - 1 : q] += ctx->hostTmp[(size_t)q];
  return DDD_OK;
}

}  // extern "C"
