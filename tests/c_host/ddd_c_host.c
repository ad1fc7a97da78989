/* A plain C99 host of the C ABI (include/ddd_gb300.h), making the calls a
 * Julia ccall, cgo or JNI binding makes: no Python, no torch, only the
 * header and libddd_gb300.so.
 *
 * Usage: ddd_c_host IN OUT
 *   IN  (native-endian binary): int64 numNode, numSeg, numPoints, nIdx;
 *       double consts[5] (aSq, mu4pi, mu8pi, mu4pinu, nuMu4pinu);
 *       double coord[3 numNode]; double bVec[3 numSeg];
 *       int64 segIdx[numSeg x 3] (column-major, 1-based);
 *       double x0[3 numPoints]; int64 idx[nIdx] (1-based).
 *   OUT: double force[6 numSeg] (all pairs), forceIdx[6 nIdx] (idx form),
 *        sigma[6 numPoints], forceBanded[6 numSeg] (all pairs with the
 *        partial-sum limit at its minimum).
 * Prints one line of return codes and report counters.  Exit status: 0 on
 * success, 3 when ddd_create finds no usable device (its message on stderr),
 * 1 on any other failure.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ddd_gb300.h"

static int read_all(FILE* f, void* dst, size_t bytes) { return bytes == 0 || fread(dst, 1, bytes, f) == bytes; }

static void* alloc(size_t bytes) { return malloc(bytes ? bytes : 1); }

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
    return 1;
  }
  FILE* in = fopen(argv[1], "rb");
  if (!in) {
    perror(argv[1]);
    return 1;
  }
  int64_t hdr[4];
  double kc[5];
  if (!read_all(in, hdr, sizeof hdr) || !read_all(in, kc, sizeof kc)) {
    fprintf(stderr, "short input\n");
    return 1;
  }
  const int64_t numNode = hdr[0], numSeg = hdr[1], M = hdr[2], nIdx = hdr[3];
  if (numNode < 0 || numSeg < 0 || M < 0 || nIdx < 0) {
    fprintf(stderr, "bad header\n");
    return 1;
  }
  double* coord = alloc((size_t)(3 * numNode) * sizeof(double));
  double* bVec = alloc((size_t)(3 * numSeg) * sizeof(double));
  int64_t* segIdx = alloc((size_t)(3 * numSeg) * sizeof(int64_t));
  double* x0 = alloc((size_t)(3 * M) * sizeof(double));
  int64_t* idx = alloc((size_t)nIdx * sizeof(int64_t));
  if (!read_all(in, coord, (size_t)(3 * numNode) * sizeof(double)) ||
      !read_all(in, bVec, (size_t)(3 * numSeg) * sizeof(double)) ||
      !read_all(in, segIdx, (size_t)(3 * numSeg) * sizeof(int64_t)) ||
      !read_all(in, x0, (size_t)(3 * M) * sizeof(double)) || !read_all(in, idx, (size_t)nIdx * sizeof(int64_t))) {
    fprintf(stderr, "short input\n");
    return 1;
  }
  fclose(in);

  ddd_ctx* ctx = ddd_create(0);
  if (!ctx) {
    fprintf(stderr, "ddd_create: %s\n", ddd_last_error(NULL));
    return 3;
  }
  const ddd_consts k = {kc[0], kc[1], kc[2], kc[3], kc[4]};
  double* force = alloc((size_t)(6 * numSeg) * sizeof(double));
  double* forceIdx = alloc((size_t)(6 * nIdx) * sizeof(double));
  double* sigma = alloc((size_t)(6 * M) * sizeof(double));
  double* forceBanded = alloc((size_t)(6 * numSeg) * sizeof(double));
  ddd_report rep;
  memset(&rep, 0, sizeof rep);

  /* calcSegSegForce(dlnParams, matParams, network) and the idx form. */
  const int rcAll = ddd_segseg_force(ctx, &k, coord, numNode, bVec, numSeg, segIdx, numSeg, NULL, numSeg, NULL, 0,
                                     force, &rep);
  const int rcIdx = ddd_segseg_force(ctx, &k, coord, numNode, bVec, numSeg, segIdx, numSeg, NULL, numSeg, idx, nIdx,
                                     forceIdx, NULL);
  /* calc_σTilde(x0, dlnParams, matParams, network). */
  const int rcSigma =
      ddd_sigma_tilde(ctx, &k, x0, M, coord, numNode, bVec, numSeg, segIdx, numSeg, numSeg, NULL, 0, sigma, NULL);
  /* The all-pairs sums in bands of tile columns (limit at its minimum). */
  const int rcLimit = ddd_set_partial_limit(ctx, 1);
  const int rcBanded = ddd_segseg_force(ctx, &k, coord, numNode, bVec, numSeg, segIdx, numSeg, NULL, numSeg, NULL, 0,
                                        forceBanded, NULL);
  const int rcReset = ddd_set_partial_limit(ctx, 0);
  /* An out-of-range node number: DDD_ERANGE and a message, nothing else. */
  int rcRange = 0;
  size_t msgLen = 0;
  if (numSeg > 0) {
    const int64_t saved = segIdx[numSeg];  /* node1 of the first segment */
    segIdx[numSeg] = numNode + 1;
    rcRange = ddd_segseg_force(ctx, &k, coord, numNode, bVec, numSeg, segIdx, numSeg, NULL, numSeg, NULL, 0, force,
                               NULL);
    msgLen = strlen(ddd_last_error(ctx));
    segIdx[numSeg] = saved;
    /* The context stays usable: the same call again, now valid. */
    const int rcAgain = ddd_segseg_force(ctx, &k, coord, numNode, bVec, numSeg, segIdx, numSeg, NULL, numSeg, NULL,
                                         0, force, NULL);
    if (rcAgain != DDD_OK) rcRange = 1000 + rcAgain;
  }
  printf("rc_all=%d rc_idx=%d rc_sigma=%d rc_limit=%d rc_banded=%d rc_reset=%d rc_range=%d msg_len=%zu "
         "pairs_general=%lld pairs_parallel=%lld version=%d\n",
         rcAll, rcIdx, rcSigma, rcLimit, rcBanded, rcReset, rcRange, msgLen, (long long)rep.pairs_general,
         (long long)rep.pairs_parallel, ddd_version());
  ddd_destroy(ctx);

  FILE* out = fopen(argv[2], "wb");
  if (!out) {
    perror(argv[2]);
    return 1;
  }
  fwrite(force, sizeof(double), (size_t)(6 * numSeg), out);
  fwrite(forceIdx, sizeof(double), (size_t)(6 * nIdx), out);
  fwrite(sigma, sizeof(double), (size_t)(6 * M), out);
  fwrite(forceBanded, sizeof(double), (size_t)(6 * numSeg), out);
  fclose(out);
  free(coord);
  free(bVec);
  free(segIdx);
  free(x0);
  free(idx);
  free(force);
  free(forceIdx);
  free(sigma);
  free(forceBanded);
  return (rcAll || rcIdx || rcSigma || rcLimit || rcBanded || rcReset) ? 1 : 0;
}
