// Host-side validation of one row of a DislocationNetwork's segIdx, shared by
// the entry points that take the network's own arrays (ddd_api.cu,
// surrogate_force.cu).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/ddd_gb300.h"

namespace ddd {

inline bool finite3(const double* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

// Row r (0-based) of segIdx (ld x 3, column-major, 1-based link / node
// numbers): indices in range, finite coordinates and Burgers vector, non-zero
// length.  DDD_OK, or a DDD_E* code with the message in `msg`.
inline int check_segment_row(const double* coord, int64_t coordCols, const double* bVec, int64_t bVecCols,
                             const int64_t* segIdx, int64_t ld, int64_t r, std::string& msg) {
  const int64_t l = segIdx[r], a = segIdx[r + ld], b = segIdx[r + 2 * ld];
  char buf[160];
  if (l < 1 || l > bVecCols || a < 1 || a > coordCols || b < 1 || b > coordCols) {
    snprintf(buf, sizeof buf, "segIdx row %lld = (%lld, %lld, %lld) out of range (bVec cols %lld, coord cols %lld)",
             (long long)(r + 1), (long long)l, (long long)a, (long long)b, (long long)bVecCols,
             (long long)coordCols);
    msg = buf;
    return DDD_ERANGE;
  }
  const double* p1 = coord + 3 * (a - 1);
  const double* p2 = coord + 3 * (b - 1);
  const double* bv = bVec + 3 * (l - 1);
  if (!finite3(p1) || !finite3(p2) || !finite3(bv)) {
    snprintf(buf, sizeof buf, "segment %lld has a non-finite coordinate or Burgers vector", (long long)(r + 1));
    msg = buf;
    return DDD_ENONFINITE;
  }
  if (p1[0] == p2[0] && p1[1] == p2[1] && p1[2] == p2[2]) {
    snprintf(buf, sizeof buf, "segment %lld has zero length", (long long)(r + 1));
    msg = buf;
    return DDD_ENONFINITE;
  }
  return DDD_OK;
}

}  // namespace ddd
