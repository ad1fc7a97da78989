"""Generates int_tables.h: the fixed-point tables of the integer-pipe logarithm
and arctangent in intmath_f64.cuh.

  kILogC[j]  = C_j, j = 0..255: m in [1 + j/256, 1 + (j+1)/256) is reduced to
               r = m C_j / 1024 - 1 (j < kILogHalfJ) or r = (m/2) C_j / 512 - 1
               (j >= kILogHalfJ, the exponent then counts one more), with
               C_j = round(1024 / (1 + (j + 1/2)/256)) except C_0 = 1024 and
               C_255 = 512, so that r = m - 1 and r = m/2 - 1 exactly next to 1.
  kILogL[j]  = -ln(C_j / 1024) or -ln(C_j / 512), fixed point 2^-116, as
               (lo, hi) two's complement words.
  kILn2      = ln 2, fixed point 2^-116.
  kIAtanT[j] = atan(j/64) and kIAtanTC[j] = pi/2 - atan(j/64), j = 0..64,
               fixed point 2^-120.
Values come from mpmath at 80 digits, rounded to the nearest unit of the fixed
point.  The script also checks the reduction bound |r| <= 2^-8 that the
logarithm's series relies on.  Run: python gen_int_tables.py > int_tables.h
"""
import mpmath

mpmath.mp.dps = 80
HALF_J = 106  # 1 + 106/256 = 1.4140625, next to sqrt(2)


def fixed(v, scale):
    return int(mpmath.nint(v * mpmath.mpf(2) ** scale))


def words(v):
    u = v & ((1 << 128) - 1)
    return "{0x%016xULL, 0x%016xULL}" % (u & ((1 << 64) - 1), u >> 64)


def log_tables():
    C, L = [], []
    rmax = mpmath.mpf(0)
    for j in range(256):
        half = j >= HALF_J
        if j == 0:
            c = 1024
        elif j == 255:
            c = 512
        else:
            c = int(mpmath.nint(1024 / (1 + (mpmath.mpf(j) + mpmath.mpf(1) / 2) / 256)))
        # r + 1 = M c 2^-62 with M = m 2^52, over m in [1 + j/256, 1 + (j+1)/256).
        lo, hi = 1 + mpmath.mpf(j) / 256, 1 + mpmath.mpf(j + 1) / 256
        for m in (lo, hi):
            rmax = max(rmax, abs(m * c / 1024 - 1))
        C.append(c)
        L.append(fixed(-mpmath.log(mpmath.mpf(c) / (512 if half else 1024)), 116))
    assert rmax <= mpmath.mpf(2) ** -8, rmax  # j = 0: r = m - 1 < 2^-8; the other bins < 2^-8.5
    return C, L


def main():
    out = ["// Generated by gen_int_tables.py; do not edit.", "#pragma once", ""]
    C, L = log_tables()
    out.append("#define IM_LOG_HALF_J %d" % HALF_J)
    out.append("static const IM_TABLE_QUAL unsigned int kILogC[256] = {\n  %s};"
               % ",\n  ".join(", ".join(str(c) for c in C[k:k + 16]) for k in range(0, 256, 16)))
    out.append("static const IM_TABLE_QUAL im_u128 kILogL[256] = {\n  %s};" % ",\n  ".join(words(v) for v in L))
    ln2 = fixed(mpmath.log(2), 116)
    out.append("static constexpr unsigned long long kILn2Lo = 0x%016xULL, kILn2Hi = 0x%016xULL;"
               % (ln2 & ((1 << 64) - 1), ln2 >> 64))
    T = [fixed(mpmath.atan(mpmath.mpf(j) / 64), 120) for j in range(65)]
    TC = [fixed(mpmath.pi / 2 - mpmath.atan(mpmath.mpf(j) / 64), 120) for j in range(65)]
    out.append("static const IM_TABLE_QUAL im_u128 kIAtanT[65] = {\n  %s};" % ",\n  ".join(words(v) for v in T))
    out.append("static const IM_TABLE_QUAL im_u128 kIAtanTC[65] = {\n  %s};" % ",\n  ".join(words(v) for v in TC))
    print("\n".join(out))


if __name__ == "__main__":
    main()
