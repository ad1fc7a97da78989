"""Generates f64_tables.h: the FP64 tables of the table-driven log and atan in
fastmath_f64.cuh.

  kLogInvC[j]  = 1 / c_j rounded to double, c_j = 1 + j/256, j = 0..256
  kLogC[j]     = ln(c_j) as (hi, lo), hi the nearest double, lo the nearest
                 double of the remainder
  kLogHalfC[j] = ln(c_j / 2) as (hi, lo)
  kAtanC[j]    = (j/64, atan(j/64) hi, lo), j = 0..64
  kAtanCompC[j]= (j/64, pi/2 - atan(j/64) hi, lo)
  ln 2 as (hi, lo) with hi rounded to 32 significant bits, so that k * hi is
  exact for |k| < 2^21.
Values come from mpmath at 60 digits and are written as C99 hexadecimal
floating literals (exact).  Run: python gen_f64_tables.py > f64_tables.h
"""
import mpmath

mpmath.mp.dps = 60


def split(x):
    hi = float(x)
    lo = float(x - mpmath.mpf(hi))
    return hi, lo


def h(v):
    return float(v).hex()


def main():
    out = ["// Generated by gen_f64_tables.py; do not edit.", "#pragma once", ""]
    inv = [h(mpmath.mpf(1) / (1 + mpmath.mpf(j) / 256)) for j in range(257)]
    out.append("static const FM_TABLE_QUAL double kLogInvC[257] = {\n  %s};" % ",\n  ".join(inv))
    for name, f in (("kLogC", lambda c: mpmath.log(c)), ("kLogHalfC", lambda c: mpmath.log(c / 2))):
        rows = []
        for j in range(257):
            hi, lo = split(f(1 + mpmath.mpf(j) / 256))
            rows.append("{%s, %s}" % (h(hi), h(lo)))
        out.append("static const FM_TABLE_QUAL fm_d2 %s[257] = {\n  %s};" % (name, ",\n  ".join(rows)))
    for name, f in (("kAtanC", lambda c: mpmath.atan(c)), ("kAtanCompC", lambda c: mpmath.pi / 2 - mpmath.atan(c))):
        rows = []
        for j in range(65):
            c = mpmath.mpf(j) / 64
            hi, lo = split(f(c))
            rows.append("{%s, %s, %s}" % (h(c), h(hi), h(lo)))
        out.append("static const FM_TABLE_QUAL fm_d3 %s[65] = {\n  %s};" % (name, ",\n  ".join(rows)))
    ln2 = mpmath.log(2)
    m, e = mpmath.frexp(ln2)
    hi = mpmath.ldexp(mpmath.floor(m * 2 ** 32), e - 32)
    out.append("#define FM_LN2_HI %s" % h(hi))
    out.append("#define FM_LN2_LO %s" % h(ln2 - hi))
    print("\n".join(out))


if __name__ == "__main__":
    main()
