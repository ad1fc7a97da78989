"""Generates df64_tables.h: double-float (hi, lo) constants for the DF log and atan.

  log table: ln(c_j), c_j = 1 + (j + 0.5)/64, j = 0..63 (reduction to |u| < 2^-8)
  atan table: atan(j/32), j = 0..32
  ln 2, pi/2, 1/3
Values come from mpmath at 60 digits; hi = nearest float, lo = nearest float of
the remainder.  Run: python gen_df64_tables.py > df64_tables.h
"""
import struct

import mpmath

mpmath.mp.dps = 60


def f32(x):
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def split(x):
    hi = f32(x)
    lo = f32(x - mpmath.mpf(hi))
    return hi, lo


def lit(v):
    return "%.9ef" % v


def row(name, vals):
    items = ",\n  ".join("{%s, %s}" % (lit(h), lit(l)) for h, l in vals)
    return "static const DDD_DF_TABLE_QUAL float2_ %s[%d] = {\n  %s};\n" % (name, len(vals), items)


def main():
    log = [split(mpmath.log(1 + (mpmath.mpf(j) + mpmath.mpf("0.5")) / 64)) for j in range(64)]
    atan = [split(mpmath.atan(mpmath.mpf(j) / 32)) for j in range(33)]
    out = ["// Generated by gen_df64_tables.py; do not edit.", "#pragma once", ""]
    out.append(row("kDfLogC", log))
    out.append(row("kDfAtanC", atan))
    for name, v in (("kDfLn2", mpmath.log(2)), ("kDfPiHalf", mpmath.pi / 2), ("kDfThird", mpmath.mpf(1) / 3)):
        h, l = split(v)
        out.append("#define %s_HI %s\n#define %s_LO %s" % (name, lit(h), name, lit(l)))
    print("\n".join(out))


if __name__ == "__main__":
    main()
