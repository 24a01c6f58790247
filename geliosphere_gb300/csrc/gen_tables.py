"""Generate pow10_table.h: 10^k for k in [-40, 40] as exact double-double
pairs (hi + lo, |lo| <= ulp(hi)/2), from exact rational arithmetic.

The table lets device code reproduce printf("%g") -> strtod() rounding of a
value to six significant digits with a single correctly rounded step.
Run: python gen_tables.py > pow10_table.h
"""
from fractions import Fraction
import math


def dd(x: Fraction):
    hi = float(x)                     # correctly rounded (Python rounds Fractions correctly)
    lo = float(x - Fraction(hi))
    return hi, lo


def main():
    print("// Generated by gen_tables.py: 10^k = kPow10Hi[k+40] + kPow10Lo[k+40], k in [-40, 40].")
    print("#pragma once")
    his, los = [], []
    for k in range(-40, 41):
        hi, lo = dd(Fraction(10) ** k)
        his.append(hi)
        los.append(lo)
    print("static __device__ __constant__ double kPow10Hi[81] = {")
    print(",\n".join("  %r" % h for h in his))
    print("};")
    print("static __device__ __constant__ double kPow10Lo[81] = {")
    print(",\n".join("  %r" % l for l in los))
    print("};")


if __name__ == "__main__":
    main()
