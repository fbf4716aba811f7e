"""Generate exp_table.h: exp(j/64) for j = -24..24 as (hi, lo) float pairs.

hi = RN_f32(exp(j/64)), lo = RN_f32(exp(j/64) - hi), computed with 60-digit decimal arithmetic, so
hi + lo carries exp(j/64) to about 2^-48 relative.  Used by the double-float exp of the lognormal
radius draw (fg_rng.cuh).

Run:  python gen_exp_table.py > exp_table.h
"""
from decimal import Decimal, getcontext

import numpy as np

getcontext().prec = 60


def main():
    print("/* Generated by gen_exp_table.py -- do not edit. exp(j/64), j = -24..24, as float pairs. */")
    print("#pragma once")
    print("#define FG_EXP64_TABLE_INIT { \\")
    rows = []
    for j in range(-24, 25):
        v = (Decimal(j) / Decimal(64)).exp()
        hi = np.float32(float(v))
        lo = np.float32(float(v - Decimal(float(hi))))
        rows.append("    {%sf, %sf}" % (np.format_float_scientific(hi, unique=True),
                                        np.format_float_scientific(lo, unique=True)))
    print(", \\\n".join(rows) + " \\")
    print("}")


if __name__ == "__main__":
    main()
