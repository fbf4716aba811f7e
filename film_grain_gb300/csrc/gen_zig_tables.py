"""Generate zig_tables.h: the 256-layer ziggurat tables of the standard normal.

The tables follow the published ZIGNOR construction (Marsaglia & Tsang 2000, "The Ziggurat
Method for Generating Random Variables"; Doornik 2005, "An Improved Ziggurat Method"):
x_0 = v / f(r), x_1 = r, x_i = f^-1(v / x_{i-1} + f(x_{i-1})) for i = 2..255, x_256 = 0 and
F_i = f(x_i), with f(x) = exp(-x^2/2), r = 3.6541528853610088, v = 0.00492867323399.
rand_distr 0.4.3's StandardNormal (used by film_grain's make_offsets, src/rng.rs:14-20, and by the
lognormal radius, src/model.rs:141-142) samples with tables built this way and stored as 18-decimal
literals, so each value here is rounded through the same "%.18f" text form.

Run:  python gen_zig_tables.py > zig_tables.h
"""
from math import exp, log, sqrt

TABLE_LEN = 256
R = 3.6541528853610088
V = 0.00492867323399


def f(x: float) -> float:
    return exp(-x * x / 2.0)


def f_inv(y: float) -> float:
    return sqrt(-2.0 * log(y))


def tables():
    xs = [0.0] * (TABLE_LEN + 1)
    xs[0] = V / f(R)
    xs[1] = R
    for i in range(2, TABLE_LEN):
        last = xs[i - 1]
        xs[i] = f_inv(V / last + f(last))
    fs = [f(x) for x in xs]
    return xs, fs


def main() -> None:
    xs, fs = tables()
    print("/* Generated by gen_zig_tables.py -- do not edit. 256-layer ZIGNOR normal tables. */")
    print("#pragma once")
    print("#define FG_ZIG_NORM_R %.18f" % R)
    for name, vals in (("FG_ZIG_NORM_X", xs), ("FG_ZIG_NORM_F", fs)):
        print("#define %s_INIT { \\" % name)
        for i in range(0, len(vals), 4):
            row = ", ".join("%.18f" % v for v in vals[i:i + 4])
            print("    %s%s \\" % (row, "," if i + 4 < len(vals) else ""))
        print("}")


if __name__ == "__main__":
    main()
