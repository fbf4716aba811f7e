"""CPU tests that compile small native checkers against the library's shared host/device headers."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(src, out, tmp_path):
    exe = str(tmp_path / out)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                    os.path.join(ROOT, "film_grain_gb300", "csrc"), "-o", exe, os.path.join(ROOT, "tests", "native", src),
                    "-lm"], check=True)
    return exe


def test_double_float_exp_matches_f64_exp_rounded(tmp_path):
    """exp_f64_to_f32 (the lognormal radius path) equals (float)exp(t) of the platform libm on 4M
    arguments, falling back to the f64 exp only within 2^-40 of an f32 rounding midpoint."""
    exe = _compile("exp_check.cpp", "exp_check", tmp_path)
    out = subprocess.run([exe, "2000000"], check=True, capture_output=True, text=True).stdout.split()
    checked, bad, fallbacks = (int(v) for v in out[-3:])
    assert checked == 4000000 and bad == 0
    assert fallbacks < checked * 1e-3
