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


def test_library_small_rng_seeding_matches_rand_core_default(tmp_path):
    """The library's SmallRng seeding (fg_rng.cuh: eight PCG32 words by jump-ahead, the emptiness
    shortcut small_first_u64, the all-zero remap) against the serial restatement of rand_core 0.6.4's
    seed_from_u64 in tests/test_oracle.py."""
    from test_oracle import M64, _splitmix_py, _xoshiro_py, _small_rng_py
    exe = _compile("rng_check.cpp", "rng_check", tmp_path)
    hs = [0, 1, 42, M64, 0x8000000000000000, 0xDEADBEEFCAFEF00D] + [_splitmix_py(k) for k in range(200)]
    out = subprocess.run([exe], input="\n".join(str(h) for h in hs), check=True, capture_output=True,
                         text=True).stdout.strip().splitlines()
    assert len(out) == len(hs) + 1
    for h, line in zip(hs, out):
        v = [int(t) for t in line.split()]
        assert v[:4] == _small_rng_py(h), h
        draws = _xoshiro_py(h, 4)
        assert v[4:8] == draws and v[8] == draws[0], h
    st, zero = 0, []
    for _ in range(4):
        st = (st + 0x9E3779B97F4A7C15) & M64
        zero.append(_splitmix_py(st - 0x9E3779B97F4A7C15 & M64))
    assert [int(t) for t in out[-1].split()] == zero


def test_bitmask_screen_and_row_hash_identities(tmp_path):
    """The sparse pass's emptiness bitmask: the one-compare first-draw screen agrees with the draw's own
    threshold test on every threshold around each draw and at the edges, and a word's row-hash inputs
    are one rotated constant plus r * 2^41 when the rows carry nothing out of the low 23 bits."""
    exe = _compile("screen_check.cpp", "screen_check", tmp_path)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    checked, bad, checked2, bad2 = (int(v) for v in out)
    assert checked == 200000 * 13 and bad == 0
    assert checked2 > 6000000 and bad2 == 0
