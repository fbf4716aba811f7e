"""CPU oracle for film_grain's integrators -- TEST INFRASTRUCTURE ONLY.

This package is the parity checker: a plain-C restatement of the reference's
``render_pixelwise`` (src/pixelwise.rs:11-106), ``render_grainwise``
(src/grainwise.rs:12-142), the RNG streams (src/rng.rs:1-52) and the host
arithmetic around them (src/model.rs, src/params.rs:223-261, src/choose.rs,
src/color.rs).  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg may import it; the product (``film_grain_gb300``) never does.

Parity against the real Rust crates is UNPINNED (no Rust toolchain, no crate
sources, and the reference ships no tests or golden vectors); the ChaCha block
function is pinned against OpenSSL's ChaCha20 keystream (tests/golden/).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "fg_oracle.c")
_LIB = os.path.join(_HERE, "_build", "liboracle.so")

CFLAGS = ["-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-fvisibility=hidden", "-Wall", "-Wno-misleading-indentation"]


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/liboracle.so (gcc, OpenMP)."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["gcc", *CFLAGS, "-o", _LIB + ".tmp", _SRC, "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(_LIB + ".tmp", _LIB)
    return _LIB


class OParams(ctypes.Structure):
    _fields_ = [("radius_dist", ctypes.c_int32), ("radius_mean", ctypes.c_float),
                ("radius_stddev", ctypes.c_float), ("radius_log_mu", ctypes.c_float),
                ("radius_log_sigma", ctypes.c_float), ("zoom", ctypes.c_float),
                ("sigma_px", ctypes.c_float), ("n_samples", ctypes.c_uint32), ("seed", ctypes.c_uint64)]


class ODerived(ctypes.Structure):
    _fields_ = [("in_w", ctypes.c_int64), ("in_h", ctypes.c_int64), ("out_w", ctypes.c_int64),
                ("out_h", ctypes.c_int64), ("inv_e_pi_r2", ctypes.c_float), ("rm", ctypes.c_float),
                ("delta", ctypes.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.POINTER
        f32p, u32p, u64p, f64p = P(ctypes.c_float), P(ctypes.c_uint32), P(ctypes.c_uint64), P(ctypes.c_double)
        i64, u64, i32, f32 = ctypes.c_int64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_float
        sig = {
            "orc_make_offsets": (None, [u64, ctypes.c_uint32, f32, f32p]),
            "orc_radius_quantile": (f32, [P(OParams), f32]),
            "orc_lognormal_params": (None, [f32, f32, f32p]),
            "orc_default_cell_delta": (f32, [f32]),
            "orc_derive": (ctypes.c_int, [P(OParams), i64, i64, i32, f32, f32, i64, i64, P(ODerived)]),
            "orc_normalize_plane": (f32, [f32p, i64, f32p]),
            "orc_lambda_plane": (None, [f32p, i64, f32, f32p]),
            "orc_choose_algorithm": (ctypes.c_int, [P(OParams), i32, f32]),
            "orc_render_pixelwise": (ctypes.c_int, [f32p, P(OParams), P(ODerived), f32p, i64, i64, i64, i64,
                                                    f32p, u32p, i32]),
            "orc_render_grainwise": (ctypes.c_int, [f32p, P(OParams), P(ODerived), f32p, i64, i64, i64, i64,
                                                    f32p, u32p, i32]),
            "orc_luma_split": (None, [f32p, i64, f32p, f32p, f32p]),
            "orc_rgb_split": (None, [f32p, i64, f32p, f32p, f32p]),
            "orc_resize_nearest": (None, [f32p, i64, i64, i64, i64, f32p]),
            "orc_luma_to_rgb8": (None, [f32p, f32p, f32p, i64, P(ctypes.c_uint8)]),
            "orc_planes_to_rgb8": (None, [f32p, f32p, f32p, i64, P(ctypes.c_uint8)]),
            "orc_splitmix64": (u64, [u64]),
            "orc_mix3": (u64, [u64, u64, i64, i64]),
            "orc_small_stream": (None, [u64, i64, u64p]),
            "orc_cell_stream": (None, [u64, i32, i32, i32, i64, u64p]),
            "orc_chacha_block": (None, [u32p, u64, u64, i32, u32p]),
            "orc_std_stream": (None, [u64, i64, u64p]),
            "orc_std_key": (None, [u64, u32p]),
            "orc_zig_tables": (None, [f64p, f64p]),
            "orc_poisson_draws": (None, [ctypes.c_double, u64, i64, f64p]),
            "orc_normal_draws": (None, [ctypes.c_double, ctypes.c_double, u64, i64, f64p]),
            "orc_uniform_f32_draws": (None, [f32, f32, u64, i64, f32p]),
            "orc_log_gamma": (ctypes.c_double, [ctypes.c_double]),
            "orc_libm_f64": (None, [i32, ctypes.c_void_p, i64, ctypes.c_void_p]),
            "orc_threads": (i32, []),
            "orc_grain_total": (u64, [f32p, P(OParams), P(ODerived), i64, i64, i32]),
            "orc_grainwise_rows": (ctypes.c_int, [f32p, P(OParams), P(ODerived), f32p, i64, i64, u64p, i32, u64p,
                                                  i32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _p(a: np.ndarray, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


# ---------------------------------------------------------------- parameter resolution
def params_struct(radius_dist: str = "const", radius_mean: float = 0.1, radius_stddev: float = 0.0,
                  zoom: float = 1.0, sigma_px: float = 0.8, n_samples: int = 32, seed: int = 5489) -> OParams:
    """Resolved Params the integrators read (ParamsBuilder::build, src/params.rs:141-179)."""
    p = OParams()
    p.radius_dist = 1 if radius_dist == "lognorm" else 0
    p.radius_mean = radius_mean
    p.zoom = zoom
    p.sigma_px = sigma_px
    p.n_samples = max(1, int(n_samples))
    p.seed = seed & 0xFFFFFFFFFFFFFFFF
    if p.radius_dist == 1:
        out = np.zeros(3, np.float32)
        lib().orc_lognormal_params(ctypes.c_float(radius_mean), ctypes.c_float(radius_stddev), _p(out, ctypes.c_float))
        p.radius_stddev, p.radius_log_mu, p.radius_log_sigma = (float(v) for v in out)
    else:
        p.radius_stddev = 0.0
        p.radius_log_mu = 0.0
        p.radius_log_sigma = 0.0
    return p


def derive(p: OParams, in_w: int, in_h: int, max_radius=("quantile", 0.999), cell_delta: float | None = None,
           size: tuple | None = None):
    d = ODerived()
    kind = 0 if max_radius[0] == "absolute" else 1
    sw, sh = (size[0], size[1] if size[1] else 0) if size else (0, 0)
    rc = lib().orc_derive(ctypes.byref(p), in_w, in_h, kind, max_radius[1], cell_delta or 0.0, sw, sh, ctypes.byref(d))
    if rc != 0:
        raise ValueError("input image is empty")
    offs = make_offsets(p.seed, p.n_samples, p.sigma_px)
    offs_in = (offs / np.float32(p.zoom)).astype(np.float32)
    return d, offs, offs_in


def make_offsets(seed: int, n: int, sigma: float) -> np.ndarray:
    out = np.zeros((max(n, 0), 2), np.float32)
    if n:
        lib().orc_make_offsets(seed & 0xFFFFFFFFFFFFFFFF, n, sigma, _p(out, ctypes.c_float))
    return out


def normalize_plane(plane: np.ndarray):
    src = np.ascontiguousarray(plane, np.float32)
    dst = np.empty_like(src)
    mx = lib().orc_normalize_plane(_p(src, ctypes.c_float), src.size, _p(dst, ctypes.c_float))
    return dst, mx


def lambda_plane(norm: np.ndarray, inv_e_pi_r2: float) -> np.ndarray:
    src = np.ascontiguousarray(norm, np.float32)
    dst = np.empty_like(src)
    lib().orc_lambda_plane(_p(src, ctypes.c_float), src.size, inv_e_pi_r2, _p(dst, ctypes.c_float))
    return dst


def render(algo: str, lam: np.ndarray, p: OParams, d: ODerived, offs: np.ndarray, rect=None, threads: int = 0):
    """Run the oracle integrator ('pixel' takes offsets_input, 'grain' takes offsets) over rect
    (ox0, oy0, ox1, oy1), default the whole plane.  Returns (plane f32, counts u32)."""
    lam = np.ascontiguousarray(lam, np.float32)
    offs = np.ascontiguousarray(offs, np.float32)
    ox0, oy0, ox1, oy1 = rect if rect else (0, 0, d.out_w, d.out_h)
    out = np.zeros((oy1 - oy0, ox1 - ox0), np.float32)
    cnt = np.zeros((oy1 - oy0, ox1 - ox0), np.uint32)
    fn = lib().orc_render_pixelwise if algo == "pixel" else lib().orc_render_grainwise
    rc = fn(_p(lam, ctypes.c_float), ctypes.byref(p), ctypes.byref(d), _p(offs, ctypes.c_float),
            ox0, oy0, ox1, oy1, _p(out, ctypes.c_float), _p(cnt, ctypes.c_uint32), threads)
    if rc != 0:
        raise RuntimeError(f"oracle render failed: {rc}")
    return out, cnt


def choose_algorithm(p: OParams, algo: int, rm: float) -> int:
    return lib().orc_choose_algorithm(ctypes.byref(p), algo, rm)


def luma_split(rgb: np.ndarray):
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w, _ = rgb.shape
    y, cb, cr = (np.empty((h, w), np.float32) for _ in range(3))
    lib().orc_luma_split(_p(rgb, ctypes.c_float), h * w, _p(y, ctypes.c_float), _p(cb, ctypes.c_float),
                         _p(cr, ctypes.c_float))
    return y, cb, cr


def rgb_split(rgb: np.ndarray):
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w, _ = rgb.shape
    planes = [np.empty((h, w), np.float32) for _ in range(3)]
    lib().orc_rgb_split(_p(rgb, ctypes.c_float), h * w, *(_p(q, ctypes.c_float) for q in planes))
    return planes


def resize_nearest(src: np.ndarray, nw: int, nh: int) -> np.ndarray:
    src = np.ascontiguousarray(src, np.float32)
    h, w = src.shape
    dst = np.empty((nh, nw), np.float32)
    lib().orc_resize_nearest(_p(src, ctypes.c_float), w, h, nw, nh, _p(dst, ctypes.c_float))
    return dst


def luma_to_rgb8(y, cb, cr) -> np.ndarray:
    y, cb, cr = (np.ascontiguousarray(a, np.float32) for a in (y, cb, cr))
    h, w = y.shape
    out = np.empty((h, w, 3), np.uint8)
    lib().orc_luma_to_rgb8(_p(y, ctypes.c_float), _p(cb, ctypes.c_float), _p(cr, ctypes.c_float), h * w,
                           _p(out, ctypes.c_uint8))
    return out


def planes_to_rgb8(p0, p1, p2) -> np.ndarray:
    p0, p1, p2 = (np.ascontiguousarray(a, np.float32) for a in (p0, p1, p2))
    h, w = p0.shape
    out = np.empty((h, w, 3), np.uint8)
    lib().orc_planes_to_rgb8(_p(p0, ctypes.c_float), _p(p1, ctypes.c_float), _p(p2, ctypes.c_float), h * w,
                             _p(out, ctypes.c_uint8))
    return out


def render_image(rgb: np.ndarray, color_mode: str, algo: int, p: OParams, max_radius=("quantile", 0.999),
                 cell_delta=None, size=None, threads: int = 0):
    """Whole-image render (render_from_workspace_impl, src/lib.rs:134-173) -> (u8 RGB, algo used)."""
    h, w, _ = rgb.shape
    d, offs, offs_in = derive(p, w, h, max_radius, cell_delta, size)
    chosen = choose_algorithm(p, algo, d.rm)
    name = "pixel" if chosen == 2 else "grain"
    planes = luma_split(rgb) if color_mode == "luma" else rgb_split(rgb)
    todo = [planes[0]] if color_mode == "luma" else planes
    rendered = []
    for plane in todo:
        norm, _ = normalize_plane(plane)
        lam = lambda_plane(norm, d.inv_e_pi_r2)
        out, _ = render(name, lam, p, d, offs_in if name == "pixel" else offs, threads=threads)
        rendered.append(out)
    if color_mode == "luma":
        cb = resize_nearest(planes[1], d.out_w, d.out_h)
        cr = resize_nearest(planes[2], d.out_w, d.out_h)
        return luma_to_rgb8(rendered[0], cb, cr), chosen
    return planes_to_rgb8(*rendered), chosen


# ---------------------------------------------------------------- RNG probes
def splitmix64(x: int) -> int:
    return lib().orc_splitmix64(x & 0xFFFFFFFFFFFFFFFF)


def mix3(seed, stream, a, b) -> int:
    return lib().orc_mix3(seed, stream, a, b)


def small_stream(seed_u64: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint64)
    lib().orc_small_stream(seed_u64, n, _p(out, ctypes.c_uint64))
    return out


def cell_stream(seed: int, i: int, j: int, pixel: bool, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint64)
    lib().orc_cell_stream(seed, i, j, 1 if pixel else 0, n, _p(out, ctypes.c_uint64))
    return out


def chacha_block(key: np.ndarray, counter: int, stream: int, rounds: int) -> np.ndarray:
    key = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(16, np.uint32)
    lib().orc_chacha_block(_p(key, ctypes.c_uint32), counter, stream, rounds, _p(out, ctypes.c_uint32))
    return out


def std_stream(seed_u64: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint64)
    lib().orc_std_stream(seed_u64, n, _p(out, ctypes.c_uint64))
    return out


def std_key(seed_u64: int) -> np.ndarray:
    out = np.zeros(8, np.uint32)
    lib().orc_std_key(seed_u64, _p(out, ctypes.c_uint32))
    return out


def zig_tables():
    x = np.zeros(257, np.float64)
    f = np.zeros(257, np.float64)
    lib().orc_zig_tables(_p(x, ctypes.c_double), _p(f, ctypes.c_double))
    return x, f


def poisson_draws(lam: float, seed_u64: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float64)
    lib().orc_poisson_draws(lam, seed_u64, n, _p(out, ctypes.c_double))
    return out


def normal_draws(mean: float, sd: float, seed_u64: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float64)
    lib().orc_normal_draws(mean, sd, seed_u64, n, _p(out, ctypes.c_double))
    return out


def uniform_f32_draws(low: float, high: float, seed_u64: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().orc_uniform_f32_draws(low, high, seed_u64, n, _p(out, ctypes.c_float))
    return out


def log_gamma(x: float) -> float:
    return lib().orc_log_gamma(x)


def libm_f64(name: str, x: np.ndarray) -> np.ndarray:
    """The platform libm's exp / log / tan on f64 values (the crate's samplers call these)."""
    src = np.ascontiguousarray(x, np.float64)
    out = np.empty_like(src)
    lib().orc_libm_f64({"exp": 0, "log": 1, "tan": 2}[name], src.ctypes.data, src.size, out.ctypes.data)
    return out


def threads() -> int:
    return lib().orc_threads()


# ---------------------------------------------------------------- bench support
def grain_total(lam: np.ndarray, p: OParams, d: ODerived, rows=None, threads: int = 0) -> int:
    lam = np.ascontiguousarray(lam, np.float32)
    y0, y1 = rows if rows else (0, d.in_h)
    return int(lib().orc_grain_total(_p(lam, ctypes.c_float), ctypes.byref(p), ctypes.byref(d), y0, y1, threads))


def grainwise_rows(lam: np.ndarray, p: OParams, d: ODerived, offs: np.ndarray, rows, count: bool = False,
                   threads: int = 0, bits: np.ndarray = None):
    """The reference's grain-wise work for input rows [y0, y1) over the whole output plane.
    Returns (stats[4] = grains, x-bounds pairs, x-and-y-bounds pairs, bits set; bit planes)."""
    lam = np.ascontiguousarray(lam, np.float32)
    offs = np.ascontiguousarray(offs, np.float32)
    lanes = (p.n_samples + 63) // 64
    if bits is None:
        bits = np.zeros(d.out_w * d.out_h * lanes, np.uint64)
    else:
        bits[:] = 0
    stats = np.zeros(4, np.uint64)
    lib().orc_grainwise_rows(_p(lam, ctypes.c_float), ctypes.byref(p), ctypes.byref(d), _p(offs, ctypes.c_float),
                             rows[0], rows[1], _p(bits, ctypes.c_uint64), 1 if count else 0, _p(stats, ctypes.c_uint64),
                             threads)
    return stats, bits
