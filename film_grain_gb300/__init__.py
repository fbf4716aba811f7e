"""film_grain_gb300 -- GB300 (sm_103a) Monte Carlo film-grain integrators.

A drop-in for the hot path of joseph-wardle/film_grain: the pixel-wise and grain-wise integrators
(src/pixelwise.rs, src/grainwise.rs), their RNG streams (src/rng.rs) and the host arithmetic of the
crate's render entry points (src/params.rs, src/model.rs, src/choose.rs, src/color.rs, src/lib.rs).
Every call goes through the C-ABI of ``libfg_gb300.so`` (include/film_grain_gb300.h); this module
mirrors the crate's names, argument meanings and errors:

    params = ParamsBuilder(radius_mean=0.12, n_samples=64, seed=42).build()
    derived = derive_common(params, (width, height))
    lam = lambda_plane(normalize_plane(plane)[0], derived.inv_e_pi_r2)
    out = render_pixelwise(lam, params, derived)            # numpy in -> numpy out
    out = render_grainwise(lam_cuda_tensor, params, derived)  # torch CUDA tensor in -> tensor out
    image, stats = render_with_input_image(rgb_f32, params)   # whole image, u8 RGB out

There is no CPU fallback: without the native library (or without a GPU for the render calls) the
calls raise.
"""
from __future__ import annotations

import ctypes
import enum
import os
import threading
from dataclasses import dataclass, field
from typing import Callable, Optional, Tuple

import numpy as np

__all__ = [
    "RadiusDist", "Algo", "ColorMode", "MaxRadius", "Roi", "ParamsBuilder", "Params", "Derived", "RenderStats",
    "RenderError", "ParamsError", "CancelledError", "GpuError", "derive_common", "default_cell_delta",
    "normalize_plane", "lambda_plane", "lambda_from_plane", "choose_algorithm", "render_pixelwise", "render_grainwise",
    "render_with_input_image", "dry_run_with_input_image", "lib", "pixelwise_diagnostics", "pixelwise_sparse_forms", "pixelwise_kernel_count",
    "make_offsets",
    "Batch", "BatchTuning",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfg_gb300.so")


class RadiusDist(enum.IntEnum):
    Const = 0
    Lognorm = 1


class Algo(enum.IntEnum):
    Auto = 0
    Grain = 1
    Pixel = 2


class ColorMode(enum.IntEnum):
    Luma = 0
    Rgb = 1


@dataclass(frozen=True)
class MaxRadius:
    """MaxRadius::Absolute(v) / MaxRadius::Quantile(p) (src/params.rs:38-42)."""
    kind: str
    value: float

    @staticmethod
    def Absolute(v: float) -> "MaxRadius":
        return MaxRadius("absolute", float(v))

    @staticmethod
    def Quantile(p: float) -> "MaxRadius":
        return MaxRadius("quantile", float(p))


@dataclass(frozen=True)
class Roi:
    x0: int
    y0: int
    x1: int
    y1: int


# ------------------------------------------------------------------ errors (RenderError, src/lib.rs:28-44)
class RenderError(RuntimeError):
    """Base of the render errors; ``code`` is the C-ABI fg_status."""

    def __init__(self, msg: str, code: int):
        super().__init__(msg)
        self.code = code


class ParamsError(RenderError, ValueError):
    pass


class CancelledError(RenderError):
    pass


class GpuError(RenderError):
    pass


_FG_OK, _FG_PARAMS, _FG_CANCELLED, _FG_CUDA, _FG_INVALID, _FG_UNSUPPORTED, _FG_NOMEM, _FG_INTERNAL = range(8)


# ------------------------------------------------------------------ C structs
class _BuilderC(ctypes.Structure):
    _fields_ = [("radius_dist", ctypes.c_int32), ("radius_mean", ctypes.c_float), ("radius_stddev", ctypes.c_float),
                ("zoom", ctypes.c_float), ("sigma_px", ctypes.c_float), ("n_samples", ctypes.c_uint32),
                ("algo", ctypes.c_int32), ("max_radius_kind", ctypes.c_int32), ("max_radius_value", ctypes.c_float),
                ("cell_delta", ctypes.c_float), ("color_mode", ctypes.c_int32), ("has_roi", ctypes.c_int32),
                ("roi_x0", ctypes.c_uint32), ("roi_y0", ctypes.c_uint32), ("roi_x1", ctypes.c_uint32),
                ("roi_y1", ctypes.c_uint32), ("size_w", ctypes.c_uint32), ("size_h", ctypes.c_uint32),
                ("seed", ctypes.c_uint64)]


class _ParamsC(ctypes.Structure):
    _fields_ = [("radius_dist", ctypes.c_int32), ("radius_mean", ctypes.c_float), ("radius_stddev", ctypes.c_float),
                ("radius_log_mu", ctypes.c_float), ("radius_log_sigma", ctypes.c_float),
                ("has_log_params", ctypes.c_int32), ("zoom", ctypes.c_float), ("sigma_px", ctypes.c_float),
                ("n_samples", ctypes.c_uint32), ("algo", ctypes.c_int32), ("max_radius_kind", ctypes.c_int32),
                ("max_radius_value", ctypes.c_float), ("cell_delta", ctypes.c_float), ("color_mode", ctypes.c_int32),
                ("has_roi", ctypes.c_int32), ("roi_x0", ctypes.c_uint32), ("roi_y0", ctypes.c_uint32),
                ("roi_x1", ctypes.c_uint32), ("roi_y1", ctypes.c_uint32), ("size_w", ctypes.c_uint32),
                ("size_h", ctypes.c_uint32), ("seed", ctypes.c_uint64)]


class _DerivedC(ctypes.Structure):
    _fields_ = [("input_width", ctypes.c_int64), ("input_height", ctypes.c_int64), ("output_width", ctypes.c_int64),
                ("output_height", ctypes.c_int64), ("inv_e_pi_r2", ctypes.c_float), ("rm", ctypes.c_float),
                ("delta", ctypes.c_float), ("n_offsets", ctypes.c_uint32)]


class _StatsC(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int32), ("input_width", ctypes.c_int64), ("input_height", ctypes.c_int64),
                ("output_width", ctypes.c_int64), ("output_height", ctypes.c_int64), ("n_samples", ctypes.c_uint32),
                ("sigma_ratio", ctypes.c_float), ("rm_ratio", ctypes.c_float)]


class _BatchImageC(ctypes.Structure):
    _fields_ = [("algo", ctypes.c_int32), ("params", ctypes.POINTER(_ParamsC)), ("derived", ctypes.POINTER(_DerivedC)),
                ("offsets", ctypes.c_void_p), ("d_lambda", ctypes.c_void_p), ("d_out", ctypes.c_void_p),
                ("h_lambda", ctypes.c_void_p)]


class _SgNetC(ctypes.Structure):
    _fields_ = [("n_res", ctypes.c_int32), ("radius_scale", ctypes.c_float), ("w_in", ctypes.c_void_p),
                ("b_in", ctypes.c_void_p), ("w_res", ctypes.c_void_p), ("b_res", ctypes.c_void_p),
                ("w_out", ctypes.c_void_p), ("b_out", ctypes.c_void_p)]


class BatchTuning(ctypes.Structure):
    """fg_batch_tuning: grain-wise tile mask budget, pixel-wise block edge, persistent CTAs per SM."""
    _fields_ = [("grain_mask_words", ctypes.c_int32), ("pixel_max_block_log2", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32)]

    def __repr__(self):
        return (f"BatchTuning(grain_mask_words={self.grain_mask_words}, "
                f"pixel_max_block_log2={self.pixel_max_block_log2}, ctas_per_sm={self.ctas_per_sm})")


# Every symbol include/film_grain_gb300.h declares, with its ctypes signature.
_P = ctypes.POINTER
_f32p = _P(ctypes.c_float)
_vp = ctypes.c_void_p
SIGNATURES = {
    "fg_params_build": (ctypes.c_int, [_P(_BuilderC), _P(_ParamsC)]),
    "fg_derive": (ctypes.c_int, [_P(_ParamsC), ctypes.c_int64, ctypes.c_int64, _P(_DerivedC), _vp, _vp]),
    "fg_choose_algorithm": (ctypes.c_int32, [_P(_ParamsC), _P(_DerivedC)]),
    "fg_default_cell_delta": (ctypes.c_float, [ctypes.c_float]),
    "fg_normalize_plane": (ctypes.c_float, [_vp, ctypes.c_int64, _vp]),
    "fg_lambda_plane": (None, [_vp, ctypes.c_int64, ctypes.c_float, _vp]),
    "fg_lambda_from_plane": (ctypes.c_float, [_vp, ctypes.c_int64, ctypes.c_float, _vp]),
    "fg_render_pixelwise": (ctypes.c_int, [_vp, _P(_ParamsC), _P(_DerivedC), _vp, _vp, _vp, _vp]),
    "fg_render_grainwise": (ctypes.c_int, [_vp, _P(_ParamsC), _P(_DerivedC), _vp, _vp, _vp, _vp]),
    "fg_render_pixelwise_async": (ctypes.c_int, [_vp, _P(_ParamsC), _P(_DerivedC), _vp, _vp, _vp]),
    "fg_render_grainwise_async": (ctypes.c_int, [_vp, _P(_ParamsC), _P(_DerivedC), _vp, _vp, _vp]),
    "fg_render_pixelwise_noalloc": (ctypes.c_int, [_vp, _P(_ParamsC), _P(_DerivedC), _vp, _vp, _vp]),
    "fg_render_image": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, _P(_ParamsC), _vp, _P(_StatsC), _vp,
                                       _vp]),
    "fg_dry_run": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, _P(_ParamsC), _P(_StatsC)]),
    "fg_last_error_message": (ctypes.c_char_p, []),
    "fg_version": (ctypes.c_char_p, []),
    "fg_pixelwise_diagnostics": (None, [_P(ctypes.c_ulonglong)]),
    "fg_pixelwise_sparse_forms": (None, [_P(ctypes.c_ulonglong)]),
    "fg_pixelwise_kernel_count": (ctypes.c_int, [_P(_ParamsC), _P(_DerivedC), ctypes.c_void_p, _P(ctypes.c_int32)]),
    "fg_batch_create": (ctypes.c_int, [_P(_BatchImageC), ctypes.c_int32, _P(BatchTuning), _P(ctypes.c_void_p)]),
    "fg_batch_run": (ctypes.c_int, [ctypes.c_void_p, _vp]),
    "fg_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "fg_batch_get_tuning": (ctypes.c_int, [ctypes.c_void_p, _P(BatchTuning)]),
    "fg_batch_kernel_count": (ctypes.c_int, [ctypes.c_void_p, _P(ctypes.c_int32)]),
    "fg_batch_autotune": (ctypes.c_int, [_P(_BatchImageC), ctypes.c_int32, _vp, _P(BatchTuning),
                                         _P(ctypes.c_float)]),
    "fg_sg_conv_forward": (ctypes.c_int, [ctypes.c_int32, _vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                          ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _vp]),
    "fg_sg_conv_wgrad": (ctypes.c_int, [ctypes.c_int32, _vp, ctypes.c_int32, _vp, ctypes.c_int32, _vp, _vp,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _vp]),
    "fg_sg_mask_grad": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, _vp]),
    "fg_sg_flip_weights": (ctypes.c_int, [_vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          _vp]),
    "fg_sg_adam": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_int64,
                                  ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int32,
                                  _vp]),
    "fg_sg_make_input": (ctypes.c_int, [_vp, _vp, ctypes.c_float, ctypes.c_uint64, _vp, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32, _vp]),
    "fg_sg_mse_grad": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_float, _vp]),
    "fg_sg_infer_workspace_bytes": (ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "fg_sg_infer": (ctypes.c_int, [_P(_SgNetC), _vp, _vp, ctypes.c_uint64, _vp, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.c_int32, _vp, ctypes.c_size_t, _vp]),
}

_lib: Optional[ctypes.CDLL] = None


def lib() -> ctypes.CDLL:
    """The native library; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"film_grain_gb300 native library missing: {LIB_PATH} "
                              "(build it with film_grain_gb300.build.build())")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def _raise(code: int):
    if code == _FG_OK:
        return
    msg = (lib().fg_last_error_message() or b"").decode()
    if code == _FG_PARAMS:
        raise ParamsError(msg, code)
    if code == _FG_CANCELLED:
        raise CancelledError(msg or "cancelled", code)
    if code in (_FG_CUDA, _FG_NOMEM, _FG_INTERNAL):
        raise GpuError(msg, code)
    raise RenderError(msg, code)


# ------------------------------------------------------------------ params
@dataclass
class ParamsBuilder:
    """ParamsBuilder (src/params.rs:70-91); defaults are the CLI's (src/main.rs:94-247)."""
    radius_mean: float = 0.10
    radius_dist: RadiusDist = RadiusDist.Const
    radius_stddev: float = 0.0
    zoom: float = 1.0
    sigma_px: float = 0.8
    n_samples: int = 32
    algo: Algo = Algo.Auto
    max_radius: MaxRadius = field(default_factory=lambda: MaxRadius.Quantile(0.999))
    cell_delta: Optional[float] = None
    color_mode: ColorMode = ColorMode.Luma
    roi: Optional[Roi] = None
    size: Optional[Tuple[int, Optional[int]]] = None
    seed: int = 5489

    def build(self) -> "Params":
        b = _BuilderC()
        b.radius_dist = int(self.radius_dist)
        b.radius_mean = self.radius_mean
        b.radius_stddev = self.radius_stddev
        b.zoom = self.zoom
        b.sigma_px = self.sigma_px
        b.n_samples = max(0, int(self.n_samples))
        b.algo = int(self.algo)
        b.max_radius_kind = 0 if self.max_radius.kind == "absolute" else 1
        b.max_radius_value = self.max_radius.value
        b.cell_delta = float("nan") if self.cell_delta is None else float(self.cell_delta)
        b.color_mode = int(self.color_mode)
        if self.roi is not None:
            b.has_roi = 1
            b.roi_x0, b.roi_y0, b.roi_x1, b.roi_y1 = self.roi.x0, self.roi.y0, self.roi.x1, self.roi.y1
        if self.size is not None:
            w, h = self.size
            if w == 0:
                raise ParamsError("parameter error: size: output width must be > 0", _FG_PARAMS)
            if h is not None and h == 0:
                raise ParamsError("parameter error: size: output height must be > 0", _FG_PARAMS)
            b.size_w, b.size_h = int(w), int(h or 0)
        b.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        out = _ParamsC()
        _raise(lib().fg_params_build(ctypes.byref(b), ctypes.byref(out)))
        return Params(out)


class Params:
    """Resolved Params (src/params.rs:45-68) backed by the C struct."""

    def __init__(self, c: _ParamsC):
        self._c = c

    def __getattr__(self, name):
        return getattr(self._c, name)

    @property
    def c(self) -> _ParamsC:
        return self._c

    def __repr__(self):
        fields = ", ".join(f"{n}={getattr(self._c, n)!r}" for n, _ in _ParamsC._fields_)
        return f"Params({fields})"


@dataclass
class Derived:
    """Derived (src/model.rs:167-179)."""
    input_width: int
    input_height: int
    output_width: int
    output_height: int
    inv_e_pi_r2: float
    rm: float
    delta: float
    offsets: np.ndarray
    offsets_input: np.ndarray
    _c: _DerivedC = field(repr=False, default=None)


@dataclass
class RenderStats:
    """RenderStats (src/lib.rs:46-55)."""
    algorithm: Algo
    input_size: Tuple[int, int]
    output_size: Tuple[int, int]
    n_samples: int
    sigma_ratio: float
    rm_ratio: float


def _stats(s: _StatsC) -> RenderStats:
    return RenderStats(Algo(s.algorithm), (s.input_width, s.input_height), (s.output_width, s.output_height),
                       s.n_samples, s.sigma_ratio, s.rm_ratio)


def default_cell_delta(radius_mean: float) -> float:
    return lib().fg_default_cell_delta(radius_mean)


def derive_common(params: Params, input_size: Tuple[int, int]) -> Derived:
    """derive_common (src/model.rs:181-226), including make_offsets (src/rng.rs:9-24)."""
    w, h = input_size
    n = params.n_samples
    offs = np.zeros((n, 2), np.float32)
    offs_in = np.zeros((n, 2), np.float32)
    d = _DerivedC()
    _raise(lib().fg_derive(ctypes.byref(params.c), int(w), int(h), ctypes.byref(d), offs.ctypes.data,
                           offs_in.ctypes.data))
    return Derived(d.input_width, d.input_height, d.output_width, d.output_height, d.inv_e_pi_r2, d.rm, d.delta,
                   offs, offs_in, d)


def make_offsets(params: Params) -> np.ndarray:
    return derive_common(params, (1, 1)).offsets


def normalize_plane(plane: np.ndarray) -> Tuple[np.ndarray, float]:
    src = np.ascontiguousarray(plane, np.float32)
    dst = np.empty_like(src)
    mx = lib().fg_normalize_plane(src.ctypes.data, src.size, dst.ctypes.data)
    return dst, mx


def lambda_from_plane(plane: np.ndarray, inv_e_pi_r2: float) -> Tuple[np.ndarray, float]:
    """lambda_plane(normalize_plane(plane)) in one host pass (bit-identical); returns (lambda, max)."""
    src = np.ascontiguousarray(plane, np.float32)
    dst = np.empty_like(src)
    mx = lib().fg_lambda_from_plane(src.ctypes.data, src.size, inv_e_pi_r2, dst.ctypes.data)
    return dst, mx


def lambda_plane(normalized: np.ndarray, inv_e_pi_r2: float) -> np.ndarray:
    src = np.ascontiguousarray(normalized, np.float32)
    dst = np.empty_like(src)
    lib().fg_lambda_plane(src.ctypes.data, src.size, inv_e_pi_r2, dst.ctypes.data)
    return dst


def choose_algorithm(params: Params, derived: Derived) -> Algo:
    return Algo(lib().fg_choose_algorithm(ctypes.byref(params.c), ctypes.byref(derived._c)))


# ------------------------------------------------------------------ integrators
def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


class _Cancel:
    """The crate's cancel closure (Fn() -> bool, polled per row / pixel / grain in the CPU path) as the
    flag the library reads: evaluated once before the call and, while the call runs, every millisecond
    by a watcher thread that sets the flag when it returns True.  The library mirrors the flag into
    the running kernels, which stop at their next work item."""

    def __init__(self, cancel: Optional[Callable[[], bool]]):
        self.flag = ctypes.c_int32(1 if (cancel is not None and cancel()) else 0)
        self._stop = threading.Event()
        self._thread = None
        if cancel is not None and not self.flag.value:
            def watch():
                while not self._stop.wait(0.001):
                    if cancel():
                        self.flag.value = 1
                        return
            self._thread = threading.Thread(target=watch, name="fg-cancel-watch", daemon=True)
            self._thread.start()

    @property
    def ptr(self):
        return ctypes.addressof(self.flag)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._thread is not None:
            self._thread.join()


def _render(fn_name: str, lam, params: Params, derived: Derived, cancel, offs: np.ndarray):
    h, w = derived.input_height, derived.input_width
    oh, ow = derived.output_height, derived.output_width
    fn = getattr(lib(), fn_name)
    if _is_torch_cuda(lam):
        import torch
        if lam.dtype != torch.float32 or not lam.is_contiguous() or lam.numel() != w * h:
            raise RenderError("lambda must be a contiguous float32 tensor of input_width*input_height", _FG_INVALID)
        out = torch.empty((oh, ow), dtype=torch.float32, device=lam.device)
        stream = torch.cuda.current_stream(lam.device).cuda_stream
        with _Cancel(cancel) as cflag:
            rc = fn(lam.data_ptr(), ctypes.byref(params.c), ctypes.byref(derived._c), offs.ctypes.data,
                    out.data_ptr(), cflag.ptr, stream)
        _raise(rc)
        return out
    src = np.ascontiguousarray(lam, np.float32)
    if src.size != w * h:
        raise RenderError("lambda plane size does not match the derived input size", _FG_INVALID)
    out = np.empty((oh, ow), np.float32)
    with _Cancel(cancel) as cflag:
        rc = fn(src.ctypes.data, ctypes.byref(params.c), ctypes.byref(derived._c), offs.ctypes.data, out.ctypes.data,
                cflag.ptr, None)
    _raise(rc)
    return out


def render_pixelwise(lam, params: Params, derived: Derived, cancel: Optional[Callable[[], bool]] = None):
    """render_pixelwise (src/pixelwise.rs:11-45).  lam: numpy (host) or torch CUDA tensor."""
    return _render("fg_render_pixelwise", lam, params, derived, cancel,
                   np.ascontiguousarray(derived.offsets_input, np.float32))


def render_grainwise(lam, params: Params, derived: Derived, cancel: Optional[Callable[[], bool]] = None):
    """render_grainwise (src/grainwise.rs:12-124).  lam: numpy (host) or torch CUDA tensor."""
    return _render("fg_render_grainwise", lam, params, derived, cancel,
                   np.ascontiguousarray(derived.offsets, np.float32))


def pixelwise_kernel_count(params: "Params", derived: "Derived") -> int:
    """Kernel launches one pixel-wise render of these params makes: 3 on the per-sample kernel, 6 on the
    sparse block pass (with the plane's emptiness bitmask and the sorted offsets), 4 on the lean block
    pass."""
    offs = np.ascontiguousarray(derived.offsets_input, np.float32)
    n = ctypes.c_int32()
    _raise(lib().fg_pixelwise_kernel_count(params.c, derived._c, offs.ctypes.data, ctypes.byref(n)))
    return n.value


def pixelwise_diagnostics() -> Tuple[int, int, int, int]:
    """(samples evaluated by per-sample regeneration, unstaged blocks, subdivisions, blocks) of this
    thread's last pixel-wise render."""
    arr = (ctypes.c_ulonglong * 4)()
    lib().fg_pixelwise_diagnostics(arr)
    return tuple(int(v) for v in arr)


def pixelwise_sparse_forms() -> Tuple[int, int]:
    """(sample-major, grain-major) blocks of the sparse block pass in this thread's last pixel-wise
    render: the two forms of its sample step, which give identical counts."""
    arr = (ctypes.c_ulonglong * 2)()
    lib().fg_pixelwise_sparse_forms(arr)
    return tuple(int(v) for v in arr)


def _output_size(rgb_shape, params: Params) -> Tuple[int, int]:
    h, w = rgb_shape[0], rgb_shape[1]
    st = _StatsC()
    _raise(lib().fg_dry_run(w, h, ctypes.byref(params.c), ctypes.byref(st)))
    return st.output_width, st.output_height


def render_with_input_image(rgb: np.ndarray, params: Params, cancel: Optional[Callable[[], bool]] = None):
    """render_with_input_image[_cancelable] (src/lib.rs:78-93): f32 RGB (H, W, 3) -> (u8 RGB, RenderStats)."""
    src = np.ascontiguousarray(rgb, np.float32)
    if src.ndim != 3 or src.shape[2] != 3:
        raise RenderError("expected an (H, W, 3) RGB array", _FG_INVALID)
    ow, oh = _output_size(src.shape, params)
    out = np.empty((oh, ow, 3), np.uint8)
    st = _StatsC()
    with _Cancel(cancel) as cflag:
        rc = lib().fg_render_image(src.ctypes.data, src.shape[1], src.shape[0], ctypes.byref(params.c),
                                   out.ctypes.data, ctypes.byref(st), cflag.ptr, None)
    _raise(rc)
    return out, _stats(st)


def dry_run_with_input_image(rgb_shape, params: Params) -> RenderStats:
    """dry_run_with_input_image (src/lib.rs:100-104) from the input's (H, W[, 3]) shape."""
    st = _StatsC()
    _raise(lib().fg_dry_run(rgb_shape[1], rgb_shape[0], ctypes.byref(params.c), ctypes.byref(st)))
    return _stats(st)


# ------------------------------------------------------------------ batches (no counterpart in the crate)
class Batch:
    """Many images (pixel-wise and grain-wise mixed, uneven sizes) rendered by one persistent launch
    behind a CUDA graph.  Each entry of ``images`` is (lam_cuda_tensor, params, derived, algo[, lam_host]);
    ``outputs`` receives one torch CUDA tensor per image, rewritten by every ``run()``."""

    def __init__(self, images, tuning: Optional[BatchTuning] = None):
        import torch
        self._keep = []
        arr = (_BatchImageC * len(images))()
        self.outputs = []
        for k, item in enumerate(images):
            lam, params, derived, algo = item[:4]
            host = item[4] if len(item) > 4 else None
            if not _is_torch_cuda(lam) or lam.dtype != torch.float32 or not lam.is_contiguous():
                raise RenderError("batch lambda planes must be contiguous float32 CUDA tensors", _FG_INVALID)
            out = torch.empty((derived.output_height, derived.output_width), dtype=torch.float32, device=lam.device)
            offs = np.ascontiguousarray(derived.offsets_input if Algo(algo) == Algo.Pixel else derived.offsets,
                                        np.float32)
            hl = None if host is None else np.ascontiguousarray(host, np.float32)
            self._keep += [lam, out, offs, hl, params, derived]
            arr[k].algo = int(algo)
            arr[k].params = ctypes.pointer(params.c)
            arr[k].derived = ctypes.pointer(derived._c)
            arr[k].offsets = offs.ctypes.data
            arr[k].d_lambda = lam.data_ptr()
            arr[k].d_out = out.data_ptr()
            arr[k].h_lambda = hl.ctypes.data if hl is not None else None
            self.outputs.append(out)
        self._arr = arr
        self._h = ctypes.c_void_p()
        _raise(lib().fg_batch_create(arr, len(images), ctypes.byref(tuning) if tuning is not None else None,
                                     ctypes.byref(self._h)))

    def run(self, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _raise(lib().fg_batch_run(self._h, st))

    @property
    def tuning(self) -> BatchTuning:
        t = BatchTuning()
        _raise(lib().fg_batch_get_tuning(self._h, ctypes.byref(t)))
        return t

    @property
    def kernel_count(self) -> int:
        """Kernel launches one run() makes (the kernel nodes of the captured graph)."""
        n = ctypes.c_int32()
        _raise(lib().fg_batch_kernel_count(self._h, ctypes.byref(n)))
        return n.value

    def close(self):
        if self._h:
            lib().fg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def autotune(images) -> Tuple[BatchTuning, float]:
        """Fastest tuning for these images (each candidate is built and timed on the GPU)."""
        import torch
        arr = (_BatchImageC * len(images))()
        keep = []
        for k, item in enumerate(images):
            lam, params, derived, algo = item[:4]
            host = item[4] if len(item) > 4 else None
            out = torch.empty((derived.output_height, derived.output_width), dtype=torch.float32, device=lam.device)
            offs = np.ascontiguousarray(derived.offsets_input if Algo(algo) == Algo.Pixel else derived.offsets,
                                        np.float32)
            hl = None if host is None else np.ascontiguousarray(host, np.float32)
            keep += [out, offs, hl]
            arr[k].algo = int(algo)
            arr[k].params = ctypes.pointer(params.c)
            arr[k].derived = ctypes.pointer(derived._c)
            arr[k].offsets = offs.ctypes.data
            arr[k].d_lambda = lam.data_ptr()
            arr[k].d_out = out.data_ptr()
            arr[k].h_lambda = hl.ctypes.data if hl is not None else None
        best = BatchTuning()
        ms = ctypes.c_float()
        _raise(lib().fg_batch_autotune(arr, len(images), torch.cuda.current_stream().cuda_stream, ctypes.byref(best),
                                       ctypes.byref(ms)))
        return best, ms.value
