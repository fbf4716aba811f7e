"""The surrogate: a residual 3x3-conv network that stands in for the MC integrators in interactive
previews.  No counterpart in the reference crate; the plain renders (render_pixelwise / render_grainwise)
stay the method of record, produce its training targets and score it.

Network (every conv 3x3, zero padding; weights bf16 on the tensor cores, f32 accumulation):
    x   = (u, N(0,1) noise, radius * radius_scale)          u = normalised intensity, radius in input px
    h0  = relu(conv_in(x) + b_in)                            3 (padded to 16) -> 32 channels
    h_l = h_{l-1} + relu(conv_l(h_{l-1}) + b_l)              32 -> 32, l = 1..n_res
    y   = u + conv_out(h_n)[0] + b_out[0]                    32 -> 1
Forward, backward and the Adam step run in the library's own kernels (include/film_grain_gb300.h,
fg_sg_*); this module owns the parameter buffers and sequences the launches.  Parameters live in one
flat f32 vector (the master copy Adam updates) mirrored by a flat bf16 vector the kernels read.

Grain.  A plain render is its expectation (u under the sample filter) plus the film grain of its grain
realisation (low frequencies: the coverage field seen through the Gaussian filter) plus the
integrator's Monte Carlo error (white, variance f(1 - f)/N per pixel).  The network renders a grain
realisation of its own from the noise input: it is trained on pairs of outputs for the same tile and
two noise fields, with a mean-square term that is blind to the noise part (the paired form
E(m - t)^2 - E d^2 / 2, m the pair's mean, d its half-difference / sqrt 2) and a spectral term that
matches the radial power of d to the grain power of the target (its residual against the expectation,
less the Monte Carlo floor).  A third pass with the noise channel's input weights zeroed is trained on
plain mean-square error, so that the same network with those weights zeroed predicts the expectation
instead (`grain=False`).
"""
from __future__ import annotations

import ctypes
import math
from typing import Dict, Optional, Tuple

import numpy as np

from . import (Algo, Batch, ParamsBuilder, RadiusDist, _SgNetC, _raise, derive_common, lambda_plane, lib,
               normalize_plane)

CONV_INPUT, CONV_RESIDUAL, CONV_OUTPUT, CONV_DGRAD_RESIDUAL, CONV_DGRAD_OUTPUT = range(5)
CH = 32          # residual stream channels
CH_IN = 16       # padded input channels (3 used)
CH_OUT = 8       # computed output channels (1 used)
N_INPUTS = 3
NOISE_CHANNEL = 1
GRAIN_FMAX = 0.75  # the spectral training term covers every radial bin of a tile (the corners reach 0.71)


def _layout(n_res: int):
    """Offsets (elements) of each tensor in the flat parameter vector; the weight blocks come first and
    every block is a multiple of 8 elements, so every weight tensor starts 16-byte aligned."""
    entries = [("w_in", (CH, 9, CH_IN)), ("w_res", (n_res, CH, 9, CH)), ("w_out", (CH_OUT, 9, CH)),
               ("b_in", (CH,)), ("b_res", (n_res, CH)), ("b_out", (CH_OUT,))]
    out, off = {}, 0
    for name, shape in entries:
        out[name] = (off, shape)
        off += int(np.prod(shape))
    return out, off


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


class SurrogateNet:
    """Parameters, Adam state and the training / inference launches of the surrogate."""

    def __init__(self, n_res: int = 8, radius_scale: float = 10.0, seed: int = 0, device: str = "cuda"):
        import torch
        self.n_res = int(n_res)
        self.radius_scale = float(radius_scale)
        self.device = torch.device(device)
        self.layout, self.n_params = _layout(self.n_res)
        self.step = 0
        w = np.zeros(self.n_params, np.float32)
        rng = np.random.default_rng(seed)
        v = self._np_view(w, "w_in")
        v[:, :, :N_INPUTS] = rng.normal(0.0, math.sqrt(2.0 / (9 * N_INPUTS)), (CH, 9, N_INPUTS))
        self._np_view(w, "w_res")[:] = rng.normal(0.0, 0.1 * math.sqrt(2.0 / (9 * CH)), (self.n_res, CH, 9, CH))
        self._np_view(w, "w_out")[0] = rng.normal(0.0, 1e-3, (9, CH))
        self.w32 = torch.from_numpy(w).to(self.device)
        self.wbf = self.w32.to(torch.bfloat16)
        self.m = torch.zeros_like(self.w32)
        self.v = torch.zeros_like(self.w32)
        self.grad = torch.zeros_like(self.w32)
        self.ema = self.w32.clone()  # exponential moving average of the weights (what inference ships)
        self.decay = torch.zeros_like(self.w32)  # decoupled weight decay per parameter (none)
        self._ws: Dict[Tuple[int, int, int], dict] = {}
        self._wt_res = torch.zeros(CH * 9 * CH, dtype=torch.bfloat16, device=self.device)
        self._wt_out = torch.zeros(CH * 9 * CH_IN, dtype=torch.bfloat16, device=self.device)

    # ------------------------------------------------------------------ views
    def _np_view(self, flat: np.ndarray, name: str) -> np.ndarray:
        off, shape = self.layout[name]
        return flat[off:off + int(np.prod(shape))].reshape(shape)

    def view(self, flat, name: str):
        off, shape = self.layout[name]
        return flat[off:off + int(np.prod(shape))].view(shape)

    def _ptr(self, flat, name: str, layer: int = 0) -> int:
        off, shape = self.layout[name]
        per = int(np.prod(shape[1:])) if name in ("w_res", "b_res") else 0
        return flat.data_ptr() + (off + layer * per) * flat.element_size()

    def net_struct(self) -> _SgNetC:
        n = _SgNetC()
        n.n_res = self.n_res
        n.radius_scale = self.radius_scale
        n.w_in, n.w_res, n.w_out = self._ptr(self.wbf, "w_in"), self._ptr(self.wbf, "w_res"), self._ptr(self.wbf, "w_out")
        n.b_in, n.b_res, n.b_out = self._ptr(self.w32, "b_in"), self._ptr(self.w32, "b_res"), self._ptr(self.w32, "b_out")
        return n

    def numpy_net(self) -> dict:
        """The network as numpy arrays: bf16-valued weights (as the kernels see them) and f32 biases."""
        wb = self.wbf.float().cpu().numpy()
        w32 = self.w32.cpu().numpy()
        return {k: (self._np_view(wb, k) if k.startswith("w_") else self._np_view(w32, k)).copy()
                for k in ("w_in", "w_res", "w_out", "b_in", "b_res", "b_out")}

    # ------------------------------------------------------------------ checkpoint / resume
    def state(self, optimizer: bool = True) -> dict:
        s = dict(w32=self.w32.cpu().numpy(), step=np.int64(self.step), n_res=np.int64(self.n_res),
                 radius_scale=np.float32(self.radius_scale))
        if optimizer:
            s.update(m=self.m.cpu().numpy(), v=self.v.cpu().numpy(), ema=self.ema.cpu().numpy())
        return s

    def save(self, path: str, optimizer: bool = True, **meta):
        """Checkpoint: f32 master weights, step and (optimizer=True) the Adam moments, so that training
        resumes exactly where it stopped; extra keyword arguments are stored as metadata."""
        np.savez(path, **self.state(optimizer), **{f"meta_{k}": np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path: str, device: str = "cuda") -> "SurrogateNet":
        import torch
        z = np.load(path)
        net = cls(int(z["n_res"]), float(z["radius_scale"]), device=device)
        net.w32.copy_(torch.from_numpy(z["w32"]))
        net.wbf.copy_(net.w32.to(torch.bfloat16))
        net.ema.copy_(net.w32)
        if "m" in z:
            net.m.copy_(torch.from_numpy(z["m"]))
            net.v.copy_(torch.from_numpy(z["v"]))
            net.ema.copy_(torch.from_numpy(z["ema"]))
        net.step = int(z["step"])
        net.meta = {k[5:]: z[k].item() if z[k].ndim == 0 else z[k] for k in z.files if k.startswith("meta_")}
        return net

    # ------------------------------------------------------------------ buffers
    def _workspace(self, nb: int, h: int, w: int, train: bool = True) -> dict:
        """Activation buffers for one batch shape.  Training keeps every layer's output and ReLU output
        for the backward pass; inference ping-pongs between two buffers."""
        import torch
        key = (nb, h, w, train)
        ws = self._ws.get(key)
        if ws is None:
            bf, dev = torch.bfloat16, self.device
            n_h = self.n_res + 1 if train else 2
            ws = dict(x=torch.empty((nb, h, w, CH_IN), dtype=bf, device=dev),
                      hs=[torch.empty((nb, h, w, CH), dtype=bf, device=dev) for _ in range(n_h)],
                      y=torch.empty((nb, h, w), dtype=torch.float32, device=dev))
            if train:
                ws.update(rs=[torch.empty((nb, h, w, CH), dtype=bf, device=dev) for _ in range(self.n_res)],
                          dy=torch.empty((nb, h, w, CH_IN), dtype=bf, device=dev),
                          dh=torch.empty((nb, h, w, CH), dtype=bf, device=dev),
                          dz=torch.empty((nb, h, w, CH), dtype=bf, device=dev),
                          loss=torch.zeros(1, dtype=torch.float32, device=dev))
            same_mode = [k for k in self._ws if k[3] == train]
            if len(same_mode) >= 2:  # two shapes per mode stay resident (grain training uses two)
                del self._ws[same_mode[0]]
            self._ws[key] = ws
        return ws

    # ------------------------------------------------------------------ launches
    def _conv(self, kind, inp, in_c, w_ptr, b_ptr, res, res_f32, out, aux, out_f32, nb, h, w):
        p = lambda t: None if t is None else t.data_ptr()
        _raise(lib().fg_sg_conv_forward(kind, p(inp), in_c, w_ptr, b_ptr, p(res), p(res_f32), p(out), p(aux),
                                        p(out_f32), nb, h, w, _stream()))

    def forward(self, u, radius, seed: int, keep: bool = False):
        """y [nb, h, w] f32 from u [nb, h, w] f32 and radius [nb] f32 (CUDA tensors).  keep=True stores
        every activation and ReLU output for the backward pass."""
        nb, h, w = u.shape
        ws = self._workspace(nb, h, w, train=keep)
        L = lib()
        _raise(L.fg_sg_make_input(u.data_ptr(), radius.data_ptr(), self.radius_scale, int(seed) & (2**64 - 1),
                                  ws["x"].data_ptr(), nb, h, w, _stream()))
        hs, rs = ws["hs"], ws.get("rs")
        self._conv(CONV_INPUT, ws["x"], CH_IN, self._ptr(self.wbf, "w_in"), self._ptr(self.w32, "b_in"), None, None,
                   hs[0], None, None, nb, h, w)
        for l in range(self.n_res):
            src, dst = (hs[l], hs[l + 1]) if keep else (hs[l % 2], hs[(l + 1) % 2])
            self._conv(CONV_RESIDUAL, src, CH, self._ptr(self.wbf, "w_res", l), self._ptr(self.w32, "b_res", l), src,
                       None, dst, rs[l] if keep else None, None, nb, h, w)
        last = hs[self.n_res] if keep else hs[self.n_res % 2]
        self._conv(CONV_OUTPUT, last, CH, self._ptr(self.wbf, "w_out"), self._ptr(self.w32, "b_out"), None, u, None,
                   None, ws["y"], nb, h, w)
        return ws["y"]

    def backward(self, u, target):
        """Gradients of mean((y - target)^2) into self.grad (zeroed first); uses the activations of the
        last forward(keep=True).  Returns the device loss-sum tensor (sum of squared errors)."""
        nb, h, w = u.shape
        ws = self._workspace(nb, h, w)
        n = nb * h * w
        ws["loss"].zero_()
        _raise(lib().fg_sg_mse_grad(ws["y"].data_ptr(), target.data_ptr(), ws["dy"].data_ptr(), ws["loss"].data_ptr(),
                                    n, 2.0 / n, _stream()))
        self._backward_layers(ws, nb, h, w)
        return ws["loss"]

    def backward_from(self, dy):
        """Gradients into self.grad (zeroed first) for a loss whose gradient with respect to the output
        of the last forward(keep=True) is dy [nb, h, w] f32."""
        import torch
        nb, h, w = dy.shape
        ws = self._workspace(nb, h, w)
        ws["dy"].zero_()
        ws["dy"][..., 0] = dy.to(torch.bfloat16)
        self._backward_layers(ws, nb, h, w)

    def _backward_layers(self, ws, nb, h, w):
        """The backward pass through every layer from the output gradient in ws["dy"]."""
        L, s = lib(), _stream()
        self.grad.zero_()
        g = self.grad
        hs, rs = ws["hs"], ws["rs"]
        _raise(L.fg_sg_conv_wgrad(CONV_OUTPUT, ws["dy"].data_ptr(), CH_IN, hs[self.n_res].data_ptr(), CH,
                                  self._ptr(g, "w_out"), self._ptr(g, "b_out"), nb, h, w, s))
        _raise(L.fg_sg_flip_weights(self._ptr(self.wbf, "w_out"), self._wt_out.data_ptr(), CH_OUT, CH, CH_IN, CH, s))
        dh, dz = ws["dh"], ws["dz"]
        self._conv(CONV_DGRAD_OUTPUT, ws["dy"], CH_IN, self._wt_out.data_ptr(), None, None, None, dh, None, None,
                   nb, h, w)
        for l in range(self.n_res - 1, -1, -1):
            _raise(L.fg_sg_mask_grad(dh.data_ptr(), rs[l].data_ptr(), dz.data_ptr(), dz.numel(), s))
            _raise(L.fg_sg_conv_wgrad(CONV_RESIDUAL, dz.data_ptr(), CH, hs[l].data_ptr(), CH,
                                      self._ptr(g, "w_res", l), self._ptr(g, "b_res", l), nb, h, w, s))
            _raise(L.fg_sg_flip_weights(self._ptr(self.wbf, "w_res", l), self._wt_res.data_ptr(), CH, CH, CH, CH, s))
            self._conv(CONV_DGRAD_RESIDUAL, dz, CH, self._wt_res.data_ptr(), None, dh, None, dh, None, None, nb, h, w)
        _raise(L.fg_sg_mask_grad(dh.data_ptr(), hs[0].data_ptr(), dz.data_ptr(), dz.numel(), s))
        _raise(L.fg_sg_conv_wgrad(CONV_INPUT, dz.data_ptr(), CH, ws["x"].data_ptr(), CH_IN, self._ptr(g, "w_in"),
                                  self._ptr(g, "b_in"), nb, h, w, s))

    def adam_step(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
                  ema_decay: float = 0.999):
        self.step += 1
        # the average's decay warms up as (1 + t) / (10 + t), so early weights fade out of it quickly
        d = min(ema_decay, (1.0 + self.step) / (10.0 + self.step))
        _raise(lib().fg_sg_adam(self.w32.data_ptr(), self.m.data_ptr(), self.v.data_ptr(), self.grad.data_ptr(),
                                self.decay.data_ptr(), self.wbf.data_ptr(), self.ema.data_ptr(), d, self.n_params, lr,
                                beta1, beta2, eps, self.step, _stream()))

    def train_step(self, u, radius, target, seed: int, lr: float = 1e-3, ema_decay: float = 0.999):
        """One Adam step on a batch under mean((y - target)^2); returns the device loss-sum tensor (read
        it only when needed)."""
        self.forward(u, radius, seed, keep=True)
        loss = self.backward(u, target)
        self.adam_step(lr, ema_decay=ema_decay)
        return loss

    def train_step_grain(self, u, radius, target, seed: int, n_target: int, lr: float = 1e-3,
                         ema_decay: float = 0.999, spec_weight: float = 0.01):
        """One Adam step of grain training on a batch of tiles (see the module docstring): the network runs
        on every tile twice, with two noise fields, and the loss is the paired mean-square term plus
        spec_weight x the spectral term: per tile and radial bin, the square difference between the pairs'
        noise-part power and the target's grain power (target renders at n_target samples), relative to
        the tile's mean square grain power plus Monte Carlo floor (plus a tenth of the batch mean) -- so
        power the network adds where the target has no grain (high frequencies) costs as much as power
        missing where it has it, and a small-radius tile weighs about as much as a large-radius one.  A
        third pass, with the noise channel's input weights zeroed, adds the plain mean-square error of
        that network (the expectation predictor; the zeroed weights get no gradient from it).
        Returns (paired MSE, spectral term) tensors."""
        import torch
        nb, h, w = u.shape
        # the expectation pass first: its gradients are kept while the pairs' pass reuses self.grad
        noise_w = self.view(self.wbf, "w_in")[:, :, NOISE_CHANNEL]
        kept = noise_w.clone()
        noise_w.zero_()
        self.forward(u, radius, seed ^ 0x5DEECE66D, keep=True)
        self.backward(u, target)
        noise_w.copy_(kept)
        self.view(self.grad, "w_in")[:, :, NOISE_CHANNEL] = 0.0
        g_mean = self.grad.clone()
        y = self.forward(torch.cat([u, u]), torch.cat([radius, radius]), seed, keep=True)
        yv = y.detach().requires_grad_(True)
        y1, y2 = yv[:nb], yv[nb:]
        mse = ((0.5 * (y1 + y2) - target) ** 2).mean() - 0.25 * ((y1 - y2) ** 2).mean()
        kmax = max(1, int(GRAIN_FMAX * min(h, w)))
        with torch.no_grad():
            pt = grain_power(target, u, n_target, kmax).float()
            floor = mc_floor(target, n_target).float()[:, None]
            # per tile, relative to its own grain power plus floor, so that small radii (whose grain
            # carries a hundredth of the power of the largest) count; a tenth of the batch's mean scale
            # is added, so that a flat black or white tile (no grain, no floor) cannot dominate
            tile = ((pt.abs() + floor) ** 2).mean(1, keepdim=True)
            scale = tile + 0.1 * tile.mean() + 1e-30
        pd = radial_power((y1 - y2) * (1.0 / math.sqrt(2.0)), kmax)
        spec = (((pd - pt) ** 2) / scale).mean()
        (mse + spec_weight * spec).backward()
        self.backward_from(yv.grad)
        self.grad.add_(g_mean)
        self.adam_step(lr, ema_decay=ema_decay)
        return mse.detach(), spec.detach()

    def use_ema(self):
        """Replace the weights by their moving average (done once training ends: the average of the
        last ~1/(1 - ema_decay) steps removes most of the step-to-step noise of training on MC targets)."""
        import torch
        self.w32.copy_(self.ema)
        self.wbf.copy_(self.w32.to(torch.bfloat16))

    def infer(self, u, radius, seed: int, out=None, grain: bool = True):
        """Whole-network forward through the single fg_sg_infer entry point; returns y [nb, h, w].
        grain=False zeroes the noise channel's input weights: the network then predicts the expected
        render instead of a grain realisation."""
        import torch
        nb, h, w = u.shape
        L = lib()
        if not grain:
            return self._mean_net().infer(u, radius, seed, out=out)
        need = L.fg_sg_infer_workspace_bytes(nb, h, w)
        if getattr(self, "_infer_ws", None) is None or self._infer_ws.numel() < need:
            self._infer_ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        if out is None:
            out = torch.empty((nb, h, w), dtype=torch.float32, device=self.device)
        net = self.net_struct()
        _raise(L.fg_sg_infer(ctypes.byref(net), u.data_ptr(), radius.data_ptr(), int(seed) & (2**64 - 1),
                             out.data_ptr(), nb, h, w, self._infer_ws.data_ptr(), self._infer_ws.numel(), _stream()))
        return out

    def _mean_net(self) -> "SurrogateNet":
        """A copy sharing nothing, with the noise channel's input weights zeroed (cached until the
        weights change step)."""
        import torch
        key = (self.step, float(self.wbf.float().sum()))
        if getattr(self, "_mean_key", None) != key:
            m = SurrogateNet(self.n_res, self.radius_scale, device=str(self.device))
            m.w32.copy_(self.w32)
            m.view(m.w32, "w_in")[:, :, NOISE_CHANNEL] = 0.0
            m.wbf.copy_(m.w32.to(torch.bfloat16))
            self._mean, self._mean_key = m, key
        return self._mean


# ---------------------------------------------------------------------- training data
def training_tiles(n: int, size: int = 64, seed: int = 0, radius_range=(0.03, 0.2)):
    """n luma tiles (blobs, ramps, step edges, smooth textures; half of them with fine uniform noise),
    normalised to [0, 1), and one grain radius per tile, uniform over radius_range.
    Returns (u [n, size, size] f32, radius [n] f32)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:size, 0:size].astype(np.float64) + 0.5
    tiles = np.empty((n, size, size), np.float32)
    for k in range(n):
        kind = rng.integers(0, 4)
        if kind == 0:
            v = np.full((size, size), rng.uniform(0.0, 0.4))
            for _ in range(rng.integers(1, 6)):
                s = rng.uniform(2.0, 24.0)
                cx, cy = rng.uniform(-8, size + 8, 2)
                v += rng.uniform(-0.4, 0.8) * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * s * s))
        elif kind == 1:
            a = rng.uniform(0, 2 * np.pi)
            lo, hi = rng.uniform(0, 1, 2)
            t = ((xx - size / 2) * np.cos(a) + (yy - size / 2) * np.sin(a)) / size + 0.5
            v = lo + (hi - lo) * np.clip(t * rng.uniform(0.5, 2.0), 0, 1)
        elif kind == 2:
            v = np.full((size, size), rng.uniform(0.0, 1.0))
            for _ in range(rng.integers(1, 4)):
                a = rng.uniform(0, 2 * np.pi)
                px, py = rng.uniform(0, size, 2)
                side = (xx - px) * np.cos(a) + (yy - py) * np.sin(a) > 0
                v += rng.uniform(-0.6, 0.6) * side
        else:
            cell = int(rng.choice([2, 4, 8, 16]))
            m = (size + cell - 1) // cell
            coarse = rng.uniform(0, 1, (m, m))
            v = np.kron(coarse, np.ones((cell, cell)))[:size, :size] * rng.uniform(0.3, 1.0) + rng.uniform(0, 0.3)
        if rng.uniform() < 0.5:
            v = v + rng.uniform(-1, 1, (size, size)) * rng.uniform(0.0, 0.08)
        tiles[k] = normalize_plane(np.clip(v, 0.0, 1.0).astype(np.float32))[0]
    radius = rng.uniform(radius_range[0], radius_range[1], n).astype(np.float32)
    return tiles, radius


def training_set(n: int, size: int = 64, seed: int = 0, radius_range=(0.03, 0.2), lognormal_frac: float = 0.5,
                 sd_frac: float = 0.4):
    """training_tiles, with a lognormal radius distribution (standard deviation sd_frac x the mean) on a
    share lognormal_frac of the tiles.  Returns (u [n, size, size], radius mean [n], radius standard
    deviation [n] (0: constant), the network's radius input [n] (grain_radius))."""
    u, radius = training_tiles(n, size, seed, radius_range)
    rng = np.random.default_rng(seed + 7)
    sd = np.where(rng.uniform(size=n) < lognormal_frac, sd_frac * radius, 0.0).astype(np.float32)
    net_radius = np.array([grain_radius(float(r), float(v), v > 0) for r, v in zip(radius, sd)], np.float32)
    return u, radius, sd, net_radius


def render_tiles(u_tiles: np.ndarray, radius: np.ndarray, n_samples: int = 256, seed: int = 0,
                 chunk: int = 1024, sigma_px: float = 0.8, radius_sd: Optional[np.ndarray] = None):
    """Plain pixel-wise renders (the method of record) of each tile at its own radius (lognormal where
    radius_sd is above 0, else constant), through batched graphs of `chunk` tiles; returns a CUDA tensor
    [n, h, w] f32."""
    import torch
    n, h, w = u_tiles.shape
    out = torch.empty((n, h, w), dtype=torch.float32, device="cuda")
    for c0 in range(0, n, chunk):
        items = []
        for k in range(c0, min(n, c0 + chunk)):
            sd = 0.0 if radius_sd is None else float(radius_sd[k])
            p = ParamsBuilder(radius_mean=float(radius[k]), radius_dist=RadiusDist.Lognorm if sd > 0 else RadiusDist.Const,
                              radius_stddev=sd, n_samples=n_samples, sigma_px=sigma_px, algo=Algo.Pixel,
                              seed=(seed * 1_000_003 + k) & (2**64 - 1)).build()
            d = derive_common(p, (w, h))
            lam = lambda_plane(u_tiles[k], d.inv_e_pi_r2)
            items.append((torch.from_numpy(lam).cuda(), p, d, Algo.Pixel, lam))
        b = Batch(items)
        b.run()
        torch.cuda.synchronize()
        for j, o in enumerate(b.outputs):
            out[c0 + j].copy_(o)
        b.close()
    return out


def train(net: SurrogateNet, u, radius, target, steps: int, batch: int = 256, lr: float = 1e-3, seed: int = 0,
          ema_decay: float = 0.999, log_every: int = 0, checkpoint: Optional[str] = None, checkpoint_every: int = 0,
          log=print, grain_n: Optional[int] = None, spec_weight: float = 0.01):
    """Adam training on (u, radius, target) CUDA tensors with a cosine learning-rate schedule from lr
    down to lr/100 and a moving average of the weights (ema_decay).  grain_n: the targets' sample count,
    for grain training (SurrogateNet.train_step_grain); None trains the plain mean-square objective.
    Resumes from net.step (a loaded checkpoint continues where it stopped).  Returns the list of logged
    (step, mean squared error) -- (step, paired MSE, spectral term) under grain training."""
    import torch
    n = u.shape[0]
    gen = torch.Generator(device="cpu")
    history = []
    for s in range(net.step, steps):
        gen.manual_seed(seed * 1_000_003 + s)
        idx = torch.randint(0, n, (batch,), generator=gen).to(u.device)
        ub, rb, tb = u.index_select(0, idx), radius.index_select(0, idx), target.index_select(0, idx)
        if s % 2 == 1:  # the integrators' statistics are isotropic: flip half the batches
            ub, tb = ub.flip(2).contiguous(), tb.flip(2).contiguous()
        step_lr = lr * (0.01 + 0.99 * 0.5 * (1.0 + math.cos(math.pi * s / max(1, steps))))
        if grain_n:
            mse, spec = net.train_step_grain(ub, rb, tb, seed=seed * 7919 + s, n_target=grain_n, lr=step_lr,
                                             ema_decay=ema_decay, spec_weight=spec_weight)
        else:
            loss = net.train_step(ub, rb, tb, seed=seed * 7919 + s, lr=step_lr, ema_decay=ema_decay)
        if log_every and ((s + 1) % log_every == 0 or s + 1 == steps):
            if grain_n:
                history.append((s + 1, float(mse), float(spec)))
                log(f"step {s + 1}: paired mse {float(mse):.3e}, spectral {float(spec):.3f}")
            else:
                history.append((s + 1, float(loss.item()) / tb.numel()))
                log(f"step {s + 1}: mse {history[-1][1]:.3e}")
        if checkpoint and checkpoint_every and (s + 1) % checkpoint_every == 0:
            net.save(checkpoint)
    return history


# ---------------------------------------------------------------------- evaluation
def raps(img):
    """Radially averaged power spectrum of (img - mean) for a [h, w] CUDA tensor: the mean FFT power
    over annuli of integer radius 1 .. min(h, w) // 2."""
    import torch
    a = img.double()
    a = a - a.mean()
    p = torch.fft.fft2(a).abs() ** 2
    h, w = a.shape
    fy = torch.fft.fftfreq(h, device=a.device, dtype=torch.float64) * h
    fx = torch.fft.fftfreq(w, device=a.device, dtype=torch.float64) * w
    r = torch.round(torch.sqrt(fy[:, None] ** 2 + fx[None, :] ** 2)).long().flatten()
    nb = min(h, w) // 2
    sums = torch.bincount(r, weights=p.flatten(), minlength=nb + 1)
    cnts = torch.bincount(r, minlength=nb + 1)
    return sums[1:nb + 1] / cnts[1:nb + 1].clamp(min=1)


def grain_radius(radius_mean: float, radius_stddev: float = 0.0, lognormal: bool = False) -> float:
    """The radius input for a radius distribution: the constant radius whose grains give the same grain
    power.  The low-frequency grain power of sparse grains is proportional to E[r^4] / E[r^2]; for a
    lognormal radius of mean m and standard deviation s (shape s2 = ln(1 + s^2 / m^2)) that is
    (m (1 + s^2 / m^2)^2.5)^2.  The network is trained on constant radii."""
    if not lognormal or radius_stddev <= 0.0:
        return float(radius_mean)
    return float(radius_mean * (1.0 + (radius_stddev / radius_mean) ** 2) ** 2.5)


def expected_render(u, sigma_px: float = 0.8):
    """The expectation of a plain zoom-1 render given u [nb, h, w]: each sample lands d pixels from its
    pixel with probability Phi((d + 1/2) / sigma) - Phi((d - 1/2) / sigma) per axis (Gaussian offsets of
    the filter's sigma), where the grains cover the fraction u; edge pixels extend outwards, as the
    renderer clamps its lambda lookups to the plane."""
    import torch
    import torch.nn.functional as F
    r = int(math.ceil(4.0 * sigma_px))
    d = torch.arange(-r, r + 1, dtype=torch.float64)
    cdf = lambda z: 0.5 * (1.0 + torch.erf(z / math.sqrt(2.0)))
    k = cdf((d + 0.5) / sigma_px) - cdf((d - 0.5) / sigma_px)
    k = (k / k.sum()).to(device=u.device, dtype=u.dtype)
    x = F.pad(u[:, None], (r, r, r, r), mode="replicate")
    x = F.conv2d(F.conv2d(x, k.view(1, 1, 1, -1)), k.view(1, 1, -1, 1))
    return x[:, 0]


_BINS: Dict[Tuple[int, int, int, str], object] = {}


def radial_power(x, kmax: int):
    """Radial power spectrum per image of x [nb, h, w]: the mean |FFT|^2 of (x - its mean) over the annuli
    of integer radius 1 .. kmax (radius k = k / size cycles per pixel on a square image).  Returns
    [nb, kmax]; differentiable (a binning matrix for tiles up to 256^2, bin sums beyond)."""
    import torch
    nb, h, w = x.shape
    a = x - x.mean(dim=(1, 2), keepdim=True)
    f = torch.fft.fft2(a)
    p = (f.real ** 2 + f.imag ** 2).reshape(nb, h * w)
    key = (h, w, kmax, str(x.device))
    m = _BINS.get(key)
    if m is None:
        fy = torch.fft.fftfreq(h, device=x.device, dtype=torch.float64) * h
        fx = torch.fft.fftfreq(w, device=x.device, dtype=torch.float64) * w
        r = torch.round(torch.sqrt(fy[:, None] ** 2 + fx[None, :] ** 2)).long().flatten()
        if h * w <= 256 * 256:
            sel = (r >= 1) & (r <= kmax)
            m = torch.zeros(h * w, kmax, dtype=torch.float64, device=x.device)
            m[torch.nonzero(sel).flatten(), r[sel] - 1] = 1.0
            m = m / m.sum(0).clamp(min=1.0)
        else:
            m = r
        _BINS[key] = m
    if m.dim() == 2:
        return p @ m.to(p.dtype)
    out = torch.zeros(nb, kmax, dtype=torch.float64, device=x.device)
    sel = (m >= 1) & (m <= kmax)
    cnt = torch.bincount(m[sel] - 1, minlength=kmax).clamp(min=1)
    for b in range(nb):
        out[b] = torch.bincount(m[sel] - 1, weights=p[b][sel].double(), minlength=kmax) / cnt
    return out


def mc_floor(img, n_samples: int):
    """Per image: the radial power of a plain render's Monte Carlo error, white with variance f (1 - f) / N
    per pixel (f the render itself), in radial_power's units (h w times the variance)."""
    h, w = img.shape[-2:]
    return h * w * (img * (1.0 - img)).double().mean(dim=(1, 2)) / float(n_samples)


def grain_power(img, u, n_samples: Optional[int], kmax: int):
    """Radial power of the grain of a render img [nb, h, w] of intensities u: the spectrum of its residual
    against the expectation (expected_render), less the Monte Carlo floor of a plain render at n_samples
    (None for a render without Monte Carlo error: a prediction)."""
    p = radial_power(img - expected_render(u), kmax)
    if n_samples:
        p = p - mc_floor(img, n_samples).to(p.dtype)[:, None]
    return p


def grain_band_error(pred, ref, u, n_pred: Optional[int], n_ref: Optional[int], fmax: float = 0.25,
                     fmin: float = 1.0 / 64.0) -> float:
    """||G_pred - G_ref||_2 / ||G_ref||_2 over the radial bins from fmin to fmax cycles/px, G the grain
    power (grain_power) averaged over the images: how far pred's grain is from ref's in spectrum.  A
    prediction without grain (u itself, the expectation) scores about 1.  The band starts at wavelengths
    of 64 px: below that, on large frames, the image content's own spectrum is so strong that any
    departure from the expectation's exact level outweighs the grain."""
    if pred.dim() == 2:
        pred, ref, u = pred[None], ref[None], u[None]
    size = min(pred.shape[-2:])
    kmax = max(1, int(fmax * size))
    k0 = min(kmax, max(1, int(math.ceil(fmin * size))))
    gp = grain_power(pred, u, n_pred, kmax).double().mean(0)[k0 - 1:]
    gr = grain_power(ref, u, n_ref, kmax).double().mean(0)[k0 - 1:]
    return float(torch_norm(gp - gr) / torch_norm(gr))


def raps_error(pred, ref) -> float:
    """||P_pred - P_ref||_2 / ||P_ref||_2 over the radial bins of one plane."""
    pp, pr = raps(pred), raps(ref)
    return float(torch_norm(pp - pr) / torch_norm(pr))


def torch_norm(t):
    return t.pow(2).sum().sqrt()


def evaluate(pred, ref) -> dict:
    """MAE over all pixels and planes, and the spectrum error per plane (max and mean), of pred against
    ref ([planes, h, w] or [h, w] CUDA tensors)."""
    if pred.dim() == 2:
        pred, ref = pred[None], ref[None]
    mae = float((pred - ref).abs().mean())
    errs = [raps_error(pred[c], ref[c]) for c in range(pred.shape[0])]
    return dict(mae=mae, raps_max=max(errs), raps_mean=float(np.mean(errs)))


# ---------------------------------------------------------------------- shipped network and CLI
import os as _os

DEFAULT_WEIGHTS = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "weights", "surrogate_c4.npz")


def load_default(device: str = "cuda") -> SurrogateNet:
    """The shipped network: trained by ``python -m film_grain_gb300.surrogate train`` on 20,000 64x64
    luma tiles rendered by the plain pixel-wise method at N=256 (radius mean U[0.03, 0.2], constant on
    half the tiles and lognormal with standard deviation 0.4 x the mean on the others; sigma 0.8)."""
    if not _os.path.exists(DEFAULT_WEIGHTS):
        raise FileNotFoundError(f"surrogate weights missing: {DEFAULT_WEIGHTS}")
    return SurrogateNet.load(DEFAULT_WEIGHTS, device=device)


def train_from_scratch(tiles: int = 20000, tile_size: int = 64, n_samples: int = 256, steps: int = 4000,
                       batch: int = 256, lr: float = 1e-3, seed: int = 0, n_res: int = 8,
                       checkpoint: Optional[str] = None, checkpoint_every: int = 500, resume: bool = False,
                       log=print, grain: bool = True, spec_weight: float = 0.01) -> Tuple[SurrogateNet, dict]:
    """Render the training tiles with the plain method and train a network on them (resuming from
    `checkpoint` when resume=True and it exists): grain training (train_step_grain) unless grain=False,
    which trains the expectation alone.  Returns (net, info)."""
    import time
    import torch
    t0 = time.time()
    u, r, sd, r_net = training_set(tiles, tile_size, seed=seed + 1)
    t1 = time.time()
    target = render_tiles(u, r, n_samples=n_samples, seed=seed + 1, radius_sd=sd)
    torch.cuda.synchronize()
    t2 = time.time()
    log(f"tiles: {tiles} x {tile_size}^2 generated in {t1 - t0:.1f} s, rendered at N={n_samples} in {t2 - t1:.1f} s")
    if resume and checkpoint and _os.path.exists(checkpoint):
        net = SurrogateNet.load(checkpoint)
        log(f"resumed from {checkpoint} at step {net.step}")
    else:
        net = SurrogateNet(n_res=n_res, seed=seed)
    ut, rt = torch.from_numpy(u).cuda(), torch.from_numpy(r_net).cuda()
    hist = train(net, ut, rt, target, steps=steps, batch=batch, lr=lr, seed=seed, log_every=max(1, steps // 10),
                 checkpoint=checkpoint, checkpoint_every=checkpoint_every, log=log,
                 grain_n=n_samples if grain else None, spec_weight=spec_weight)
    net.use_ema()
    torch.cuda.synchronize()
    t3 = time.time()
    info = dict(tiles=tiles, tile_size=tile_size, n_samples=n_samples, steps=steps, batch=batch, lr=lr, seed=seed,
                render_s=t2 - t1, train_s=t3 - t2, final_mse=hist[-1][1] if hist else float("nan"),
                objective="grain (paired MSE + spectral)" if grain else "MSE", spec_weight=spec_weight if grain else 0.0,
                final_spectral=hist[-1][2] if hist and grain else float("nan"))
    log(f"trained {steps} steps (batch {batch}) in {t3 - t2:.1f} s")
    return net, info


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(prog="python -m film_grain_gb300.surrogate")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train", help="render training tiles with the plain method and train the network")
    t.add_argument("--tiles", type=int, default=20000)
    t.add_argument("--tile-size", type=int, default=64)
    t.add_argument("--n-samples", type=int, default=256)
    t.add_argument("--steps", type=int, default=4000)
    t.add_argument("--batch", type=int, default=256)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--n-res", type=int, default=8)
    t.add_argument("--out", default=DEFAULT_WEIGHTS, help="weights file (no optimizer state)")
    t.add_argument("--checkpoint", default=None, help="checkpoint with Adam moments, written every --checkpoint-every")
    t.add_argument("--checkpoint-every", type=int, default=500)
    t.add_argument("--resume", action="store_true", help="continue from --checkpoint")
    t.add_argument("--mean-only", action="store_true", help="train the expectation alone (no grain)")
    t.add_argument("--spec-weight", type=float, default=0.01, help="weight of the spectral term of grain training")
    a = ap.parse_args(argv)
    from .build import build
    build()
    net, info = train_from_scratch(a.tiles, a.tile_size, a.n_samples, a.steps, a.batch, a.lr, a.seed, a.n_res,
                                   a.checkpoint, a.checkpoint_every, a.resume, grain=not a.mean_only,
                                   spec_weight=a.spec_weight)
    _os.makedirs(_os.path.dirname(_os.path.abspath(a.out)), exist_ok=True)
    net.save(a.out, optimizer=False, **info)
    print(f"wrote {a.out}")


if __name__ == "__main__":
    main()
