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
NOISE_WEIGHT_DECAY = 100.0  # per-step shrink 1 - lr * 100 of the noise channel's input weights


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
        # Decoupled weight decay per parameter: only the noise channel's input weights.  Under the MSE
        # objective the optimal output does not depend on the noise, but Adam turns their zero-mean
        # gradients into a random walk of step ~lr; the decay holds them near zero.
        dec = np.zeros(self.n_params, np.float32)
        self._np_view(dec, "w_in")[:, :, 1] = NOISE_WEIGHT_DECAY
        self.decay = torch.from_numpy(dec).to(self.device)
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
            self._ws = {k: v for k, v in self._ws.items() if k[3] != train}  # one shape per mode stays resident
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
        L, s = lib(), _stream()
        n = nb * h * w
        self.grad.zero_()
        ws["loss"].zero_()
        g = self.grad
        _raise(L.fg_sg_mse_grad(ws["y"].data_ptr(), target.data_ptr(), ws["dy"].data_ptr(), ws["loss"].data_ptr(), n,
                                2.0 / n, s))
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
        return ws["loss"]

    def adam_step(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
                  ema_decay: float = 0.999):
        self.step += 1
        # the average's decay warms up as (1 + t) / (10 + t), so early weights fade out of it quickly
        d = min(ema_decay, (1.0 + self.step) / (10.0 + self.step))
        _raise(lib().fg_sg_adam(self.w32.data_ptr(), self.m.data_ptr(), self.v.data_ptr(), self.grad.data_ptr(),
                                self.decay.data_ptr(), self.wbf.data_ptr(), self.ema.data_ptr(), d, self.n_params, lr,
                                beta1, beta2, eps, self.step, _stream()))

    def train_step(self, u, radius, target, seed: int, lr: float = 1e-3, ema_decay: float = 0.999):
        """One Adam step on a batch; returns the device loss-sum tensor (read it only when needed)."""
        self.forward(u, radius, seed, keep=True)
        loss = self.backward(u, target)
        self.adam_step(lr, ema_decay=ema_decay)
        return loss

    def use_ema(self):
        """Replace the weights by their moving average (done once training ends: the average of the
        last ~1/(1 - ema_decay) steps removes most of the step-to-step noise of training on MC targets)."""
        import torch
        self.w32.copy_(self.ema)
        self.wbf.copy_(self.w32.to(torch.bfloat16))

    def infer(self, u, radius, seed: int, out=None):
        """Whole-network forward through the single fg_sg_infer entry point; returns y [nb, h, w]."""
        import torch
        nb, h, w = u.shape
        L = lib()
        need = L.fg_sg_infer_workspace_bytes(nb, h, w)
        if getattr(self, "_infer_ws", None) is None or self._infer_ws.numel() < need:
            self._infer_ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        if out is None:
            out = torch.empty((nb, h, w), dtype=torch.float32, device=self.device)
        net = self.net_struct()
        _raise(L.fg_sg_infer(ctypes.byref(net), u.data_ptr(), radius.data_ptr(), int(seed) & (2**64 - 1),
                             out.data_ptr(), nb, h, w, self._infer_ws.data_ptr(), self._infer_ws.numel(), _stream()))
        return out


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


def render_tiles(u_tiles: np.ndarray, radius: np.ndarray, n_samples: int = 256, seed: int = 0,
                 chunk: int = 1024, sigma_px: float = 0.8):
    """Plain pixel-wise renders (the method of record) of each tile at its own radius, through batched
    graphs of `chunk` tiles; returns a CUDA tensor [n, h, w] f32."""
    import torch
    n, h, w = u_tiles.shape
    out = torch.empty((n, h, w), dtype=torch.float32, device="cuda")
    for c0 in range(0, n, chunk):
        items = []
        for k in range(c0, min(n, c0 + chunk)):
            p = ParamsBuilder(radius_mean=float(radius[k]), radius_dist=RadiusDist.Const, n_samples=n_samples,
                              sigma_px=sigma_px, algo=Algo.Pixel, seed=(seed * 1_000_003 + k) & (2**64 - 1)).build()
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
          log=print):
    """Adam training on (u, radius, target) CUDA tensors with a cosine learning-rate schedule from lr
    down to lr/100 and a moving average of the weights (ema_decay).  Resumes from net.step (a loaded
    checkpoint continues where it stopped).  Returns the list of (step, mean squared error) logged."""
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
        loss = net.train_step(ub, rb, tb, seed=seed * 7919 + s, lr=step_lr, ema_decay=ema_decay)
        if log_every and ((s + 1) % log_every == 0 or s + 1 == steps):
            mse = float(loss.item()) / tb.numel()
            history.append((s + 1, mse))
            log(f"step {s + 1}: mse {mse:.3e}")
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
    luma tiles rendered by the plain pixel-wise method at N=256 (radius U[0.03, 0.2], sigma 0.8)."""
    if not _os.path.exists(DEFAULT_WEIGHTS):
        raise FileNotFoundError(f"surrogate weights missing: {DEFAULT_WEIGHTS}")
    return SurrogateNet.load(DEFAULT_WEIGHTS, device=device)


def train_from_scratch(tiles: int = 20000, tile_size: int = 64, n_samples: int = 256, steps: int = 8000,
                       batch: int = 256, lr: float = 1e-3, seed: int = 0, n_res: int = 8,
                       checkpoint: Optional[str] = None, checkpoint_every: int = 500, resume: bool = False,
                       log=print) -> Tuple[SurrogateNet, dict]:
    """Render the training tiles with the plain method and train a network on them (resuming from
    `checkpoint` when resume=True and it exists).  Returns (net, info)."""
    import time
    import torch
    t0 = time.time()
    u, r = training_tiles(tiles, tile_size, seed=seed + 1)
    t1 = time.time()
    target = render_tiles(u, r, n_samples=n_samples, seed=seed + 1)
    torch.cuda.synchronize()
    t2 = time.time()
    log(f"tiles: {tiles} x {tile_size}^2 generated in {t1 - t0:.1f} s, rendered at N={n_samples} in {t2 - t1:.1f} s")
    if resume and checkpoint and _os.path.exists(checkpoint):
        net = SurrogateNet.load(checkpoint)
        log(f"resumed from {checkpoint} at step {net.step}")
    else:
        net = SurrogateNet(n_res=n_res, seed=seed)
    ut, rt = torch.from_numpy(u).cuda(), torch.from_numpy(r).cuda()
    hist = train(net, ut, rt, target, steps=steps, batch=batch, lr=lr, seed=seed, log_every=max(1, steps // 10),
                 checkpoint=checkpoint, checkpoint_every=checkpoint_every, log=log)
    net.use_ema()
    torch.cuda.synchronize()
    t3 = time.time()
    info = dict(tiles=tiles, tile_size=tile_size, n_samples=n_samples, steps=steps, batch=batch, lr=lr, seed=seed,
                render_s=t2 - t1, train_s=t3 - t2, final_mse=hist[-1][1] if hist else float("nan"))
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
    t.add_argument("--steps", type=int, default=8000)
    t.add_argument("--batch", type=int, default=256)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--n-res", type=int, default=8)
    t.add_argument("--out", default=DEFAULT_WEIGHTS, help="weights file (no optimizer state)")
    t.add_argument("--checkpoint", default=None, help="checkpoint with Adam moments, written every --checkpoint-every")
    t.add_argument("--checkpoint-every", type=int, default=500)
    t.add_argument("--resume", action="store_true", help="continue from --checkpoint")
    a = ap.parse_args(argv)
    from .build import build
    build()
    net, info = train_from_scratch(a.tiles, a.tile_size, a.n_samples, a.steps, a.batch, a.lr, a.seed, a.n_res,
                                   a.checkpoint, a.checkpoint_every, a.resume)
    _os.makedirs(_os.path.dirname(_os.path.abspath(a.out)), exist_ok=True)
    net.save(a.out, optimizer=False, **info)
    print(f"wrote {a.out}")


if __name__ == "__main__":
    main()
