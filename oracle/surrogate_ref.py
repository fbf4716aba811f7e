"""CPU oracle for the surrogate network -- TEST INFRASTRUCTURE ONLY.

The surrogate (a residual 3x3-conv network standing in for the MC integrators) has no counterpart in
the reference crate, so this module is its checker: a numpy restatement of the network's forward pass,
its mean-squared-error loss and its backward pass.  Only ``tests/`` may import it.

Layout matches the device path: activations NHWC, weights [cout][9 taps][cin] with tap = 3*ky + kx,
zero padding.  With ``bf16=True`` every tensor the device stores in bf16 is rounded to bf16
(round-to-nearest-even) at the same point, and every sum is accumulated in f32; with ``bf16=False``
the same functions run in f64 without rounding (used for the finite-difference check of the
backward pass itself).  The data gradient is computed by col2im (scatter of the column gradient),
not by the flipped-weight convolution the device uses, so the two paths are independent.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round f32 values to the nearest bf16 (ties to even), returned as f32."""
    a = np.ascontiguousarray(a, np.float32)
    bits = a.view(np.uint32).astype(np.uint64)
    bits = (bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000
    return bits.astype(np.uint32).view(np.float32).reshape(a.shape)


def _cols(x: np.ndarray) -> np.ndarray:
    """im2col of a 3x3 zero-padded conv: (n, h, w, c) -> (n, h, w, 9, c), tap = 3*ky + kx."""
    n, h, w, c = x.shape
    xp = np.zeros((n, h + 2, w + 2, c), x.dtype)
    xp[:, 1:-1, 1:-1] = x
    return np.stack([xp[:, ky:ky + h, kx:kx + w] for ky in range(3) for kx in range(3)], axis=3)


def conv(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    """z[n, y, x, co] = sum_{tap, ci} w[co, tap, ci] * x[n, y + ky - 1, x + kx - 1, ci]."""
    n, h, wd, c = x.shape
    cols = _cols(x).reshape(n * h * wd, 9 * c)
    return (cols @ w.reshape(w.shape[0], 9 * c).T).reshape(n, h, wd, w.shape[0])


def conv_wgrad(g: np.ndarray, x: np.ndarray) -> np.ndarray:
    """dW[co, tap, ci] = sum_p g[p, co] * x[p + shift(tap), ci]."""
    n, h, wd, c = x.shape
    cols = _cols(x).reshape(n * h * wd, 9 * c)
    return (g.reshape(-1, g.shape[-1]).T @ cols).reshape(g.shape[-1], 9, c)


def conv_dgrad(g: np.ndarray, w: np.ndarray) -> np.ndarray:
    """dx of z = conv(x, w) given dz = g, by col2im."""
    n, h, wd, co = g.shape
    c = w.shape[2]
    dcols = (g.reshape(-1, co) @ w.reshape(co, 9 * c)).reshape(n, h, wd, 9, c)
    dxp = np.zeros((n, h + 2, wd + 2, c), dcols.dtype)
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        dxp[:, ky:ky + h, kx:kx + wd] += dcols[:, :, :, tap]
    return dxp[:, 1:-1, 1:-1]


def forward(x, u, net, bf16: bool = True):
    """x (n, h, w, 16) network input, u (n, h, w) intensity; net: dict w_in, b_in, w_res, b_res, w_out, b_out.
    Returns (y, cache)."""
    dt = np.float32 if bf16 else np.float64
    rnd = bf16_round if bf16 else (lambda a: a)
    x = np.asarray(x, dt)
    h = rnd(np.maximum(conv(x, np.asarray(net["w_in"], dt)) + np.asarray(net["b_in"], dt), 0))
    hs, rs = [h], []
    for l in range(len(net["w_res"])):
        r = np.maximum(conv(h, np.asarray(net["w_res"][l], dt)) + np.asarray(net["b_res"][l], dt), 0)
        rs.append(rnd(r))
        h = rnd(h + r)
        hs.append(h)
    z = conv(h, np.asarray(net["w_out"], dt))
    y = np.asarray(u, dt) + z[..., 0] + dt(net["b_out"][0])
    return y, dict(x=x, hs=hs, rs=rs)


def backward(y, t, cache, net, bf16: bool = True):
    """Gradients of loss = mean((y - t)^2) for every parameter; returns (loss, grads dict)."""
    dt = np.float32 if bf16 else np.float64
    rnd = bf16_round if bf16 else (lambda a: a)
    n = y.size
    e = np.asarray(y, dt) - np.asarray(t, dt)
    loss = float(np.sum(e.astype(np.float64) ** 2) / n)
    co_out = net["w_out"].shape[0]
    dy = np.zeros(y.shape + (co_out,), dt)
    dy[..., 0] = rnd((dt(2.0 / n) * e).astype(dt))
    hs, rs, x = cache["hs"], cache["rs"], cache["x"]
    grads = {}
    grads["w_out"] = conv_wgrad(dy, hs[-1])
    grads["b_out"] = dy.reshape(-1, co_out).sum(0)
    dh = rnd(conv_dgrad(dy, np.asarray(net["w_out"], dt)))
    L = len(net["w_res"])
    gw, gb = [None] * L, [None] * L
    for l in range(L - 1, -1, -1):
        dz = np.where(rs[l] > 0, dh, 0).astype(dt)
        gw[l] = conv_wgrad(dz, hs[l])
        gb[l] = dz.reshape(-1, dz.shape[-1]).sum(0)
        dh = rnd(dh + conv_dgrad(dz, np.asarray(net["w_res"][l], dt)))
    dz0 = np.where(hs[0] > 0, dh, 0).astype(dt)
    grads["w_in"] = conv_wgrad(dz0, x)
    grads["b_in"] = dz0.reshape(-1, dz0.shape[-1]).sum(0)
    grads["w_res"] = np.stack(gw) if L else np.zeros((0,) + tuple(net["w_res"].shape[1:]), dt)
    grads["b_res"] = np.stack(gb) if L else np.zeros((0, 32), dt)
    return loss, grads


def adam(w, m, v, g, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, decay=0.0):
    """One Adam step (Kingma & Ba 2015) with bias correction and decoupled weight decay (AdamW,
    Loshchilov & Hutter 2019): w -= lr * (m_hat / (sqrt(v_hat) + eps) + decay * w); returns (w, m, v)."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return w - lr * (mh / (np.sqrt(vh) + eps) + decay * w), m, v


def raps(img: np.ndarray) -> np.ndarray:
    """Radially averaged power spectrum of (img - mean): mean FFT power over annuli of integer radius
    1 .. min(h, w) // 2 (the surrogate's spectrum metric)."""
    a = np.asarray(img, np.float64)
    a = a - a.mean()
    p = np.abs(np.fft.fft2(a)) ** 2
    h, w = a.shape
    fy = np.fft.fftfreq(h) * h
    fx = np.fft.fftfreq(w) * w
    r = np.rint(np.sqrt(fy[:, None] ** 2 + fx[None, :] ** 2)).astype(np.int64)
    nb = min(h, w) // 2
    sums = np.bincount(r.ravel(), weights=p.ravel(), minlength=nb + 1)
    cnts = np.bincount(r.ravel(), minlength=nb + 1)
    return sums[1:nb + 1] / np.maximum(cnts[1:nb + 1], 1)
