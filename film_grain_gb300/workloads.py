"""Seeded synthetic inputs with the shapes and value distributions of the benchmark workloads.

No image dataset is involved: each workload is generated from its seed.
- ramp_noise: horizontal linear ramp 0 -> 1 plus uniform noise +-0.05, clamped to [0, 1]
  (the 256 x 256 luma pixel-wise workload).
- blobs: isotropic Gaussian blobs (amplitude U[0.2, 0.9], sigma U[30, 150] px) over a 0.1 background,
  clamped to [0, 1], each channel seeded independently (the 1024^2 x 3 grain-wise workload and the
  4096^2 x 3 large-frame workload).  `scale` shrinks the blobs for small test planes: sixteen blobs of
  30-150 px on a plane of a few hundred pixels or less add up to a saturated plane, while sigma x
  max(w, h) / 1536 keeps about half of it near the background and a few percent saturated.
"""
from __future__ import annotations

import numpy as np


def ramp_noise(width: int = 256, height: int = 256, seed: int = 42) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ramp = np.linspace(0.0, 1.0, width, dtype=np.float64)[None, :].repeat(height, 0)
    v = ramp + rng.uniform(-0.05, 0.05, size=(height, width))
    return np.clip(v, 0.0, 1.0).astype(np.float32)


def blobs_plane(width: int, height: int, seed: int, n_blobs: int = 16, background: float = 0.1,
                scale: float = 1.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.2, 0.9, n_blobs)
    sig = rng.uniform(30.0, 150.0, n_blobs) * scale
    cx = rng.uniform(0, width, n_blobs)
    cy = rng.uniform(0, height, n_blobs)
    xs = np.arange(width, dtype=np.float64) + 0.5
    ys = np.arange(height, dtype=np.float64) + 0.5
    v = np.full((height, width), background, np.float64)
    for a, s, x0, y0 in zip(amp, sig, cx, cy):
        gx = np.exp(-((xs - x0) ** 2) / (2 * s * s))
        gy = np.exp(-((ys - y0) ** 2) / (2 * s * s))
        v += a * gy[:, None] * gx[None, :]
    return np.clip(v, 0.0, 1.0).astype(np.float32)


def blobs_rgb(width: int, height: int, seed: int, scale: float = 1.0) -> np.ndarray:
    """(H, W, 3) f32 RGB, each channel an independently seeded blob plane."""
    return np.stack([blobs_plane(width, height, seed * 3 + c, scale=scale) for c in range(3)], axis=-1)


def small_scale(width: int, height: int) -> float:
    """The blob scale of a small test plane (blobs_plane's `scale`)."""
    return max(width, height) / 1536.0


def gray_rgb(plane: np.ndarray) -> np.ndarray:
    return np.repeat(plane[:, :, None], 3, axis=2).astype(np.float32)


def batched_sweep(n_images: int = 64, seed: int = 7, sizes=(128, 256, 512, 1024, 2048),
                  radii=(0.025, 0.05, 0.1, 0.2), samples=(16, 64, 256)):
    """The uneven batch: n luma images of the blob family, each with a seeded size (square, uniform over
    `sizes`), constant grain radius (uniform over `radii`), N (uniform over `samples`) and image seed.
    Returns a list of dicts (size, radius, n, seed, image_seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_images):
        out.append(dict(size=int(rng.choice(sizes)), radius=float(rng.choice(radii)), n=int(rng.choice(samples)),
                        seed=int(rng.integers(0, 2**32)), image_seed=1000 + k))
    return out
