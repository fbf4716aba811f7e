"""The lambda prelude on the device against the host (the crate's normalize_plane / lambda_plane,
src/model.rs:228-265, with the platform logf that f32::ln calls).

lambda_plane takes the logarithm of max(1 - c, 1e-6) with c clamped to [0, 1 - 1e-6]; 1 - c is a
multiple of 2^-24 in f32, so every input the logarithm can see is k * 2^-24 (17 <= k <= 2^24) or
1e-6.  The first test feeds c = 1 - k * 2^-24 for every k (and NaN, negative and > 1 values), so
the device's logarithm is checked on its whole reachable domain, bit for bit.
"""
import ctypes

import numpy as np
import pytest

from film_grain_gb300 import workloads

pytestmark = pytest.mark.gpu


def _host_and_device(fgl, torch, fn, src, *args):
    L = fgl.lib()
    host = np.empty_like(src)
    rh = getattr(L, fn)(src.ctypes.data, src.size, *args, host.ctypes.data)
    d_src = torch.from_numpy(src).cuda()
    d_out = torch.empty_like(d_src)
    rd = getattr(L, fn)(d_src.data_ptr(), src.size, *args, d_out.data_ptr())
    torch.cuda.synchronize()
    return host, d_out.cpu().numpy(), rh, rd


def test_device_lambda_every_reachable_input(cuda, fgl):
    torch = cuda
    k = np.arange(1, (1 << 24) + 1, dtype=np.float64)
    c = (1.0 - k * 2.0 ** -24).astype(np.float32)                 # exact: safe = k * 2^-24
    extra = np.array([np.nan, -1.0, -0.0, 0.0, 2.0, 1.0, 0.9999995, 1e-30, np.inf, -np.inf], np.float32)
    src = np.concatenate([c, extra])
    for inv in (0.5, 13.28, 1.0 / (np.pi * 7.25e-4)):
        host, dev, _, _ = _host_and_device(fgl, torch, "fg_lambda_plane", src, ctypes.c_float(inv))
        bad = np.flatnonzero(host.view(np.uint32) != dev.view(np.uint32))
        assert bad.size == 0, f"inv {inv}: {bad.size} inputs differ, first c = {src[bad[:5]]}"


def test_device_normalize_and_lambda_from_plane(cuda, fgl):
    torch = cuda
    rng = np.random.default_rng(5)
    planes = [workloads.blobs_plane(320, 200, 2, scale=workloads.small_scale(320, 200)),  # already in [0, 1]
              (rng.random((256, 256)) * 3.7).astype(np.float32),                    # normalised by its max
              np.where(rng.random((64, 96)) < 0.01, np.nan, rng.random((64, 96))).astype(np.float32),
              np.full((17, 13), 0.25, np.float32),
              np.array([[-0.0, 0.0, np.nan, -np.nan, 0.5], [1.0, -1.0, np.inf, -np.inf, 0.25]], np.float32)]
    for plane in planes:
        for fn, args in (("fg_normalize_plane", ()), ("fg_lambda_from_plane", (ctypes.c_float(21.5),))):
            host, dev, mh, md = _host_and_device(fgl, torch, fn, plane, *args)
            assert np.array_equal(host.view(np.uint32), dev.view(np.uint32)), fn
            assert np.float32(mh) == np.float32(md), (fn, mh, md)
