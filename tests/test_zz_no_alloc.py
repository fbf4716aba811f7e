"""The allocation-free pixel-wise entry point, called through the C-ABI.

fg_render_pixelwise_noalloc is for callers that may not allocate GPU memory themselves -- a host
that budgets all device memory and only lends a plug-in its own buffers, or a real-time preview loop
that cannot afford cudaMalloc/cudaFree between frames.  Its scratch is a fixed array inside the
library, shared by every call, so this test makes two calls in a row on different inputs (the second
would expose any stale scratch) and requires each output to equal, bit for bit, what the regular
fg_render_pixelwise produces.  This file is collected last so that a run stopping at the first
failure has already run every other test; it also passes when run alone.
"""
import ctypes

import numpy as np
import pytest

from film_grain_gb300 import workloads

pytestmark = pytest.mark.gpu


def _case(fgl, plane, **kw):
    p = fgl.ParamsBuilder(**kw).build()
    d = fgl.derive_common(p, (plane.shape[1], plane.shape[0]))
    lam = fgl.lambda_plane(fgl.normalize_plane(plane)[0], d.inv_e_pi_r2)
    return p, d, lam


def test_noalloc_matches_pixelwise_two_calls(cuda, fgl):
    torch = cuda
    L = fgl.lib()
    cases = [
        _case(fgl, workloads.ramp_noise(256, 256, 42), radius_mean=0.12, n_samples=64, seed=42),
        _case(fgl, workloads.blobs_plane(160, 120, 5), radius_mean=0.05, radius_dist=fgl.RadiusDist.Lognorm,
              radius_stddev=0.025, zoom=1.5, n_samples=37, seed=9),
    ]
    for p, d, lam in cases:
        want = fgl.render_pixelwise(lam, p, d)
        lam_dev = torch.from_numpy(lam).cuda()
        out = torch.full((d.output_height, d.output_width), float("nan"), dtype=torch.float32, device="cuda")
        offs = np.ascontiguousarray(d.offsets_input, np.float32)
        stream = torch.cuda.current_stream().cuda_stream
        rc = L.fg_render_pixelwise_noalloc(lam_dev.data_ptr(), ctypes.byref(p.c), ctypes.byref(d._c),
                                           offs.ctypes.data, out.data_ptr(), stream)
        assert rc == 0, L.fg_last_error_message().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
            f"{np.count_nonzero(got != want)} pixels differ"


def test_noalloc_rejects_planes_beyond_its_scratch(cuda, fgl):
    torch = cuda
    L = fgl.lib()
    p, d, lam = _case(fgl, np.full((600, 600), 0.5, np.float32), radius_mean=0.1, n_samples=4)
    lam_dev = torch.from_numpy(lam).cuda()
    out = torch.empty((d.output_height, d.output_width), dtype=torch.float32, device="cuda")
    offs = np.ascontiguousarray(d.offsets_input, np.float32)
    rc = L.fg_render_pixelwise_noalloc(lam_dev.data_ptr(), ctypes.byref(p.c), ctypes.byref(d._c), offs.ctypes.data,
                                       out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 5  # FG_ERR_UNSUPPORTED
    assert "at most" in L.fg_last_error_message().decode()
