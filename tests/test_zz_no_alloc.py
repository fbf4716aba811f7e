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
        _case(fgl, workloads.blobs_plane(160, 120, 5, scale=workloads.small_scale(160, 120)), radius_mean=0.05, radius_dist=fgl.RadiusDist.Lognorm,
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


def _noalloc(fgl, torch, p, d, lam):
    L = fgl.lib()
    lam_dev = torch.from_numpy(lam).cuda()
    out = torch.full((d.output_height, d.output_width), float("nan"), dtype=torch.float32, device="cuda")
    offs = np.ascontiguousarray(d.offsets_input, np.float32)
    rc = L.fg_render_pixelwise_noalloc(lam_dev.data_ptr(), ctypes.byref(p.c), ctypes.byref(d._c), offs.ctypes.data,
                                       out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    msg = L.fg_last_error_message().decode()
    if rc == 0:
        torch.cuda.synchronize()
    return rc, out, msg


def test_noalloc_fills_its_cell_table_exactly(cuda, fgl):
    """A 512 x 512 input plane fills the scratch's cell table to the last entry; N = 4096 fills its
    offset slots.  Both equal the regular render bit for bit."""
    torch = cuda
    for plane, kw in ((workloads.blobs_plane(512, 512, 11, scale=workloads.small_scale(512, 512)), dict(radius_mean=0.1, n_samples=16, seed=3)),
                      (workloads.ramp_noise(48, 40, 2), dict(radius_mean=0.12, n_samples=4096, seed=5))):
        p, d, lam = _case(fgl, plane, **kw)
        want = fgl.render_pixelwise(lam, p, d)
        rc, out, msg = _noalloc(fgl, torch, p, d, lam)
        assert rc == 0, msg
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
            f"{np.count_nonzero(got != want)} pixels differ"


def test_noalloc_rejects_samples_beyond_its_scratch(cuda, fgl):
    torch = cuda
    p, d, lam = _case(fgl, workloads.ramp_noise(16, 16, 1), radius_mean=0.12, n_samples=4097)
    rc, _, msg = _noalloc(fgl, torch, p, d, lam)
    assert rc == 5 and "4096" in msg  # FG_ERR_UNSUPPORTED


_RESET_SCRIPT = r'''
import ctypes, glob, os, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import film_grain_gb300 as fg
from film_grain_gb300 import workloads
cands = sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")) + sorted(glob.glob("/usr/local/cuda/targets/*/lib/libcudart.so*"))
rt = ctypes.CDLL(cands[0])
L = fg.lib()
plane = workloads.blobs_plane(96, 80, 4, scale=workloads.small_scale(96, 80))
p = fg.ParamsBuilder(radius_mean=0.1, n_samples=24, seed=8).build()
d = fg.derive_common(p, (96, 80))
lam = fg.lambda_plane(fg.normalize_plane(plane)[0], d.inv_e_pi_r2)
want = fg.render_pixelwise(lam, p, d)
offs = np.ascontiguousarray(d.offsets_input, np.float32)
n_out = d.output_width * d.output_height
for rnd in range(2):
    dl, do = ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(dl), ctypes.c_size_t(lam.nbytes)) == 0
    assert rt.cudaMalloc(ctypes.byref(do), ctypes.c_size_t(4 * n_out)) == 0
    assert rt.cudaMemcpy(dl, lam.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(lam.nbytes), 1) == 0
    rc = L.fg_render_pixelwise_noalloc(dl.value, ctypes.byref(p.c), ctypes.byref(d._c), offs.ctypes.data, do.value, None)
    assert rc == 0, L.fg_last_error_message()
    got = np.empty(n_out, np.float32)
    assert rt.cudaMemcpy(got.ctypes.data_as(ctypes.c_void_p), do, ctypes.c_size_t(4 * n_out), 2) == 0
    assert np.array_equal(got.view(np.uint32), want.reshape(-1).view(np.uint32)), rnd
    if rnd == 0:
        assert rt.cudaDeviceReset() == 0  # ends this process's context; the next call must look up anew
print("reset ok")
'''


def test_noalloc_after_context_reset(cuda, fgl, tmp_path):
    """In a fresh process: a call, cudaDeviceReset (which destroys the process's context on the
    device), then a call on new buffers; both equal the regular render."""
    import os
    import subprocess
    import sys
    script = tmp_path / "reset_case.py"
    script.write_text(_RESET_SCRIPT)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, str(script), root], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "reset ok" in r.stdout, r.stdout + r.stderr
