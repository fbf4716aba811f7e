"""Cancellation inside a running launch.

The crate's CPU integrators poll their cancel closure per row, pixel, grain and offset
(src/pixelwise.rs:28, src/grainwise.rs:30-93) and return RenderError::Cancelled; the viewer relies on
it to drop a superseded render (latest job wins).  Here the closure is polled by a host thread, the
library mirrors it into mapped memory and the persistent / block kernels stop at their next work
item.  Each case renders a plane that takes a few hundred milliseconds, cancels it a quarter of the
way in, and checks that the call returns early with the kernel-side stop reported, and that the next
render of the same plane is bit-identical to an uncancelled one.  No GPU fault is involved: the
kernels read a flag and return.
"""
import time

import numpy as np
import pytest

from film_grain_gb300 import workloads

pytestmark = pytest.mark.gpu

CASES = {
    # the block kernels (lean pass, deferred fat pass)
    "pixel_blocks": dict(size=4096, algo="pixel", kw=dict(radius_mean=0.025, radius_stddev=0.01, n_samples=256, seed=42,
                                                          lognorm=True)),
    # the per-sample kernel
    "pixel_per_sample": dict(size=4096, algo="pixel", kw=dict(radius_mean=0.025, n_samples=256, seed=7)),
    # the grain-wise persistent kernel on a saturated plane (u = 1: thousands of grains per pixel)
    "grain": dict(size=1024, algo="grain", level=1.0, kw=dict(radius_mean=0.025, n_samples=256, seed=42)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_cancel_stops_a_running_launch(cuda, fgl, name):
    torch = cuda
    case = CASES[name]
    kw = dict(case["kw"])
    if kw.pop("lognorm", False):
        kw["radius_dist"] = fgl.RadiusDist.Lognorm
    kw["algo"] = fgl.Algo.Pixel if case["algo"] == "pixel" else fgl.Algo.Grain
    p = fgl.ParamsBuilder(**kw).build()
    if "level" in case:
        plane = np.full((case["size"], case["size"]), case["level"], np.float32)
    else:
        plane = workloads.blobs_plane(case["size"], case["size"], 3)
    d = fgl.derive_common(p, (case["size"], case["size"]))
    lam = torch.from_numpy(fgl.lambda_plane(fgl.normalize_plane(plane)[0], d.inv_e_pi_r2)).cuda()
    render = fgl.render_pixelwise if case["algo"] == "pixel" else fgl.render_grainwise
    if case["algo"] == "pixel":
        want_kernels = (3,) if name == "pixel_per_sample" else (4, 6)
        assert fgl.pixelwise_kernel_count(p, d) in want_kernels  # the case exercises the kernel it names

    render(lam, p, d)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    want = render(lam, p, d)
    torch.cuda.synchronize()
    full = time.perf_counter() - t0
    assert full > 0.1, f"plane too fast ({full * 1e3:.1f} ms) to cancel in flight"

    start = time.perf_counter()
    with pytest.raises(fgl.CancelledError) as err:
        render(lam, p, d, cancel=lambda: time.perf_counter() - start > 0.25 * full)
    elapsed = time.perf_counter() - start
    assert "inside a kernel" in str(err.value)
    assert elapsed < 0.75 * full, f"cancelled call took {elapsed * 1e3:.0f} ms of {full * 1e3:.0f} ms"

    again = render(lam, p, d)
    torch.cuda.synchronize()
    assert torch.equal(again.view(torch.int32), want.view(torch.int32))


def test_cancel_whole_image_inside_a_launch(cuda, fgl):
    """fg_render_image (render_with_input_image_cancelable, src/lib.rs:86-93) on a 2048^2 RGB frame."""
    rgb = workloads.blobs_rgb(2048, 2048, 1)
    p = fgl.ParamsBuilder(radius_mean=0.025, radius_dist=fgl.RadiusDist.Lognorm, radius_stddev=0.01, n_samples=256,
                          seed=42, algo=fgl.Algo.Pixel, color_mode=fgl.ColorMode.Rgb).build()
    want, _ = fgl.render_with_input_image(rgb, p)
    t0 = time.perf_counter()
    fgl.render_with_input_image(rgb, p)
    full = time.perf_counter() - t0
    start = time.perf_counter()
    with pytest.raises(fgl.CancelledError):
        fgl.render_with_input_image(rgb, p, cancel=lambda: time.perf_counter() - start > 0.25 * full)
    assert time.perf_counter() - start < 0.75 * full
    again, _ = fgl.render_with_input_image(rgb, p)
    assert np.array_equal(again, want)
