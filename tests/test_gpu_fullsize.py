"""GPU parity at the benchmark sizes.

The oracle cannot render whole benchmark frames in test time, so the frames are rendered on the GPU
and checked (1) bit for bit on output tiles the oracle renders exactly (its rectangle mode draws every
grain that can reach the tile), and (2) through size-independent properties: determinism and mean
preservation (coverage of intensity u is u in expectation, src/model.rs:252-265).
"""
import numpy as np
import pytest

from film_grain_gb300 import workloads

pytestmark = pytest.mark.gpu


def _plane_setup(fgl, orc, plane, **kw):
    h, w = plane.shape
    dist = kw.get("dist", "const")
    p = fgl.ParamsBuilder(radius_mean=kw["radius"], radius_stddev=kw.get("sd", 0.0), zoom=kw.get("zoom", 1.0),
                          n_samples=kw["n"], seed=kw["seed"],
                          radius_dist=fgl.RadiusDist.Lognorm if dist == "lognorm" else fgl.RadiusDist.Const).build()
    d = fgl.derive_common(p, (w, h))
    lam = fgl.lambda_plane(fgl.normalize_plane(plane)[0], d.inv_e_pi_r2)
    op = orc.params_struct(dist, kw["radius"], kw.get("sd", 0.0), kw.get("zoom", 1.0), 0.8, kw["n"], kw["seed"])
    od, offs, offs_in = orc.derive(op, w, h)
    return p, d, lam, op, od, offs, offs_in


def test_grainwise_full_frame_1024_rgb(cuda, fgl, orc):
    """The 1024^2 x 3 blob frame, lognormal 0.05/0.025, zoom 2, N=128 (the benchmark frame)."""
    torch = cuda
    rgb = workloads.blobs_rgb(1024, 1024, 0)
    for c in range(3):
        plane = np.ascontiguousarray(rgb[:, :, c])
        p, d, lam, op, od, offs, offs_in = _plane_setup(fgl, orc, plane, radius=0.05, dist="lognorm", sd=0.025,
                                                        zoom=2.0, n=128, seed=42)
        lam_dev = torch.from_numpy(lam).cuda()
        a = fgl.render_grainwise(lam_dev, p, d)
        b = fgl.render_grainwise(lam_dev, p, d)
        torch.cuda.synchronize()
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "renders are not deterministic"
        norm = fgl.normalize_plane(plane)[0]
        assert abs(float(a.mean()) - float(norm.mean())) < 0.01
        # tiles: a corner, the frame centre, and the brightest region of the plane
        iy, ix = np.unravel_index(int(np.argmax(lam)), lam.shape)
        ty, tx = min(2 * iy, 2048 - 48), min(2 * ix, 2048 - 48)
        for (x0, y0) in ((0, 0), (1000 + 16 * c, 1000), (tx, ty)):
            want, _ = orc.render("grain", lam, op, od, offs, rect=(x0, y0, x0 + 48, y0 + 48))
            got = a[y0:y0 + 48, x0:x0 + 48]
            diff = np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))
            assert diff == 0, f"plane {c} tile ({x0},{y0}): {diff} pixels differ"


def test_pixelwise_large_frame_4096(cuda, fgl, orc):
    """One 4096^2 blob plane, lognormal 0.025/0.01, N=256 (the large-frame workload)."""
    torch = cuda
    plane = workloads.blobs_plane(4096, 4096, 3)
    p, d, lam, op, od, offs, offs_in = _plane_setup(fgl, orc, plane, radius=0.025, dist="lognorm", sd=0.01, n=256,
                                                    seed=42)
    out = fgl.render_pixelwise(torch.from_numpy(lam).cuda(), p, d)
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    norm = fgl.normalize_plane(plane)[0]
    assert abs(float(out.mean()) - float(norm.mean())) < 0.01
    iy, ix = np.unravel_index(int(np.argmax(lam)), lam.shape)
    for (x0, y0) in ((0, 0), (2048, 2050), (min(ix, 4096 - 24), min(iy, 4096 - 24))):
        want, _ = orc.render("pixel", lam, op, od, offs_in, rect=(x0, y0, x0 + 24, y0 + 24))
        got = out[y0:y0 + 24, x0:x0 + 24]
        diff = np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))
        assert diff == 0, f"tile ({x0},{y0}): {diff} pixels differ"
