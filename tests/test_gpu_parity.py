"""GPU parity: the sm_103a integrators against the CPU oracle, bit for bit.

Every case renders the same seeded plane through the library's C-ABI (host lambda plane -> GPU
integrator) and through the oracle (a C restatement of src/pixelwise.rs / src/grainwise.rs), and
requires the f32 output planes to be bit-identical (coverage counts equal, the same count * (1/N)).
"""
import numpy as np
import pytest

from film_grain_gb300 import workloads

pytestmark = pytest.mark.gpu


def _setup(fgl, orc, plane, radius=0.1, dist="const", sd=0.0, zoom=1.0, n=32, seed=5489, sigma=0.8,
           cell=None, maxr=None, size=None):
    h, w = plane.shape
    kw = dict(radius_mean=radius, radius_dist=fgl.RadiusDist.Lognorm if dist == "lognorm" else fgl.RadiusDist.Const,
              radius_stddev=sd, zoom=zoom, n_samples=n, seed=seed, sigma_px=sigma, cell_delta=cell, size=size)
    if maxr is not None:
        kw["max_radius"] = fgl.MaxRadius.Absolute(maxr)
    p = fgl.ParamsBuilder(**kw).build()
    d = fgl.derive_common(p, (w, h))
    norm, _ = fgl.normalize_plane(plane)
    lam = fgl.lambda_plane(norm, d.inv_e_pi_r2)
    op = orc.params_struct(dist, radius, sd, zoom, sigma, n, seed)
    od, offs, offs_in = orc.derive(op, w, h, ("absolute", maxr) if maxr is not None else ("quantile", 0.999), cell,
                                   size)
    onorm, _ = orc.normalize_plane(plane)
    olam = orc.lambda_plane(onorm, od.inv_e_pi_r2)
    assert np.array_equal(lam.view(np.uint32), olam.view(np.uint32)), "lambda planes differ"
    assert np.array_equal(d.offsets, offs) and np.array_equal(d.offsets_input, offs_in)
    assert (d.output_width, d.output_height, d.rm, d.delta) == (od.out_w, od.out_h, od.rm, od.delta)
    return p, d, lam, op, od, offs, offs_in


def _check(algo, fgl, orc, plane, **kw):
    p, d, lam, op, od, offs, offs_in = _setup(fgl, orc, plane, **kw)
    if algo == "pixel":
        got = fgl.render_pixelwise(lam, p, d)
        want, _ = orc.render("pixel", lam, op, od, offs_in)
    else:
        got = fgl.render_grainwise(lam, p, d)
        want, _ = orc.render("grain", lam, op, od, offs)
    assert got.shape == want.shape
    diff = np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))
    assert diff == 0, f"{diff} of {got.size} pixels differ (max abs {np.abs(got - want).max()})"
    return got


def _blobs(w, h, seed=11):
    """A blob plane with blobs scaled to its size: dark background, mid tones and saturated spots."""
    return workloads.blobs_plane(w, h, seed, scale=workloads.small_scale(w, h))


# ------------------------------------------------------------------ pixel-wise
def test_pixelwise_ramp_256_n64(cuda, fgl, orc):
    """The 256x256 luma ramp workload: const radius 0.12, N=64, zoom 1, seed 42."""
    out = _check("pixel", fgl, orc, workloads.ramp_noise(256, 256, 42), radius=0.12, n=64, seed=42)
    slow, unstaged, subdiv, blocks = fgl.pixelwise_diagnostics()
    # interior blocks stage their windows; only border blocks, which own few samples, regenerate
    assert blocks > 0 and unstaged < blocks // 4 and slow < 0.05 * 256 * 256 * 64
    assert abs(float(out.mean()) - 0.5) < 0.01


@pytest.mark.parametrize("n", [1, 7, 37, 100])
def test_pixelwise_sample_counts(cuda, fgl, orc, n):
    _check("pixel", fgl, orc, _blobs(48, 40), radius=0.1, n=n, seed=3)


def test_pixelwise_lognormal(cuda, fgl, orc):
    _check("pixel", fgl, orc, _blobs(64, 48), radius=0.05, dist="lognorm", sd=0.025, n=40, seed=7)


@pytest.mark.parametrize("zoom", [0.5, 1.5, 2.0, 3.0])
def test_pixelwise_zoom(cuda, fgl, orc, zoom):
    _check("pixel", fgl, orc, _blobs(40, 36), radius=0.1, n=16, zoom=zoom, seed=9)


def test_pixelwise_cell_and_absolute_max_radius(cuda, fgl, orc):
    _check("pixel", fgl, orc, _blobs(40, 40), radius=0.15, n=20, cell=0.37, maxr=0.3, seed=13)


def test_pixelwise_rejection_regime(cuda, fgl, orc):
    """cell 1.0, radius 0.2: lambda*delta^2 >= 12 in bright areas (Poisson rejection branch)."""
    plane = np.clip(workloads.ramp_noise(32, 32, 5) * 1.2, 0, 1).astype(np.float32)
    _check("pixel", fgl, orc, plane, radius=0.2, n=16, cell=1.0, seed=17)


def test_pixelwise_dense_subdivides(cuda, fgl, orc):
    """A saturated plane with many samples per cell: every window overflows shared memory and, as the
    samples reach more than four windows' worth of cells, splits into quadrants."""
    plane = np.ones((24, 24), np.float32)
    _check("pixel", fgl, orc, plane, radius=0.05, n=256, seed=19)
    _, _, subdiv, _ = fgl.pixelwise_diagnostics()
    assert subdiv > 0


def test_pixelwise_dense_regenerates(cuda, fgl, orc):
    """A saturated plane whose blocks' samples reach about as many cells as a window holds: the whole
    plane runs the per-sample kernel (dense form)."""
    plane = np.ones((24, 24), np.float32)
    _check("pixel", fgl, orc, plane, radius=0.05, n=64, seed=19)
    slow, unstaged, subdiv, _ = fgl.pixelwise_diagnostics()
    assert subdiv == 0 and unstaged > 0 and slow == 24 * 24 * 64


def test_pixelwise_dense_block_regenerates(cuda, fgl, orc):
    """A saturated plane on the block kernel (samples reach 2.7 windows of cells): its overflowing
    dense windows regenerate per sample instead of subdividing."""
    plane = np.ones((24, 24), np.float32)
    _check("pixel", fgl, orc, plane, radius=0.05, n=128, seed=19)
    slow, unstaged, subdiv, _ = fgl.pixelwise_diagnostics()
    assert subdiv == 0 and unstaged > 0 and slow > 0


def test_pixelwise_mixed_density_blocks(cuda, fgl, orc):
    """A dark left half (0.1) and a bright right half (0.95) on the block kernel: sparse windows
    stage, dense ones regenerate."""
    plane = np.where(np.arange(64)[None, :] < 32, 0.1, 0.95).astype(np.float32).repeat(64, 0)
    _check("pixel", fgl, orc, plane, radius=0.05, n=128, seed=37)
    slow, unstaged, _, blocks = fgl.pixelwise_diagnostics()
    assert 0 < unstaged < blocks


@pytest.mark.parametrize("n", [16, 64])
def test_pixelwise_sparse_regenerates(cuda, fgl, orc, n):
    """Radius 0.025 (cells of 1/40 pixel) with few samples per pixel: the samples reach fewer cells
    than a staged window holds, so the plane runs the per-sample kernel (both forms: dark background
    and bright blobs)."""
    _check("pixel", fgl, orc, _blobs(48, 40), radius=0.025, n=n, seed=29)
    slow, unstaged, _, _ = fgl.pixelwise_diagnostics()
    assert unstaged > 0 and slow == 48 * 40 * n


def test_pixelwise_regen_zoom_and_lognormal(cuda, fgl, orc):
    """The per-sample kernel with zoom 2 and log-normal radii (ranges of 7 or 8 cells per axis: up to
    the full 64-cell mask)."""
    _check("pixel", fgl, orc, _blobs(40, 36), radius=0.05, dist="lognorm", sd=0.02, n=2, zoom=2.0, seed=41)
    slow, _, _, _ = fgl.pixelwise_diagnostics()
    assert slow == 80 * 72 * 2


def test_pixelwise_lognormal_small_radius(cuda, fgl, orc):
    """Log-normal radius 0.025/0.01 at N=256 (the large-frame workload's parameters): staged windows."""
    _check("pixel", fgl, orc, _blobs(40, 32), radius=0.025, dist="lognorm", sd=0.01, n=256, seed=31)


@pytest.mark.parametrize("n,zoom,dist,radius", [(256, 1.0, "lognorm", 0.04), (64, 1.0, "const", 0.08),
                                                (16, 1.0, "lognorm", 0.15), (256, 2.0, "lognorm", 0.04),
                                                (100, 0.5, "const", 0.1)])
def test_pixelwise_sparse_pass_forms(cuda, fgl, orc, n, zoom, dist, radius):
    """The sparse block pass (6 launches) in its forms: one offset per thread (N = 256) or several
    threads per offset sharing its rows (N 64, 16); rectangles within the 4 x 4 range table (zoom 1) or
    beyond it (zoom 2: cell ranges computed per sample); zoom 0.5; on a plane large enough for the
    4 x 4-pixel blocks, mixing dense and sparse regions.  The sample step runs grain-major (each staged
    grain tests the samples within its radius) at N = 256, sample-major where a grain can reach half a
    pixel (log-normal r 0.15: max radius 0.46)."""
    plane = _blobs(160, 128, seed=5)
    kw = dict(radius=radius, dist=dist, sd=0.4 * radius if dist == "lognorm" else 0.0, zoom=zoom, n=n, seed=41)
    p, d, *_ = _setup(fgl, orc, plane, **kw)
    assert fgl.pixelwise_kernel_count(p, d) == 6
    _check("pixel", fgl, orc, plane, **kw)
    sample_major, grain_major = fgl.pixelwise_sparse_forms()
    if n == 256:
        assert grain_major > 0
    if radius == 0.15:
        assert sample_major > 0 and grain_major == 0


@pytest.mark.parametrize("radius,n,zoom", [(0.025, 256, 1.0), (0.05, 128, 0.75), (0.1, 64, 1.0), (0.04, 32, 3.0),
                                           (0.08, 256, 1.0)])
def test_pixelwise_grain_major_form(cuda, fgl, orc, radius, n, zoom):
    """The sparse pass's grain-major form against the oracle: log-normal radii, zoom in and out (the
    phase bands wrap and span several bins), N from 32 to 256, a plane with dense blobs and empty
    regions.  At r 0.08, N 256 a grain has about 13 candidates, more than a warp's queue holds for 32
    grains, so the warps test their candidates lane by lane."""
    plane = _blobs(144, 112, seed=9)
    kw = dict(radius=radius, dist="lognorm", sd=0.4 * radius, zoom=zoom, n=n, seed=77)
    _check("pixel", fgl, orc, plane, **kw)
    sample_major, grain_major = fgl.pixelwise_sparse_forms()
    assert grain_major > 0


def test_pixelwise_empty_and_tiny(cuda, fgl, orc):
    _check("pixel", fgl, orc, np.zeros((16, 16), np.float32), radius=0.1, n=8)
    _check("pixel", fgl, orc, np.full((1, 1), 0.5, np.float32), radius=0.1, n=8)
    _check("pixel", fgl, orc, np.full((2, 3), 0.7, np.float32), radius=0.3, n=5, zoom=2.0)


def test_pixelwise_wide_filter(cuda, fgl, orc):
    _check("pixel", fgl, orc, _blobs(32, 32), radius=0.1, n=32, sigma=4.0, seed=21)


def test_pixelwise_forced_size(cuda, fgl, orc):
    """--size changes the output grid while the integrator keeps mapping with params.zoom."""
    _check("pixel", fgl, orc, _blobs(40, 30), radius=0.1, n=12, size=(50, None), seed=23)


# ------------------------------------------------------------------ grain-wise
def test_grainwise_blob_crop_lognormal_zoom2_n128(cuda, fgl, orc):
    """A 96x80 crop of the 1024^2 blob workload: lognormal 0.05/0.025, zoom 2, N=128."""
    plane = workloads.blobs_plane(1024, 1024, 0)[300:380, 400:496]
    _check("grain", fgl, orc, np.ascontiguousarray(plane), radius=0.05, dist="lognorm", sd=0.025, zoom=2.0, n=128,
           seed=42)


@pytest.mark.parametrize("n", [1, 31, 33, 200])
def test_grainwise_sample_counts(cuda, fgl, orc, n):
    _check("grain", fgl, orc, _blobs(40, 36), radius=0.1, n=n, seed=5)


@pytest.mark.parametrize("zoom", [0.5, 1.0, 1.5, 4.0])
def test_grainwise_zoom(cuda, fgl, orc, zoom):
    _check("grain", fgl, orc, _blobs(36, 30), radius=0.08, n=24, zoom=zoom, seed=29)


def test_grainwise_large_radius(cuda, fgl, orc):
    """radius_out > 0.5 px: the disks cover several pixel centres per offset."""
    _check("grain", fgl, orc, _blobs(24, 24), radius=0.8, n=16, zoom=2.0, maxr=1.0, seed=31)


def test_grainwise_empty_and_tiny(cuda, fgl, orc):
    _check("grain", fgl, orc, np.zeros((16, 16), np.float32), radius=0.1, n=8)
    _check("grain", fgl, orc, np.full((1, 1), 0.5, np.float32), radius=0.1, n=8)


def test_grainwise_forced_size(cuda, fgl, orc):
    _check("grain", fgl, orc, _blobs(40, 30), radius=0.1, n=12, size=(33, 70), seed=37)


# ------------------------------------------------------------------ whole-image path with the fused colour epilogue
@pytest.mark.parametrize("mode", ["luma", "rgb"])
@pytest.mark.parametrize("algo", ["pixel", "grain"])
def test_render_image_matches_oracle(cuda, fgl, orc, mode, algo):
    rgb = workloads.blobs_rgb(48, 40, 3, scale=workloads.small_scale(48, 40))
    p = fgl.ParamsBuilder(radius_mean=0.1, n_samples=24, zoom=1.5, seed=77,
                          color_mode=fgl.ColorMode.Luma if mode == "luma" else fgl.ColorMode.Rgb,
                          algo=fgl.Algo.Pixel if algo == "pixel" else fgl.Algo.Grain).build()
    got, stats = fgl.render_with_input_image(rgb, p)
    op = orc.params_struct("const", 0.1, 0.0, 1.5, 0.8, 24, 77)
    want, chosen = orc.render_image(rgb, mode, 2 if algo == "pixel" else 1, op)
    assert stats.algorithm == (fgl.Algo.Pixel if algo == "pixel" else fgl.Algo.Grain)
    assert got.shape == want.shape
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} bytes differ"


def test_render_image_roi(cuda, fgl, orc):
    rgb = workloads.blobs_rgb(64, 64, 4, scale=workloads.small_scale(64, 64))
    p = fgl.ParamsBuilder(radius_mean=0.1, n_samples=16, seed=5, roi=fgl.Roi(8, 4, 40, 36)).build()
    got, stats = fgl.render_with_input_image(rgb, p)
    op = orc.params_struct("const", 0.1, 0.0, 1.0, 0.8, 16, 5)
    want, _ = orc.render_image(np.ascontiguousarray(rgb[4:36, 8:40]), "luma", 0, op)
    assert stats.input_size == (32, 32)
    assert np.array_equal(got, want)


def test_cancel_before_launch(cuda, fgl):
    plane = _blobs(16, 16)
    p = fgl.ParamsBuilder(n_samples=4).build()
    d = fgl.derive_common(p, (16, 16))
    lam = fgl.lambda_plane(fgl.normalize_plane(plane)[0], d.inv_e_pi_r2)
    with pytest.raises(fgl.CancelledError):
        fgl.render_pixelwise(lam, p, d, cancel=lambda: True)


def test_device_tensors_in_and_out(cuda, fgl, orc):
    """torch CUDA tensors go through the same entry point without host staging."""
    torch = cuda
    plane = _blobs(40, 32)
    p, d, lam, op, od, offs, offs_in = _setup(fgl, orc, plane, radius=0.1, n=16, seed=41)
    out = fgl.render_grainwise(torch.from_numpy(lam).cuda(), p, d)
    torch.cuda.synchronize()
    want, _ = orc.render("grain", lam, op, od, offs)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))
