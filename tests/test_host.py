"""CPU tests of the library's host side: the C-ABI exports, parameter resolution and the host
arithmetic, each against the oracle (no GPU calls)."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(fgl):
    header = open(os.path.join(ROOT, "include", "film_grain_gb300.h")).read()
    declared = set(re.findall(r"FG_API\s+[\w\s\*]+?\b(fg_\w+)\s*\(", header))
    assert len(declared) >= 15
    lib = fgl.lib()
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(fgl.SIGNATURES), declared ^ set(fgl.SIGNATURES)


CASES = [
    dict(dist="const", radius=0.12, sd=0.0, zoom=1.0, sigma=0.8, n=64, seed=42, size=(256, 256)),
    dict(dist="lognorm", radius=0.05, sd=0.025, zoom=2.0, sigma=0.8, n=128, seed=42, size=(1024, 1024)),
    dict(dist="lognorm", radius=0.025, sd=0.01, zoom=1.0, sigma=0.8, n=256, seed=7, size=(4096, 4096)),
    dict(dist="lognorm", radius=0.2, sd=0.0, zoom=0.5, sigma=1.7, n=3, seed=2**63 + 5, size=(33, 17)),
    dict(dist="const", radius=0.7, sd=0.0, zoom=3.25, sigma=0.3, n=1000, seed=0, size=(5, 9)),
]


@pytest.mark.parametrize("c", CASES)
def test_derive_matches_oracle(fgl, orc, c):
    dist = fgl.RadiusDist.Lognorm if c["dist"] == "lognorm" else fgl.RadiusDist.Const
    p = fgl.ParamsBuilder(radius_mean=c["radius"], radius_dist=dist, radius_stddev=c["sd"], zoom=c["zoom"],
                          sigma_px=c["sigma"], n_samples=c["n"], seed=c["seed"]).build()
    d = fgl.derive_common(p, c["size"])
    op = orc.params_struct(c["dist"], c["radius"], c["sd"], c["zoom"], c["sigma"], c["n"], c["seed"])
    od, offs, offs_in = orc.derive(op, *c["size"])
    assert (p.radius_log_mu, p.radius_log_sigma, p.radius_stddev) == (op.radius_log_mu, op.radius_log_sigma,
                                                                      op.radius_stddev)
    assert (d.output_width, d.output_height) == (od.out_w, od.out_h)
    assert (d.inv_e_pi_r2, d.rm, d.delta) == (od.inv_e_pi_r2, od.rm, od.delta)
    assert np.array_equal(d.offsets.view(np.uint32), offs.view(np.uint32))
    assert np.array_equal(d.offsets_input.view(np.uint32), offs_in.view(np.uint32))
    assert fgl.choose_algorithm(p, d) == orc.choose_algorithm(op, 0, od.rm)


def test_choose_algorithm_rules(fgl):
    """src/choose.rs:4-26 on the benchmark workloads and the rule boundaries."""
    def algo(**kw):
        p = fgl.ParamsBuilder(**kw).build()
        return fgl.choose_algorithm(p, fgl.derive_common(p, (64, 64)))
    assert algo(radius_mean=0.12, n_samples=64) == fgl.Algo.Pixel
    assert algo(radius_mean=0.05, radius_dist=fgl.RadiusDist.Lognorm, radius_stddev=0.025, n_samples=128) == \
        fgl.Algo.Grain
    # rule 1 (sigma/mu < 0.1, mu < 0.5, N <= 64) wins before the rm/mu > 8 rule
    assert algo(radius_mean=0.1, n_samples=24, max_radius=fgl.MaxRadius.Absolute(0.9)) == fgl.Algo.Pixel
    lognorm = dict(radius_mean=0.1, radius_dist=fgl.RadiusDist.Lognorm, radius_stddev=0.02)
    assert algo(n_samples=24, max_radius=fgl.MaxRadius.Absolute(0.9), **lognorm) == fgl.Algo.Grain  # rule 2
    assert algo(n_samples=24, **lognorm) == fgl.Algo.Pixel  # rule 3
    assert algo(n_samples=40, **lognorm) == fgl.Algo.Grain  # fall-through
    assert algo(radius_mean=0.1, n_samples=97) == fgl.Algo.Grain
    assert algo(radius_mean=0.1, n_samples=8, algo=fgl.Algo.Grain) == fgl.Algo.Grain


def test_pixelwise_kernel_choice(fgl):
    """The plane-level choice between the per-sample kernel (3 launches per plane) and the block
    kernels (6: the cell table, the plane's emptiness bitmask, the offsets sorted by x, the sparse and
    fat block passes, the epilogue): an interior root block's samples x the cells of one sample's range, against 1.5 x the
    cells of its staged window."""
    def kernels(**kw):
        p = fgl.ParamsBuilder(algo=fgl.Algo.Pixel, **kw).build()
        return fgl.pixelwise_kernel_count(p, fgl.derive_common(p, (256, 256)))
    assert kernels(radius_mean=0.025, n_samples=16) == 3      # reach / window 0.09
    assert kernels(radius_mean=0.025, n_samples=64) == 3      # 0.34
    assert kernels(radius_mean=0.05, n_samples=64) == 3       # 1.37
    assert kernels(radius_mean=0.025, n_samples=256) == 3     # 1.37
    assert kernels(radius_mean=0.05, n_samples=256) == 6      # 5.5
    assert kernels(radius_mean=0.1, n_samples=64) == 6        # 5.5
    assert kernels(radius_mean=0.12, n_samples=64) == 6       # the 256^2 luma workload, 7.3
    assert kernels(radius_mean=0.025, radius_dist=fgl.RadiusDist.Lognorm, radius_stddev=0.01,
                   n_samples=256) == 6                        # the 4096^2 frame's parameters, 6.8
    assert kernels(radius_mean=0.05, radius_dist=fgl.RadiusDist.Lognorm, radius_stddev=0.02, n_samples=2,
                   zoom=2.0) == 3                             # a 64-cell range: the widest the kernel takes
    # a range wider than the per-sample kernel's 64-cell mask stays on the block kernels
    assert kernels(radius_mean=0.3, n_samples=1, cell_delta=0.05) == 6


def test_lambda_and_normalize_match_oracle(fgl, orc):
    rng = np.random.default_rng(3)
    for scale in (1.0, 3.7):
        plane = (rng.random((65, 97)) * scale).astype(np.float32)
        n1, m1 = fgl.normalize_plane(plane)
        n2, m2 = orc.normalize_plane(plane)
        assert m1 == m2 and np.array_equal(n1.view(np.uint32), n2.view(np.uint32))
        for inv in (22.104853, 101.85916, 1e4):
            l1 = fgl.lambda_plane(n1, inv)
            l2 = orc.lambda_plane(n2, inv)
            assert np.array_equal(l1.view(np.uint32), l2.view(np.uint32))


def test_new_entry_points_reject_null_arguments(fgl):
    """fg_pixelwise_kernel_count and fg_batch_kernel_count return FG_ERR_INVALID (4) on null arguments;
    fg_lambda_from_plane on an empty plane returns 0 without touching memory."""
    import ctypes
    L = fgl.lib()
    n = ctypes.c_int32(-1)
    assert L.fg_pixelwise_kernel_count(None, None, None, ctypes.byref(n)) == 4 and n.value == -1
    p = fgl.ParamsBuilder(radius_mean=0.1, n_samples=8, algo=fgl.Algo.Pixel).build()
    d = fgl.derive_common(p, (16, 16))
    assert L.fg_pixelwise_kernel_count(p.c, d._c, None, ctypes.byref(n)) == 4
    assert L.fg_batch_kernel_count(None, ctypes.byref(n)) == 4
    assert L.fg_lambda_from_plane(None, 0, 1.0, None) == 0.0


def test_lambda_planes_split_over_threads(fgl, orc):
    """Planes large enough to be split over the host threads (per-chunk maxima), with values above 1
    (the normalising branch), a negative value and a NaN: normalize + lambda, and the fused pass, against
    the oracle bit for bit."""
    rng = np.random.default_rng(5)
    for scale in (1.0, 2.5):
        plane = (rng.random((1024, 1031)) * scale).astype(np.float32)
        plane[3, 5] = -0.25
        plane[700, 9] = np.nan
        plane[1023, 1030] = np.float32(scale * 1.01)  # the maximum sits in the last chunk
        n1, m1 = fgl.normalize_plane(plane)
        n2, m2 = orc.normalize_plane(plane)
        assert m1 == m2 and np.array_equal(n1.view(np.uint32), n2.view(np.uint32))
        for inv in (22.104853, 1e4):
            l1 = fgl.lambda_plane(n1, inv)
            assert np.array_equal(l1.view(np.uint32), orc.lambda_plane(n2, inv).view(np.uint32))
            l3, m3 = fgl.lambda_from_plane(plane, inv)
            assert m3 == m1 and np.array_equal(l3.view(np.uint32), l1.view(np.uint32))


@pytest.mark.parametrize("kw,field", [
    (dict(radius_mean=0.0), "radius"), (dict(radius_mean=float("nan")), "radius"),
    (dict(radius_stddev=-1.0), "radius-stddev"), (dict(zoom=0.0), "zoom"), (dict(sigma_px=-2.0), "sigma"),
    (dict(cell_delta=-0.5), "cell"),
])
def test_params_validation(fgl, kw, field):
    with pytest.raises(fgl.ParamsError, match=field):
        fgl.ParamsBuilder(**kw).build()


def test_max_radius_validation(fgl):
    with pytest.raises(fgl.ParamsError, match="quantile"):
        fgl.ParamsBuilder(max_radius=fgl.MaxRadius.Quantile(1.0)).build()
    with pytest.raises(fgl.ParamsError, match="absolute"):
        fgl.ParamsBuilder(max_radius=fgl.MaxRadius.Absolute(-1.0)).build()
    with pytest.raises(fgl.ParamsError, match="roi"):
        fgl.ParamsBuilder(roi=fgl.Roi(4, 4, 4, 8)).build()


def test_n_samples_zero_becomes_one(fgl):
    assert fgl.ParamsBuilder(n_samples=0).build().n_samples == 1


def test_size_and_dry_run(fgl, orc):
    p = fgl.ParamsBuilder(size=(100, None)).build()
    st = fgl.dry_run_with_input_image((30, 40, 3), p)
    od, _, _ = orc.derive(orc.params_struct(), 40, 30, size=(100, None))
    assert st.output_size == (od.out_w, od.out_h) == (100, 75)
    p = fgl.ParamsBuilder(zoom=1.5, roi=fgl.Roi(2, 3, 12, 9)).build()
    st = fgl.dry_run_with_input_image((30, 40, 3), p)
    assert st.input_size == (10, 6) and st.output_size == (15, 9)
    with pytest.raises(fgl.RenderError, match="ROI exceeds"):
        fgl.dry_run_with_input_image((8, 8, 3), p)


def test_empty_input_is_an_error(fgl):
    p = fgl.ParamsBuilder().build()
    with pytest.raises(fgl.RenderError, match="empty"):
        fgl.derive_common(p, (0, 5))


def test_ziggurat_tables_agree(orc):
    """The library's generated tables equal the oracle's run-time construction, value for value."""
    x, f = orc.zig_tables()
    src = open(os.path.join(ROOT, "film_grain_gb300", "csrc", "zig_tables.h")).read()
    def table(name):
        body = src.split(f"#define {name}_INIT {{")[1].split("}")[0]
        return np.array([float(v) for v in re.findall(r"[-\d.eE]+", body.replace("\\", ""))])
    assert np.array_equal(table("FG_ZIG_NORM_X"), x)
    assert np.array_equal(table("FG_ZIG_NORM_F"), f)


def test_render_requires_gpu_and_fails_loudly(fgl):
    """Without a GPU the render entry points raise: there is no CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = fgl.ParamsBuilder(n_samples=4).build()
    d = fgl.derive_common(p, (8, 8))
    with pytest.raises(fgl.GpuError):
        fgl.render_pixelwise(np.ones((8, 8), np.float32), p, d)
