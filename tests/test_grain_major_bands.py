"""The grain-major form of the pixel-wise sparse pass (fg_pixelwise_sparse.cuh, sparse_grain_pass) finds
the samples a grain covers through a band of offset phases.  This CPU test restates, in f32 numpy
arithmetic, the band and the candidate pixel the kernel computes, with the plane conditions and the
rounding margin of plan_grain_major (fg_pixelwise.cu), and checks against a brute force over pixels
and offsets that every (grain, sample) pair passing the reference's disk test (src/pixelwise.rs:96-99)
is a candidate, at its candidate pixel."""
import numpy as np
import pytest

f = np.float32
BINS = 16
RINT = f(12582912.0)


def _eps(out_size, zoom, offs):
    coord = out_size + float(np.abs(offs).max()) * zoom + 2.0
    return coord * 2.0**-21 + 2.0**-20, coord


def _bins(v):
    fr = (v - np.floor(v)).astype(f)
    return np.minimum((fr * f(BINS)).astype(np.int64), BINS - 1)


@pytest.mark.parametrize("zoom,rm,sigma,size,n", [(1.0, 0.07, 0.8, 4096, 256), (1.0, 0.3, 0.8, 4096, 64),
                                                  (2.0, 0.15, 0.5, 8192, 100), (0.5, 0.2, 1.0, 512, 100),
                                                  (1.0, 0.36, 0.8, 60000, 64), (3.0, 0.12, 0.3, 30000, 32)])
def test_phase_band_holds_every_covered_sample(zoom, rm, sigma, size, n):
    rng = np.random.default_rng(int(zoom * 100 + n))
    z = f(zoom)
    iz = f(f(1.0) / z)
    offs = rng.normal(0.0, sigma, (n, 2)).astype(f)
    eps, coord = _eps(size, zoom, offs)
    assert coord < 2.0**21 and rm * zoom + eps <= 0.4  # the plane allows the form
    ozx, ozy = (offs[:, 0] * z).astype(f), (offs[:, 1] * z).astype(f)
    xbin, ybin = _bins(ozx), _bins(ozy)
    hits = 0
    for _ in range(120):
        r = f(rng.uniform(0.0, rm))
        rr = f(r * r)
        gx, gy = f(rng.uniform(0.0, size * iz)), f(rng.uniform(0.0, size * iz))
        # brute force: every pixel near the grain, every offset, the reference's xg and disk test
        xs = np.arange(int(gx * zoom) - 3, int(gx * zoom) + 4)
        ys = np.arange(int(gy * zoom) - 3, int(gy * zoom) + 4)
        truth = set()
        for k in range(n):
            dx = (((xs.astype(f) + f(0.5)) * iz - offs[k, 0]).astype(f) - gx).astype(f)
            dy = (((ys.astype(f) + f(0.5)) * iz - offs[k, 1]).astype(f) - gy).astype(f)
            d2 = ((dx * dx).astype(f)[None, :] + (dy * dy).astype(f)[:, None]).astype(f)
            truth |= {(k, int(xs[i]), int(ys[j])) for j, i in zip(*np.nonzero(d2 <= rr))}
        # the kernel's band, bins and candidate pixels
        w = f(np.sqrt(np.float64(rr)) * np.float64(z * f(1.0000039)) + eps)
        px, py = f(f(gx * z) - f(0.5)), f(f(gy * z) - f(0.5))
        lx, ly = f(f(np.floor(px) - px) - w), f(f(np.floor(py) - py) - w)
        lx, ly = f(lx - np.floor(lx)), f(ly - np.floor(ly))
        bx = {b % BINS for b in range(min(int(lx * BINS), BINS - 1), int((lx + f(2) * w) * BINS) + 1)}
        by = {b % BINS for b in range(min(int(ly * BINS), BINS - 1), int((ly + f(2) * w) * BINS) + 1)}
        found = set()
        for k in np.nonzero(np.isin(xbin, list(bx)) & np.isin(ybin, list(by)))[0]:
            rx = f(f(f(px + ozx[k]) + RINT) - RINT)
            ry = f(f(f(py + ozy[k]) + RINT) - RINT)
            dx = f(f(f(f(rx + f(0.5)) * iz) - offs[k, 0]) - gx)
            dy = f(f(f(f(ry + f(0.5)) * iz) - offs[k, 1]) - gy)
            if f(f(dx * dx) + f(dy * dy)) <= rr:
                found.add((int(k), int(rx), int(ry)))
        assert found == truth
        hits += len(truth)
    assert hits > 0
