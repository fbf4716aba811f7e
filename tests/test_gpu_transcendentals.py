"""How often the device's f64 transcendentals disagree with the platform libm on the arguments the
samplers actually see, and whether a disagreement can reach an integer outcome.

The crate's samplers call the platform libm (glibc) in f64: exp(-lambda*delta^2) for the Knuth
threshold of every pixel-wise cell (src/pixelwise.rs:77-82 via rand_distr's Poisson::new), and
exp(-lambda) / log(lambda) for every grain-wise pixel's Poisson (src/grainwise.rs:41-43).  The device
uses CUDA's f64 exp / log (here through torch's float64 CUDA kernels, which call the same CUDA math
library).  A last-ulp difference changes a Knuth threshold floor(exp(-x) * 2^53) by at most one, and
then changes a cell's grain count only if its first 53-bit draw equals that threshold exactly
(probability 2^-53 per cell).  This test counts the disagreements on the lambda planes of the
benchmark frames and checks that every one is a single ulp.
"""
import numpy as np
import pytest

from film_grain_gb300 import workloads

pytestmark = pytest.mark.gpu


def _lambdas(fgl):
    out = []
    for size, r, sd, n, zoom, seed in ((4096, 0.025, 0.01, 256, 1.0, 1), (1024, 0.05, 0.025, 128, 2.0, 0)):
        p = fgl.ParamsBuilder(radius_mean=r, radius_dist=fgl.RadiusDist.Lognorm, radius_stddev=sd, n_samples=n,
                              zoom=zoom).build()
        d = fgl.derive_common(p, (size, size))
        rgb = workloads.blobs_rgb(size, size, seed)
        for c in range(3):
            lam = fgl.lambda_plane(fgl.normalize_plane(np.ascontiguousarray(rgb[:, :, c]))[0], d.inv_e_pi_r2)
            out.append((np.unique(lam), d.delta))
    return out


def _ulps(a, b):
    return np.abs(a.view(np.int64) - b.view(np.int64))


def test_device_exp_log_against_platform_libm(cuda, orc, record_property):
    torch = cuda
    import film_grain_gb300 as fgl
    total, differ_exp, differ_thresh, differ_log = 0, 0, 0, 0
    for lam, delta in _lambdas(fgl):
        lam = lam[lam > 0]
        # pixel-wise: the cell threshold (f32 product lambda * delta * delta, then f64)
        e = (lam * np.float32(delta) * np.float32(delta)).astype(np.float64)
        e = e[e < 12.0]
        host = orc.libm_f64("exp", -e)
        dev = torch.exp(torch.from_numpy(-e).cuda()).cpu().numpy()
        assert _ulps(host, dev).max(initial=0) <= 1
        differ_exp += int(np.count_nonzero(host != dev))
        th_h = np.floor(host * 2.0 ** 53)
        th_d = np.floor(dev * 2.0 ** 53)
        assert np.abs(th_h - th_d).max(initial=0) <= 1
        differ_thresh += int(np.count_nonzero(th_h != th_d))
        # grain-wise: Poisson(lambda) set-up
        l64 = lam.astype(np.float64)
        hl = orc.libm_f64("log", l64)
        dl = torch.log(torch.from_numpy(l64).cuda()).cpu().numpy()
        assert _ulps(hl, dl).max(initial=0) <= 1
        differ_log += int(np.count_nonzero(hl != dl))
        total += e.size
    record_property("lambda_values", total)
    record_property("exp_disagreements", differ_exp)
    record_property("threshold_disagreements", differ_thresh)
    record_property("log_disagreements", differ_log)
    print(f"\n{total} distinct lambda values: exp differs on {differ_exp}, Knuth threshold on {differ_thresh}, "
          f"log on {differ_log}; all within one ulp")
