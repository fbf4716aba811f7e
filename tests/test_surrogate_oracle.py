"""The surrogate's CPU oracle checked on its own (no GPU): the backward pass against central finite
differences in f64, bf16 rounding, Adam, and the spectrum metric on known signals."""
import numpy as np

from oracle import surrogate_ref as sr


def _net(rng, n_res=2, scale=0.3):
    return dict(w_in=rng.normal(0, scale, (32, 9, 16)), b_in=rng.normal(0, 0.1, 32),
                w_res=rng.normal(0, scale / 3, (n_res, 32, 9, 32)), b_res=rng.normal(0, 0.1, (n_res, 32)),
                w_out=np.concatenate([rng.normal(0, scale, (1, 9, 32)), np.zeros((7, 9, 32))]),
                b_out=rng.normal(0, 0.1, 8))


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    net = _net(rng)
    x = np.zeros((2, 5, 6, 16))
    x[..., :3] = rng.normal(0, 1, (2, 5, 6, 3))
    u = rng.uniform(0, 1, (2, 5, 6))
    t = rng.uniform(0, 1, (2, 5, 6))
    y, cache = sr.forward(x, u, net, bf16=False)
    loss, grads = sr.backward(y, t, cache, net, bf16=False)

    def loss_at(n2):
        y2, _ = sr.forward(x, u, n2, bf16=False)
        return float(np.mean((y2 - t) ** 2))

    assert abs(loss - loss_at(net)) < 1e-12
    checked = 0
    for name in ("w_in", "b_in", "w_res", "b_res", "w_out", "b_out"):
        flat = net[name].reshape(-1)
        g = grads[name].reshape(-1)
        idx = rng.choice(flat.size, size=min(6, flat.size), replace=False)
        if name == "w_in":  # include used input channels
            idx = np.concatenate([idx, [0, 1, 2, 16 * 4 + 1]])
        if name in ("w_out", "b_out"):
            idx = np.concatenate([idx[:3], [0, 5]])
        for i in idx:
            h = 1e-6
            n_p = {k: v.copy() for k, v in net.items()}
            n_m = {k: v.copy() for k, v in net.items()}
            n_p[name].reshape(-1)[i] += h
            n_m[name].reshape(-1)[i] -= h
            fd = (loss_at(n_p) - loss_at(n_m)) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (name, i, fd, g[i])
            checked += 1
    assert checked >= 30


def test_bf16_round_ties_to_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e-3], np.float32)
    r = sr.bf16_round(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even (mantissa 0)
    assert r[2] == np.float32(1.0 + 4 * 2 ** -8)  # tie -> even (rounds up)
    assert r[3] == 1.0
    assert r[4] == -2.5
    assert abs(r[5] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def test_adam_first_step_moves_by_lr():
    w = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -1e-3, 0.0])
    w2, m, v = sr.adam(w, np.zeros(3), np.zeros(3), g, 1, lr=1e-3)
    # the bias-corrected first step is lr * sign(g) (up to eps) and 0 where g = 0
    assert np.allclose(w2, w - 1e-3 * np.sign(g), atol=1e-8)


def test_raps_of_known_signals():
    n = 64
    yy, xx = np.mgrid[0:n, 0:n]
    cosine = np.cos(2 * np.pi * 5 * xx / n)
    p = sr.raps(cosine)
    assert p.shape == (n // 2,)
    assert np.argmax(p) == 4          # radius 5 -> bin index 4
    assert p[4] > 1e3 * np.delete(p, 4).max()
    rng = np.random.default_rng(0)
    white = sr.raps(rng.normal(0, 1, (256, 256)))
    # white noise: flat spectrum with mean power n^2 * variance
    assert abs(white[8:].mean() / (256 * 256) - 1.0) < 0.05
    assert np.allclose(sr.raps(np.full((16, 16), 3.0)), 0.0)


def _sg():
    import pytest
    torch = pytest.importorskip("torch")
    from film_grain_gb300 import surrogate
    return torch, surrogate


def test_radial_power_of_white_noise_and_gradient():
    """White noise of variance v has radial power h*w*v in every bin; the binning-matrix path and the
    bin-sum path (large planes) agree; the power is differentiable through the FFT."""
    torch, sg = _sg()
    g = torch.Generator().manual_seed(1)
    x = torch.randn(8, 64, 64, generator=g, dtype=torch.float64) * 0.5
    p = sg.radial_power(x, 40)
    assert abs(float(p[:, 4:].mean()) / (64 * 64 * 0.25) - 1.0) < 0.05
    big = torch.randn(1, 512, 512, generator=g, dtype=torch.float64)
    pb = sg.radial_power(big, 200)  # bin-sum path
    assert abs(float(pb[0, 8:].mean()) / (512 * 512) - 1.0) < 0.05
    # one small image through both paths: the bin-sum path equals the matrix path bin for bin
    m = sg.radial_power(x[:1], 30)
    sg._BINS[(64, 64, 30, str(x.device))] = None
    key = (64, 64, 30, str(x.device))
    fy = torch.fft.fftfreq(64, dtype=torch.float64) * 64
    r = torch.round(torch.sqrt(fy[:, None] ** 2 + fy[None, :] ** 2)).long().flatten()
    sg._BINS[key] = r
    assert torch.allclose(sg.radial_power(x[:1], 30), m, rtol=1e-10)
    del sg._BINS[key]
    y = x.clone().requires_grad_(True)
    sg.radial_power(y, 10).sum().backward()
    assert float(y.grad.abs().sum()) > 0


def test_expected_render_weights():
    """The expectation filter is the box-integrated Gaussian: it keeps constants, spreads a single bright
    pixel by Phi((d + 1/2)/sigma) - Phi((d - 1/2)/sigma) per axis, and replicates the edges."""
    import math
    torch, sg = _sg()
    u = torch.full((1, 16, 16), 0.3, dtype=torch.float64)
    assert torch.allclose(sg.expected_render(u), u)
    d = torch.zeros((1, 17, 17), dtype=torch.float64)
    d[0, 8, 8] = 1.0
    e = sg.expected_render(d)
    phi = lambda z: 0.5 * (1.0 + math.erf(z / math.sqrt(2.0)))
    w1 = (phi(1.5 / 0.8) - phi(0.5 / 0.8))
    w0 = (phi(0.5 / 0.8) - phi(-0.5 / 0.8))
    tot = sum(phi((k + 0.5) / 0.8) - phi((k - 0.5) / 0.8) for k in range(-4, 5))
    assert abs(float(e[0, 8, 9]) - w0 * w1 / tot ** 2) < 1e-12
    assert abs(float(e.sum()) - 1.0) < 1e-12


def test_grain_radius_and_band_error():
    """The lognormal radius maps to the constant radius of equal E[r^4]/E[r^2] (checked by sampling);
    grain_band_error is 0 for identical grain, about 1 for a prediction without grain, and the Monte
    Carlo floor of a plain render is removed before the comparison."""
    import numpy as np
    torch, sg = _sg()
    m, s = 0.025, 0.01
    s2 = np.log(1.0 + (s / m) ** 2)
    r = np.random.default_rng(2).lognormal(np.log(m) - s2 / 2, np.sqrt(s2), 2_000_000)
    assert abs(sg.grain_radius(m, s, lognormal=True) / np.sqrt(np.mean(r ** 4) / np.mean(r ** 2)) - 1.0) < 0.01
    assert sg.grain_radius(0.1) == 0.1
    g = torch.Generator().manual_seed(3)
    u = torch.full((4, 64, 64), 0.5, dtype=torch.float64)
    grain = sg.expected_render(torch.randn(4, 64, 64, generator=g, dtype=torch.float64)) * 0.2
    ref = u + grain
    assert sg.grain_band_error(ref, ref, u, None, None) == 0.0
    assert abs(sg.grain_band_error(u, ref, u, None, None) - 1.0) < 1e-9
    # a plain render at N = 64 carries white Monte Carlo noise of variance f (1 - f) / N on top: with the
    # floor removed its grain matches; without, the noise counts as grain
    noisy = ref + torch.randn(4, 64, 64, generator=g, dtype=torch.float64) * np.sqrt(0.25 / 64)
    with_floor = sg.grain_band_error(noisy, ref, u, 64, None, fmax=0.5)
    without = sg.grain_band_error(noisy, ref, u, None, None, fmax=0.5)
    assert with_floor < 0.1 and without > 2.0 * with_floor, (with_floor, without)
