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
