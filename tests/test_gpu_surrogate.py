"""The surrogate's kernels against the CPU oracle (oracle/surrogate_ref.py), and what training gains.

Tolerances: the device and the oracle store the same tensors in bf16 at the same points and both
accumulate in f32, but in different orders, so a value within rounding distance of a bf16 boundary can
round to the neighbouring bf16 (one part in 256) and carry that into later layers.  Outputs are
therefore compared by max abs error (forward) and by relative L2 norm per gradient tensor (backward),
with the bounds stated in each test.
"""
import numpy as np
import pytest

from oracle import surrogate_ref as sr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg(cuda, fgl):
    from film_grain_gb300 import surrogate
    return surrogate


def _random_net(sg, torch, n_res=3, seed=1):
    net = sg.SurrogateNet(n_res=n_res, seed=seed)
    rng = np.random.default_rng(seed + 100)
    w = net.w32.cpu().numpy()
    net._np_view(w, "w_in")[:, :, :3] = rng.normal(0, 0.4, (32, 9, 3))
    net._np_view(w, "w_res")[:] = rng.normal(0, 0.06, (n_res, 32, 9, 32))
    net._np_view(w, "w_out")[0] = rng.normal(0, 0.05, (9, 32))
    net._np_view(w, "b_in")[:] = rng.normal(0, 0.1, 32)
    net._np_view(w, "b_res")[:] = rng.normal(0, 0.05, (n_res, 32))
    net._np_view(w, "b_out")[0] = 0.01
    net.w32.copy_(torch.from_numpy(w))
    net.wbf.copy_(net.w32.to(torch.bfloat16))
    net.ema.copy_(net.w32)
    return net


def _inputs(torch, nb, h, w, seed=5):
    rng = np.random.default_rng(seed)
    u = rng.uniform(0, 1, (nb, h, w)).astype(np.float32)
    t = np.clip(u + rng.normal(0, 0.1, u.shape), 0, 1).astype(np.float32)
    r = rng.uniform(0.03, 0.2, nb).astype(np.float32)
    return torch.from_numpy(u).cuda(), torch.from_numpy(r).cuda(), torch.from_numpy(t).cuda()


def test_make_input_channels_and_noise(sg, cuda):
    torch = cuda
    net = sg.SurrogateNet(n_res=1)
    u, r, _ = _inputs(torch, 2, 256, 256)
    net.forward(u, r, seed=77, keep=True)
    x = net._workspace(2, 256, 256)["x"].float().cpu().numpy()
    assert np.array_equal(x[..., 0], sr.bf16_round(u.cpu().numpy()))
    want_r = sr.bf16_round(r.cpu().numpy() * np.float32(net.radius_scale))
    assert np.array_equal(x[..., 2], np.broadcast_to(want_r[:, None, None], x[..., 2].shape))
    assert not x[..., 3:].any()
    z = x[..., 1].ravel()
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert abs(np.mean(z ** 4) - 3.0) < 0.1  # Gaussian kurtosis
    net.forward(u, r, seed=77, keep=True)
    assert np.array_equal(net._workspace(2, 256, 256)["x"].float().cpu().numpy(), x)
    net.forward(u, r, seed=78, keep=True)
    assert not np.array_equal(net._workspace(2, 256, 256)["x"].float().cpu().numpy()[..., 1], x[..., 1])


@pytest.mark.parametrize("shape", [(2, 8, 32), (3, 37, 45), (1, 64, 64), (2, 40, 300)])
def test_forward_matches_oracle(sg, cuda, shape):
    """Max abs error of y within 2e-2 (y is O(1); one bf16 step of a hidden activation moves it ~1e-3).
    (2, 40, 300): the residual layers' tensor-core kernel with several 128-pixel column tiles (the last one
    partial) and 16-row strips (the last one partial)."""
    torch = cuda
    nb, h, w = shape
    net = _random_net(sg, torch)
    u, r, _ = _inputs(torch, nb, h, w)
    y = net.forward(u, r, seed=9, keep=True).cpu().numpy()
    x = net._workspace(nb, h, w)["x"].float().cpu().numpy()
    y_ref, _ = sr.forward(x, u.cpu().numpy(), net.numpy_net())
    err = np.abs(y - y_ref).max()
    assert err < 2e-2, err
    assert np.abs(y - u.cpu().numpy()).max() > 0.05  # the network is not the identity here
    y_inf = net.infer(u, r, seed=9).cpu().numpy()
    assert np.array_equal(y_inf.view(np.uint32), y.view(np.uint32)), "fg_sg_infer differs from the layer calls"


@pytest.mark.parametrize("shape", [(2, 16, 32), (2, 19, 41)])
def test_gradients_match_oracle(sg, cuda, shape):
    """Every parameter gradient within 3e-2 relative L2 of the oracle's (bf16 activations, f32 sums)."""
    torch = cuda
    nb, h, w = shape
    net = _random_net(sg, torch)
    u, r, t = _inputs(torch, nb, h, w)
    net.forward(u, r, seed=11, keep=True)
    loss_sum = float(net.backward(u, t).item())
    ws = net._workspace(nb, h, w)
    x = ws["x"].float().cpu().numpy()
    y_ref, cache = sr.forward(x, u.cpu().numpy(), net.numpy_net())
    loss_ref, g_ref = sr.backward(y_ref, t.cpu().numpy(), cache, net.numpy_net())
    assert abs(loss_sum / (nb * h * w) - loss_ref) <= 1e-2 * loss_ref
    g = net.grad.cpu().numpy()
    for name in ("w_in", "b_in", "w_res", "b_res", "w_out", "b_out"):
        got, want = net._np_view(g, name), g_ref[name].astype(np.float32)
        if name == "w_in":  # channels 3..15 of the input are zero: their gradient must be exactly 0
            assert not got[:, :, 3:].any()
            got, want = got[:, :, :3], want[:, :, :3]
        if name in ("w_out", "b_out"):
            assert not got[1:].any(), "unused output channels must get no gradient"
            got, want = got[:1], want[:1]
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel < 3e-2, (name, rel)


def test_adam_matches_oracle(sg, cuda):
    torch = cuda
    net = _random_net(sg, torch, n_res=2)
    u, r, t = _inputs(torch, 2, 16, 32)
    w0 = net.w32.cpu().numpy().astype(np.float64)
    m = np.zeros_like(w0)
    v = np.zeros_like(w0)
    ema = w0.copy()
    for step in (1, 2):
        net.forward(u, r, seed=step, keep=True)
        net.backward(u, t)
        g = net.grad.cpu().numpy().astype(np.float64)
        net.adam_step(lr=1e-3, ema_decay=0.999)
        w0, m, v = sr.adam(w0, m, v, g, step, lr=1e-3, decay=net.decay.cpu().numpy().astype(np.float64))
        d = (1.0 + step) / (10.0 + step)  # the decay's warm-up
        ema = d * ema + (1 - d) * w0
        got = net.w32.cpu().numpy()
        assert np.abs(got - w0).max() < 1e-6
        assert np.abs(net.ema.cpu().numpy() - ema).max() < 1e-6
        assert np.array_equal(net.wbf.float().cpu().numpy(), sr.bf16_round(got))


def test_checkpoint_resume(sg, cuda, tmp_path):
    torch = cuda
    net = _random_net(sg, torch, n_res=2)
    u, r, t = _inputs(torch, 4, 32, 32)
    for s in range(3):
        net.train_step(u, r, t, seed=s)
    path = str(tmp_path / "ck.npz")
    net.save(path)
    net2 = sg.SurrogateNet.load(path)
    assert net2.step == 3
    for a, b in ((net.w32, net2.w32), (net.wbf, net2.wbf), (net.m, net2.m), (net.v, net2.v), (net.ema, net2.ema)):
        assert torch.equal(a, b)
    # the gradient sums are float atomics, so the next step agrees to rounding, not bit for bit
    net.train_step(u, r, t, seed=3)
    net2.train_step(u, r, t, seed=3)
    torch.cuda.synchronize()
    assert torch.allclose(net.w32, net2.w32, rtol=0, atol=1e-6)
    assert torch.allclose(net.m, net2.m, rtol=1e-3, atol=1e-7)


def test_training_gains_over_no_network(sg, cuda):
    """A short grain-training run on plain N=256 renders of tiles (constant and lognormal radii), scored
    on held-out tiles.
    (a) With its noise weights zeroed the network predicts the expected render (the mean of 16
        independently seeded N=1024 renders: a single render carries a grain realisation and MC noise no
        predictor can know) with less than half the MAE of the method without a network (the intensity u
        itself) and of the untrained network, and beats the plain render at N=16.
    (b) With its noise input it renders grain: the spectrum of its residual against the expectation over
        1/64 .. 1/4 cycles/px is within half the error of u's (u has no grain) from the grain of a plain
        N=1024 render."""
    torch = cuda
    u_tr, r_tr, sd_tr, rn_tr = sg.training_set(4096, seed=1)
    t_tr = sg.render_tiles(u_tr, r_tr, n_samples=256, seed=1, radius_sd=sd_tr)
    u_te, r_te, sd_te, rn_te = sg.training_set(128, seed=99)
    refs = [sg.render_tiles(u_te, r_te, n_samples=1024, seed=99 + k, radius_sd=sd_te) for k in range(16)]
    ref = sum(refs) / 16
    low = sg.render_tiles(u_te, r_te, n_samples=16, seed=123, radius_sd=sd_te)
    ut, rt = torch.from_numpy(u_tr).cuda(), torch.from_numpy(rn_tr).cuda()
    ue, re = torch.from_numpy(u_te).cuda(), torch.from_numpy(rn_te).cuda()
    net = sg.SurrogateNet(n_res=8, seed=0)
    mae_untrained = float((net.infer(ue, re, seed=5, grain=False) - ref).abs().mean())
    hist = sg.train(net, ut, rt, t_tr, steps=2000, batch=64, lr=1e-3, seed=0, log_every=500, log=lambda s: None,
                    grain_n=256)
    net.use_ema()
    mae_net = float((net.infer(ue, re, seed=5, grain=False) - ref).abs().mean())
    mae_id = float((ue - ref).abs().mean())
    mae_low = float((low - ref).abs().mean())
    floor = float((refs[0] - refs[1]).abs().mean()) / np.sqrt(2)  # one N=1024 render's own deviation
    gb_net = sg.grain_band_error(net.infer(ue, re, seed=5), refs[0], ue, None, 1024)
    gb_id = sg.grain_band_error(ue, refs[0], ue, None, 1024)
    print(f"MAE vs mean of 16 N=1024 renders: trained {mae_net:.4f}, identity {mae_id:.4f}, "
          f"untrained {mae_untrained:.4f}, plain N=16 {mae_low:.4f}, single N=1024 render {floor:.4f}; "
          f"grain-band error vs an N=1024 render: trained {gb_net:.3f}, identity {gb_id:.3f}; train {hist}")
    assert mae_net < 0.5 * mae_id
    assert mae_net < 0.5 * mae_untrained
    assert mae_net < mae_low
    assert gb_net < 0.5 * gb_id


def test_evaluator_matches_oracle(sg, cuda):
    """The device spectrum metric (torch FFT) against the numpy oracle, and MAE / spectrum error on
    known pairs."""
    torch = cuda
    rng = np.random.default_rng(4)
    img = rng.normal(0, 1, (96, 128)).astype(np.float32) + np.linspace(0, 3, 128, dtype=np.float32)[None, :]
    got = sg.raps(torch.from_numpy(img).cuda()).cpu().numpy()
    want = sr.raps(img)
    assert np.allclose(got, want, rtol=1e-9, atol=1e-9 * want.max())
    a = torch.from_numpy(img).cuda()
    e = sg.evaluate(a, a)
    assert e["mae"] == 0.0 and e["raps_max"] < 1e-12  # the device bin sums are atomics: order-dependent
    e = sg.evaluate(a + 0.5, a)  # a constant offset changes the MAE but not the spectrum of (img - mean)
    assert abs(e["mae"] - 0.5) < 1e-6 and e["raps_max"] < 1e-6  # f32 rounding of img + 0.5
    e = sg.evaluate(2 * a, a)  # doubling the image quadruples its power
    assert abs(e["raps_max"] - 3.0) < 1e-9
