"""The batched persistent kernel: every image of a mixed batch equals its per-image render, bit for bit."""
import numpy as np
import pytest

from film_grain_gb300 import workloads

pytestmark = pytest.mark.gpu


def _images(fgl, torch, specs):
    images, want = [], []
    for sp in specs:
        plane = workloads.blobs_plane(sp["w"], sp["h"], sp["image_seed"])
        p = fgl.ParamsBuilder(radius_mean=sp["radius"], n_samples=sp["n"], seed=sp["seed"], zoom=sp.get("zoom", 1.0),
                              radius_dist=sp.get("dist", fgl.RadiusDist.Const),
                              radius_stddev=sp.get("sd", 0.0)).build()
        d = fgl.derive_common(p, (sp["w"], sp["h"]))
        lam = fgl.lambda_plane(fgl.normalize_plane(plane)[0], d.inv_e_pi_r2)
        algo = fgl.choose_algorithm(p, d) if sp.get("algo") is None else sp["algo"]
        render = fgl.render_pixelwise if algo == fgl.Algo.Pixel else fgl.render_grainwise
        want.append(render(lam, p, d))
        images.append((torch.from_numpy(lam).cuda(), p, d, algo, lam))
    return images, want


SPECS = [
    dict(w=64, h=48, radius=0.1, n=16, seed=1, image_seed=11),                      # auto -> pixel
    dict(w=96, h=96, radius=0.2, n=256, seed=2, image_seed=12),                     # auto -> grain
    dict(w=40, h=70, radius=0.05, n=64, seed=3, image_seed=13, zoom=1.5),
    dict(w=128, h=128, radius=0.025, n=16, seed=4, image_seed=14),
    dict(w=80, h=60, radius=0.05, n=37, seed=5, image_seed=15, dist=1, sd=0.025, algo=1),
    dict(w=33, h=17, radius=0.1, n=200, seed=6, image_seed=16, zoom=2.0),
    dict(w=70, h=50, radius=0.1, n=24, seed=7, image_seed=17, algo=2, zoom=0.5),
    dict(w=1, h=1, radius=0.1, n=8, seed=8, image_seed=18, algo=1),
]


def test_batch_matches_per_image(cuda, fgl):
    torch = cuda
    images, want = _images(fgl, torch, SPECS)
    b = fgl.Batch(images)
    # zeroing, per-sample, lean, persistent and epilogue kernels
    assert b.kernel_count == 5
    for _ in range(2):  # two replays of the captured graph
        b.run()
        torch.cuda.synchronize()
        for k, (out, w) in enumerate(zip(b.outputs, want)):
            got = out.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), w.view(np.uint32)), f"image {k} differs"
    b.close()


def test_batch_autotune_and_tuned_batch(cuda, fgl):
    torch = cuda
    images, want = _images(fgl, torch, SPECS[:4])
    best, ms = fgl.Batch.autotune(images)
    assert ms > 0 and best.ctas_per_sm >= 1 and best.grain_mask_words >= 1024
    b = fgl.Batch(images, best)
    b.run()
    torch.cuda.synchronize()
    for out, w in zip(b.outputs, want):
        assert np.array_equal(out.cpu().numpy().view(np.uint32), w.view(np.uint32))
    assert b.tuning.grain_mask_words == best.grain_mask_words
    b.close()


def test_batch_of_sweep_images_matches_oracle_tiles(cuda, fgl, orc):
    """Images of the uneven 64-image sweep (workloads.batched_sweep(64, 7): blob planes of 128^2 to
    2048^2, radius 0.025-0.2, N 16-256) -- the first of each (size, algorithm) pair, up to ten --
    rendered together in one batch and checked bit for bit on tiles that the oracle renders exactly
    (a corner, the centre and the brightest region of each image)."""
    torch = cuda
    chosen, seen = [], set()
    for sp in workloads.batched_sweep(64, seed=7):
        p = fgl.ParamsBuilder(radius_mean=sp["radius"], n_samples=sp["n"], seed=sp["seed"]).build()
        d = fgl.derive_common(p, (sp["size"], sp["size"]))
        algo = fgl.choose_algorithm(p, d)
        if (sp["size"], algo) in seen:
            continue
        seen.add((sp["size"], algo))
        plane = workloads.blobs_plane(sp["size"], sp["size"], sp["image_seed"])
        lam = fgl.lambda_plane(fgl.normalize_plane(plane)[0], d.inv_e_pi_r2)
        chosen.append((sp, p, d, algo, lam))
    chosen = chosen[:10]
    assert {c[3] for c in chosen} == {fgl.Algo.Pixel, fgl.Algo.Grain}
    images = [(torch.from_numpy(lam).cuda(), p, d, algo, lam) for sp, p, d, algo, lam in chosen]
    b = fgl.Batch(images)
    b.run()
    torch.cuda.synchronize()
    for k, (sp, p, d, algo, lam) in enumerate(chosen):
        out = b.outputs[k].cpu().numpy()
        size, t = sp["size"], min(32, sp["size"])
        op = orc.params_struct("const", sp["radius"], 0.0, 1.0, 0.8, sp["n"], sp["seed"])
        od, offs, offs_in = orc.derive(op, size, size)
        iy, ix = np.unravel_index(int(np.argmax(lam)), lam.shape)
        for x0, y0 in ((0, 0), (size // 2 - t // 2, size // 2 - t // 2), (min(ix, size - t), min(iy, size - t))):
            name = "pixel" if algo == fgl.Algo.Pixel else "grain"
            want, _ = orc.render(name, lam, op, od, offs_in if name == "pixel" else offs,
                                 rect=(x0, y0, x0 + t, y0 + t))
            got = out[y0:y0 + t, x0:x0 + t]
            diff = np.count_nonzero(got.view(np.uint32) != want.view(np.uint32))
            assert diff == 0, f"image {k} ({size}^2 {name}, r {sp['radius']}, N {sp['n']}) tile ({x0},{y0}): {diff} differ"
    b.close()
