"""Benchmark of the GB300 film-grain integrators (one JSON line on rank 0).

Default workload (``--workload pixel_rgb_4096``, the largest single-GPU configuration): plain
pixel-wise, RGB, 4096x4096x3 f32 input of 16 seeded Gaussian blobs per channel over a 0.1 background,
lognormal grain radius mean 0.025 px / std 0.01, filter sigma 0.8, N = 256, zoom 1.  A step renders one
frame (three planes).  Metric: MC samples/s = output pixels x channels x N per second.

- ``value``: the three pixel-wise render calls per step on device-resident lambda planes (HBM), timed
  with CUDA events around exactly K steps, L2 flushed (256 MiB write) before every step.
- ``e2e``: the same frame through the public C-ABI entry point fg_render_image from pinned host f32 RGB
  to pinned host u8 RGB (host colour split, lambda planes, H2D, kernels, fused colour, D2H).
- ``roofline``: SM instruction issue (this path is integer/f32 ALU work: no dense contraction, almost
  no HBM traffic).  achieved = algorithmic lane-ops per launch / the launch's CUDA-event duration; the
  lane-op count is a model of a minimal exact implementation (PW_COST / GW_COST below) evaluated on
  quantities of the same frame; peak = SMs x 128 lanes x the SM clock sampled during the run.
- ``cpu_baseline``: the CPU oracle (a C restatement of the reference's integrator, OpenMP over output
  rows as the reference's rayon loop) timed on a band of output rows of the same frame.
- ``configs``: the other benchmark configurations, each measured the same way with fewer steps
  (default run at one GPU only): the 256^2 luma pixel-wise ramp, the 1024^2 x 3 -> 2048^2 x 3
  grain-wise frame, the uneven 64-image sweep (batched graph vs per-image launches) and the surrogate
  against the plain method on the 4096^2 x 3 frame.
- ``--impl reference``: that CPU oracle alone, all host threads, each step one band.

Multi-GPU (torchrun): every rank renders its own frame (replicas, weak scaling); value = all ranks'
samples / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "grain_rgb_1024": dict(desc="plain grain-wise RGB 1024x1024x3 -> 2048x2048x3, lognormal r 0.05/0.025, N 128, zoom 2",
                           w=1024, h=1024, mode="rgb", algo="grain", radius=0.05, dist="lognorm", sd=0.025, zoom=2.0,
                           n=128, seed=42, image_seed=0),
    "pixel_luma_256": dict(desc="plain pixel-wise luma 256x256 ramp+noise, const r 0.12, N 64, zoom 1, seed 42",
                           w=256, h=256, mode="luma", algo="pixel", radius=0.12, dist="const", sd=0.0, zoom=1.0, n=64,
                           seed=42, image_seed=42),
    "grain_rgb_512": dict(desc="profiling case: grain-wise RGB 512x512x3 blobs, lognormal r 0.05/0.025, N 128, zoom 2",
                          w=512, h=512, mode="rgb", algo="grain", radius=0.05, dist="lognorm", sd=0.025, zoom=2.0,
                          n=128, seed=42, image_seed=0),
    "pixel_rgb_1024": dict(desc="profiling case: pixel-wise RGB 1024x1024x3 blobs, lognormal r 0.025/0.01, N 256",
                           w=1024, h=1024, mode="rgb", algo="pixel", radius=0.025, dist="lognorm", sd=0.01, zoom=1.0,
                           n=256, seed=42, image_seed=1),
    "grain_luma_512_saturated": dict(desc="profiling case: grain-wise luma 512x512 saturated plane (u = 1), const r "
                                          "0.025, N 256, zoom 1 (about 7000 grains per pixel)",
                                     w=512, h=512, mode="luma", algo="grain", radius=0.025, dist="const", sd=0.0,
                                     zoom=1.0, n=256, seed=42, image_seed=0, source="flat", level=1.0),
    "pixel_luma_2048_sparse": dict(desc="profiling case: pixel-wise luma 2048x2048 blobs, const r 0.025, N 64, zoom 1 "
                                        "(the per-sample kernel)",
                                   w=2048, h=2048, mode="luma", algo="pixel", radius=0.025, dist="const", sd=0.0,
                                   zoom=1.0, n=64, seed=42, image_seed=5, source="blobs"),
    "pixel_luma_1024_flat": dict(desc="profiling case: pixel-wise luma 1024x1024 flat plane u = 0.13 (the 4096^2 "
                                      "frame's background), lognormal r 0.025/0.01, N 256, zoom 1",
                                 w=1024, h=1024, mode="luma", algo="pixel", radius=0.025, dist="lognorm", sd=0.01,
                                 zoom=1.0, n=256, seed=42, image_seed=0, source="flat", level=0.13),
    "pixel_rgb_4096": dict(desc="plain pixel-wise RGB 4096x4096x3 blobs, lognormal r 0.025/0.01, N 256, zoom 1",
                           w=4096, h=4096, mode="rgb", algo="pixel", radius=0.025, dist="lognorm", sd=0.01, zoom=1.0,
                           n=256, seed=42, image_seed=1),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def make_input(wl):
    from film_grain_gb300 import workloads
    source = wl.get("source")
    if source == "flat":
        return np.full((wl["h"], wl["w"], 3), wl["level"], np.float32)
    if source == "blobs":
        return workloads.gray_rgb(workloads.blobs_plane(wl["w"], wl["h"], wl["image_seed"]))
    if wl["mode"] == "luma" and wl["algo"] == "pixel":
        return workloads.gray_rgb(workloads.ramp_noise(wl["w"], wl["h"], wl["image_seed"]))
    return workloads.blobs_rgb(wl["w"], wl["h"], wl["image_seed"])


def build_params(fg, wl):
    return fg.ParamsBuilder(radius_mean=wl["radius"],
                            radius_dist=fg.RadiusDist.Lognorm if wl["dist"] == "lognorm" else fg.RadiusDist.Const,
                            radius_stddev=wl["sd"], zoom=wl["zoom"], n_samples=wl["n"], seed=wl["seed"],
                            color_mode=fg.ColorMode.Rgb if wl["mode"] == "rgb" else fg.ColorMode.Luma,
                            algo=fg.Algo.Grain if wl["algo"] == "grain" else fg.Algo.Pixel).build()


def host_planes(rgb, mode):
    """The colour workspace planes the integrators see (load_rgb_workspace / load_luma_workspace)."""
    c = np.clip(rgb, 0.0, 1.0).astype(np.float32)
    if mode == "rgb":
        return [np.ascontiguousarray(c[:, :, i]) for i in range(3)]
    y = (np.float32(0.2126) * c[:, :, 0] + np.float32(0.7152) * c[:, :, 1]) + np.float32(0.0722) * c[:, :, 2]
    return [np.ascontiguousarray(np.clip(y, 0.0, 1.0).astype(np.float32))]


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.idx = gpu_index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_grain_baseline(oracle, planes, wl, threads, band_rows=None, bands=1, count=True):
    """Time the oracle on `bands` input-row bands per plane (4 rows per host thread, so every thread
    of the row-parallel loop is busy); extrapolate to the frame by grain count.
    Returns (samples_per_s, seconds_measured, sample description, per-plane work counts)."""
    band_rows = band_rows or 4 * threads
    p = oracle.params_struct(wl["dist"], wl["radius"], wl["sd"], wl["zoom"], 0.8, wl["n"], wl["seed"])
    h, w = planes[0].shape
    d, offs, _ = oracle.derive(p, w, h)
    frame_samples = d.out_w * d.out_h * len(planes) * wl["n"]
    t_frame, t_meas, counts = 0.0, 0.0, []
    bits = np.zeros(d.out_w * d.out_h * ((wl["n"] + 63) // 64), np.uint64)
    for ci, plane in enumerate(planes):
        lam = oracle.lambda_plane(oracle.normalize_plane(plane)[0], d.inv_e_pi_r2)
        g_full = oracle.grain_total(lam, p, d, threads=threads)
        g_band, t_band, st_tot = 0, 0.0, np.zeros(4, np.uint64)
        for b in range(bands):
            y0 = int((b + 0.5) * h / bands) - band_rows // 2
            if count:
                st, _ = oracle.grainwise_rows(lam, p, d, offs, (y0, y0 + band_rows), count=True, threads=threads,
                                              bits=bits)
                st_tot += st
            t0 = time.perf_counter()
            st, _ = oracle.grainwise_rows(lam, p, d, offs, (y0, y0 + band_rows), count=False, threads=threads,
                                          bits=bits)
            t_band += time.perf_counter() - t0
            g_band += int(st[0])
        t_meas += t_band
        t_frame += t_band * g_full / max(1, g_band)
        gb = max(1, int(st_tot[0]))
        counts.append(dict(grains=g_full, px_per_grain=float(st_tot[1]) / gb, py_per_grain=float(st_tot[2]) / gb,
                           hits_per_grain=float(st_tot[3]) / gb))
    desc = (f"{bands} bands x {band_rows} input rows per plane ({len(planes)} planes) through the reference's full "
            f"grain-wise loop; frame time extrapolated by grain count")
    return frame_samples / t_frame, t_meas, desc, counts


def cpu_pixel_baseline(oracle, planes, wl, threads, rows=None):
    p = oracle.params_struct(wl["dist"], wl["radius"], wl["sd"], wl["zoom"], 0.8, wl["n"], wl["seed"])
    h, w = planes[0].shape
    d, offs, offs_in = oracle.derive(p, w, h)
    lam = oracle.lambda_plane(oracle.normalize_plane(planes[0])[0], d.inv_e_pi_r2)
    r = rows or d.out_h
    y0 = max(0, d.out_h // 2 - r // 2)
    t0 = time.perf_counter()
    oracle.render("pixel", lam, p, d, offs_in, rect=(0, y0, d.out_w, y0 + r), threads=threads)
    dt = time.perf_counter() - t0
    samples = d.out_w * r * wl["n"]
    return samples / dt, dt, f"output rows {y0}..{y0 + r} of plane 0 ({samples} samples)", None


# DRAM bytes per launch from ncu captures of the dominant kernels on their profiling cases (the
# --profile-once runs), per unit of work: sg_conv32_tc_kernel (the residual conv) on the 1024^2 x 3
# surrogate input, 373.9 MB read+write for 3 x 1024^2 px; grainwise_persistent_kernel on a 512^2 ->
# 1024^2 plane of the grain-wise blob frame, 18.25 MB per 1024^2 output pixels (the lambda plane plus the
# sample-mask lines that miss L2); cell_mask_kernel + pixelwise_sparse_kernel on the 1024^2 flat plane
# of the large frame's parameters, 170.3 + 247.6 MB per 1024^2 output pixels (the emptiness bitmask
# written, then read with the cell table).
SG_CONV_DRAM_BYTES_PER_PX = 373.9e6 / (3 * 1024 * 1024)
GRAINWISE_DRAM_BYTES_PER_OUT_PX = 18.25e6 / (1024 * 1024)
PIXELWISE_DRAM_BYTES_PER_OUT_PX = (170.3e6 + 247.6e6) / (1024 * 1024)

# Algorithmic lane-ops of the pixel-wise path (an exact method that hashes every cell once): per cell
# its hash and first uniform (~65: the row stage of mix3, one SplitMix64, ~24; the four PCG32 seed words
# that the first xoshiro256++ output needs, ~8 each; that output and the threshold compare, ~9), per
# non-empty cell the Knuth continuation (~60), per grain its generation (150 lognormal / 70 const), per
# sample its point and cell range (~30), and ~8 per disk test, a sample testing the grains of its cell
# range until the first hit (all of them when uncovered, half on average when covered).  Expectations
# from the lambda plane.
PW_COST = dict(cell=65, nonempty=60, grain_lognorm=150, grain_const=70, sample=30, test=8)


def pixelwise_lane_ops(lam, wl, derived, out_px):
    lam = lam.astype(np.float64)
    d, rm = float(derived.delta), float(derived.rm)
    h, w = lam.shape
    cells = (w + 2 * rm) * (h + 2 * rm) / (d * d)
    nonempty = float(np.sum(1.0 - np.exp(-lam * d * d))) / (d * d)
    grains = float(lam.sum())
    samples = float(out_px) * wl["n"]
    u = 1.0 - np.exp(-lam / float(derived.inv_e_pi_r2))
    tests = samples * float(np.mean(lam * (2 * rm + d) ** 2 * (1.0 - u / 2)))
    c_g = PW_COST["grain_lognorm"] if wl["dist"] == "lognorm" else PW_COST["grain_const"]
    terms = dict(cells=cells, nonempty_cells=nonempty, grains=grains, samples=samples, tests=tests)
    terms["total"] = (PW_COST["cell"] * cells + PW_COST["nonempty"] * nonempty + c_g * grains +
                      PW_COST["sample"] * samples + PW_COST["test"] * tests)
    return terms


# The per-sample path (planes whose samples reach fewer cells than a staged window): every sample
# decides emptiness for the cells of its range (hash + threshold) and regenerates the non-empty ones
# until a grain covers it.  Minimal lane-ops: a sample's set-up, one emptiness test per cell of its
# range, and a Poisson draw plus the grains' generation and disk tests for each non-empty cell; the
# early exit is credited as half the non-empty cells of a covered sample.
PW_REGEN_COST = dict(sample=40, cell=65, nonempty=60, grain=30)


def pixelwise_regen_lane_ops(lam, wl, derived, out_px):
    lam = lam.astype(np.float64)
    d, rm = float(derived.delta), float(derived.rm)
    cells = (2.0 * rm / d + 1.0) ** 2  # cells of one sample's range
    samples = float(out_px) * wl["n"]
    p_ne = float(np.mean(1.0 - np.exp(-lam * d * d)))
    u = float(np.mean(1.0 - np.exp(-lam / float(derived.inv_e_pi_r2))))
    nonempty = samples * cells * p_ne * (1.0 - u / 2)
    grains = samples * cells * float(np.mean(lam * d * d)) * (1.0 - u / 2)
    terms = dict(samples=samples, cells=samples * cells, nonempty_cells=nonempty, grains=grains)
    terms["total"] = (PW_REGEN_COST["sample"] * samples + PW_REGEN_COST["cell"] * samples * cells +
                      PW_REGEN_COST["nonempty"] * nonempty + PW_REGEN_COST["grain"] * grains)
    return terms


# Algorithmic lane-ops of the grain-wise path: the lane-op counts of a minimal exact implementation.
# A grain: three xoshiro steps (~18 each), two uniforms (5 each), and for a lognormal radius the
# ziggurat normal (~12) and a double-float exp (~70), plus clamps (~10): 150 (70 for a constant
# radius).  A pair whose x bounds are tested: 2 adds, 2 subtracts, ceil, floor, 3 compares (10); whose
# y bounds are tested too: 8 more; a centre hit: the disk test and the bit set (12).  Each output
# pixel: its popcount pass (3 + 2 per mask word).
GW_COST = dict(grain_lognorm=150, grain_const=70, x_pair=10, y_pair=8, hit=12, out_base=3, out_word=2)


def grainwise_lane_ops(count, wl, out_px):
    words = (wl["n"] + 31) // 32
    g = count["grains"]
    per_grain = GW_COST["grain_lognorm"] if wl["dist"] == "lognorm" else GW_COST["grain_const"]
    return (g * (per_grain + GW_COST["x_pair"] * count["px_per_grain"] + GW_COST["y_pair"] * count["py_per_grain"] +
                 GW_COST["hit"] * count["hits_per_grain"]) + out_px * (GW_COST["out_base"] + GW_COST["out_word"] * words))


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def surrogate_compare(fg, sg, net, steps, warmup, plain_steps, clocks=None, seed=7):
    """The large frame (4096^2 x 3 blob family, lognormal r 0.025/0.01, sigma 0.8): the surrogate's
    ms/frame against the plain pixel-wise render at N=256, both on device-resident inputs with a 256 MiB
    L2 flush before every frame, and both scored (MAE, spectrum error) against a plain render at N=1024
    with another seed.  Returns a dict of the measurements."""
    import torch
    from film_grain_gb300 import workloads
    wl = WORKLOADS["pixel_rgb_4096"]
    size = wl["w"]
    planes = host_planes(workloads.blobs_rgb(size, size, wl["image_seed"]), "rgb")
    u_host = np.stack([fg.normalize_plane(p)[0] for p in planes])
    u_dev = torch.from_numpy(u_host).cuda()
    # the lognormal radius as the constant radius of equal grain power (the network's training radii are
    # constant)
    radius = torch.full((3,), sg.grain_radius(wl["radius"], wl["sd"], lognormal=True), dtype=torch.float32,
                        device="cuda")
    y = torch.empty_like(u_dev)
    L = fg.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def plain(n_samples, pseed, out):
        p = fg.ParamsBuilder(radius_mean=wl["radius"], radius_dist=fg.RadiusDist.Lognorm, radius_stddev=wl["sd"],
                             n_samples=n_samples, seed=pseed, algo=fg.Algo.Pixel).build()
        d = fg.derive_common(p, (size, size))
        lam = [torch.from_numpy(fg.lambda_plane(u_host[c], d.inv_e_pi_r2)).cuda() for c in range(3)]
        offs = np.ascontiguousarray(d.offsets_input, np.float32)

        def run():
            for c in range(3):
                rc = L.fg_render_pixelwise_async(lam[c].data_ptr(), p.c, d._c, offs.ctypes.data, out[c].data_ptr(), sp)
                if rc != 0:
                    raise RuntimeError(L.fg_last_error_message().decode())
        return run

    def timed(fn, k):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for e0, e1 in evs:
            flush.fill_(1.0)
            e0.record(stream)
            fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return sum(e0.elapsed_time(e1) for e0, e1 in evs) / k

    sur = lambda: net.infer(u_dev, radius, seed=seed, out=y)
    plain256 = torch.empty_like(u_dev)
    run256 = plain(256, wl["seed"], plain256)
    for _ in range(warmup):
        sur()
    run256()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    sur_ms = timed(sur, steps)
    clk = clocks.stop() if clocks else None
    plain_ms = timed(run256, plain_steps)

    # the dominant kernel: the 32 -> 32 residual conv, timed per launch through the layer-by-layer path
    ws = net._workspace(3, size, size, train=False)
    net.forward(u_dev, radius, seed=seed)
    hs = ws["hs"]
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(net.n_res)]
    for l, (e0, e1) in enumerate(evs):
        e0.record(stream)
        net._conv(sg.CONV_RESIDUAL, hs[l % 2], sg.CH, net._ptr(net.wbf, "w_res", l), net._ptr(net.w32, "b_res", l),
                  hs[l % 2], None, hs[(l + 1) % 2], None, None, 3, size, size)
        e1.record(stream)
    torch.cuda.synchronize()
    conv_ms = sum(e0.elapsed_time(e1) for e0, e1 in evs) / len(evs)
    px = 3 * size * size
    conv_flop = px * 9 * sg.CH * sg.CH * 2
    conv_bytes = px * sg.CH * 2 * 2  # read h (the residual is the same tensor), write h'

    ref1024 = torch.empty_like(u_dev)
    plain(1024, wl["seed"] + 1000, ref1024)()
    # the method without the network at the network's cost: plain pixel-wise with N scaled to its time
    n_eq = max(1, int(round(256 * sur_ms / plain_ms)))
    plain_eq = torch.empty_like(u_dev)
    plain(n_eq, wl["seed"], plain_eq)()
    torch.cuda.synchronize()
    q_sur = sg.evaluate(y, ref1024)
    q_plain = sg.evaluate(plain256, ref1024)
    q_eq = dict(sg.evaluate(plain_eq, ref1024), n_samples=n_eq)
    q_id = sg.evaluate(u_dev, ref1024)
    # the same network with its noise input off predicts the expectation instead of a grain realisation
    y_mean = net.infer(u_dev, radius, seed=seed, grain=False)
    q_mean = sg.evaluate(y_mean, ref1024)
    # grain-band spectrum error (radial bins from 1/64 to 1/4 cycles/px of each render's residual against
    # the expectation, Monte Carlo floors of plain renders removed) against the N=1024 render
    grain_band = {"surrogate": sg.grain_band_error(y, ref1024, u_dev, None, 1024),
                  "surrogate_no_noise": sg.grain_band_error(y_mean, ref1024, u_dev, None, 1024),
                  "identity": sg.grain_band_error(u_dev, ref1024, u_dev, None, 1024),
                  "plain_n256": sg.grain_band_error(plain256, ref1024, u_dev, 256, 1024)}

    # end to end: pinned host u planes in, pinned host f32 planes out
    pin_u = torch.from_numpy(u_host).pin_memory()
    pin_y = torch.empty_like(pin_u).pin_memory()
    u_e2e = torch.empty_like(u_dev)

    def e2e():
        u_e2e.copy_(pin_u, non_blocking=True)
        net.infer(u_e2e, radius, seed=seed, out=y)
        pin_y.copy_(y, non_blocking=True)
    for _ in range(warmup):
        e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        e2e()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) / steps * 1e3
    return dict(size=size, sur_ms=sur_ms, plain_ms=plain_ms, conv_ms=conv_ms, conv_flop=conv_flop,
                conv_bytes=conv_bytes, q_sur=q_sur, q_plain=q_plain, q_eq=q_eq, q_id=q_id, q_mean=q_mean,
                grain_band=grain_band, e2e_ms=e2e_ms,
                h2d=4 * px, d2h=4 * px, clocks=clk, launches_per_frame=3 + net.n_res, wl=wl, planes=planes)


def surrogate_line(steps, warmup, world, retrain=False, cpu=True):
    """The surrogate against the plain method on the large frame (4096^2 x 3 blobs): returns the line."""
    import torch
    import film_grain_gb300 as fg
    from film_grain_gb300 import surrogate as sg
    if retrain or not os.path.exists(sg.DEFAULT_WEIGHTS):
        net, info = sg.train_from_scratch(log=log)
        prov = dict(source="trained in this run", **info)
    else:
        net = sg.load_default()
        prov = dict(source="film_grain_gb300/weights/surrogate_c4.npz", **{k: (v.item() if hasattr(v, "item") else v)
                                                                           for k, v in net.meta.items()})
    clocks = ClockSampler(torch.cuda.current_device())
    r = surrogate_compare(fg, sg, net, steps, warmup, plain_steps=min(steps, 3), clocks=clocks)
    peaks, basis = _peaks()
    ach = r["conv_flop"] / (r["conv_ms"] / 1e3) / 1e12
    line = {"metric": "surrogate ms/frame (4096^2 RGB)", "value": r["sur_ms"], "unit": "ms/frame", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": r["sur_ms"], "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (f32 accumulate)",
            "data": "synthetic (seeded blob frame)",
            "config": {"workload": "surrogate_rgb_4096",
                       "description": "4096x4096x3 blob frame, lognormal r 0.025/0.01, sigma 0.8, zoom 1: "
                                      "surrogate vs plain pixel-wise N=256, scored against plain N=1024",
                       "plain_ms_per_frame": r["plain_ms"], "speedup_vs_plain": r["plain_ms"] / r["sur_ms"],
                       "l2": "256 MiB flush write before every frame", "network": prov},
            "quality": {"surrogate_vs_n1024": r["q_sur"], "plain_n256_vs_n1024": r["q_plain"],
                        "plain_equal_time_vs_n1024": r["q_eq"], "identity_vs_n1024": r["q_id"],
                        "surrogate_no_noise_vs_n1024": r["q_mean"],
                        "grain_band_error_vs_n1024": r["grain_band"],
                        "targets": {"mae": 0.01, "raps": 0.02}},
            # the 32 -> 32 residual conv: 18.4 kFLOP and 128 B (64 B in, 64 B out) per pixel, 144 FLOP/B,
            # below the GB300's ridge (bf16 peak / HBM bandwidth): HBM-bound
            "roofline": {"bound": "hbm", "achieved": r["conv_bytes"] / (r["conv_ms"] / 1e3) / 1e9,
                         "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": r["conv_bytes"] / (r["conv_ms"] / 1e3) / (peaks["hbm_gbs"] * 1e9),
                         "traffic": SG_CONV_DRAM_BYTES_PER_PX * 3 * r["size"] ** 2,
                         "traffic_basis": "ncu dram bytes of sg_conv32_tc_kernel on the 1024^2 x 3 surrogate "
                                          "input, scaled by pixels",
                         "kernel": "sg_conv32_tc_kernel (tcgen05, one residual layer of the 4096^2 x 3 frame)",
                         "launch_ms": r["conv_ms"], "flop_per_launch": r["conv_flop"],
                         "algorithmic_bytes_per_launch": r["conv_bytes"], "tensor_tflops": ach,
                         "tensor_frac": ach / peaks["bf16_tflops"], "tensor_peak": peaks["bf16_tflops"],
                         "peak_basis": f"HBM copy and bf16 burst, {basis}"},
            "e2e": {"value": r["e2e_ms"], "unit": "ms/frame", "h2d_bytes_per_step": r["h2d"] + 12,
                    "d2h_bytes_per_step": r["d2h"], "path": "pinned f32 u planes -> fg_sg_infer -> pinned f32 planes"},
            "gpu_launches": steps * r["launches_per_frame"], "clocks": r["clocks"]}
    if cpu:
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        rate, secs, desc, _ = cpu_pixel_baseline(oracle, r["planes"], r["wl"], threads, rows=threads)
        frame = 3 * r["size"] * r["size"] * r["wl"]["n"]
        line["cpu_baseline"] = {"value": frame / rate * 1e3, "unit": "ms/frame", "cores": threads, "kind": "port",
                                "sample": f"plain pixel-wise N=256 oracle on {desc}, extrapolated to the frame",
                                "seconds": secs}
    return line


def batch_line(steps, warmup, world):
    """The uneven sweep: 64 luma images (blob family), sizes over {128..2048}^2, radius over
    {0.025..0.2}, N over {16, 64, 256}, algorithm chosen per image by the crate's Auto rule.  value =
    all images' samples / the autotuned batched graph's time; the per-image launch time is reported,
    and per size class the per-image time of those images alone."""
    import torch
    import film_grain_gb300 as fg
    from film_grain_gb300 import workloads
    L = fg.lib()
    specs = workloads.batched_sweep(64, seed=7)
    images, host_lam, samples = [], [], 0
    for sp in specs:
        plane = workloads.blobs_plane(sp["size"], sp["size"], sp["image_seed"])
        p = fg.ParamsBuilder(radius_mean=sp["radius"], n_samples=sp["n"], seed=sp["seed"]).build()
        d = fg.derive_common(p, (sp["size"], sp["size"]))
        lam = fg.lambda_plane(fg.normalize_plane(plane)[0], d.inv_e_pi_r2)
        algo = fg.choose_algorithm(p, d)
        images.append((torch.from_numpy(lam).cuda(), p, d, algo, lam))
        host_lam.append(lam)
        samples += d.output_width * d.output_height * sp["n"]
    stream = torch.cuda.current_stream()
    sp_ = stream.cuda_stream
    outs = [torch.empty((im[2].output_height, im[2].output_width), device="cuda") for im in images]
    offs = [np.ascontiguousarray(im[2].offsets_input if im[3] == fg.Algo.Pixel else im[2].offsets, np.float32)
            for im in images]

    def per_image(idx=None):
        for k, ((lam, p, d, algo, _), o, of) in enumerate(zip(images, outs, offs)):
            if idx is not None and k not in idx:
                continue
            fn = L.fg_render_pixelwise_async if algo == fg.Algo.Pixel else L.fg_render_grainwise_async
            if fn(lam.data_ptr(), p.c, d._c, of.ctypes.data, o.data_ptr(), sp_) != 0:
                raise RuntimeError(L.fg_last_error_message().decode())

    def timed(fn, k, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    t_per_image = timed(per_image, steps, warmup)
    classes = {}
    for k, sp in enumerate(specs):
        classes.setdefault(sp["size"], []).append(k)
    by_size = {}
    for size, idx in sorted(classes.items()):
        ids = set(idx)
        ms = timed(lambda: per_image(ids), max(1, steps // 2), 1)
        by_size[str(size)] = {"images": len(idx), "per_image_ms": ms,
                              "samples": sum(images[k][2].output_width * images[k][2].output_height * specs[k]["n"]
                                             for k in idx)}
    b_default = fg.Batch(images)
    t_default = timed(b_default.run, steps, warmup)
    b_default.close()
    best, t_tune = fg.Batch.autotune(images)
    b = fg.Batch(images, best)
    for size, idx in sorted(classes.items()):
        sub = fg.Batch([images[k] for k in idx], best)
        by_size[str(size)]["batched_ms"] = timed(sub.run, max(1, steps // 2), 1)
        sub.close()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t_batch = timed(b.run, steps, warmup)
    clk = clocks.stop()
    # end to end: pinned lambda planes in, f32 planes out, around the batched graph
    pin_in = [torch.from_numpy(h).pin_memory() for h in host_lam]
    pin_out = [torch.empty(o.shape, dtype=torch.float32).pin_memory() for o in b.outputs]

    def e2e():
        for (lam, *_), pi in zip(images, pin_in):
            lam.copy_(pi, non_blocking=True)
        b.run()
        for o, po in zip(b.outputs, pin_out):
            po.copy_(o, non_blocking=True)
    t_e2e = timed(e2e, steps, warmup)
    h2d = sum(h.nbytes for h in host_lam)
    d2h = sum(o.numel() * 4 for o in b.outputs)
    line = {"metric": "MC samples/s", "value": samples / (t_batch / 1e3), "unit": "samples/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": t_batch, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64-rng/f32", "data": "synthetic (seeded)",
            "config": {"workload": "batch_sweep_64", "images": len(images),
                       "pixel_images": sum(1 for im in images if im[3] == fg.Algo.Pixel),
                       "frame_samples": samples, "per_image_launch_ms": t_per_image,
                       "batched_default_ms": t_default, "batched_autotuned_ms": t_batch,
                       "speedup_vs_per_image": t_per_image / t_batch, "tuning": repr(best),
                       "autotune_best_ms": t_tune, "by_size": by_size,
                       "l2": "inputs and scratch far larger than L2"},
            "e2e": {"value": samples / (t_e2e / 1e3), "unit": "samples/s", "ms_per_step": t_e2e,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "pinned lambda planes -> fg_batch_run -> pinned f32 planes"},
            "gpu_launches": b.kernel_count * steps, "clocks": clk}
    b.close()
    return line


def replica_max(dist, value, device):
    """The largest of the ranks' values: a barrier, then an all-reduce MAX of one float (the whole job's
    time is its slowest replica's)."""
    import torch
    dist.barrier()
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(samples_per_frame, steps, world, elapsed):
    """Whole-job throughput of `world` replicas that each render `steps` frames, the job's time being the
    slowest replica's `elapsed` seconds."""
    return samples_per_frame * steps * world / elapsed


def plain_line(wl_name, steps, warmup, rank=0, world=1, dist=None, cpu=True, e2e_steps=None):
    """One plain workload (WORKLOADS[wl_name]) through the per-plane render calls: returns the line
    (rank 0) or None (other ranks)."""
    import torch
    import film_grain_gb300 as fg
    wl = WORKLOADS[wl_name]
    L = fg.lib()
    rgb = make_input(wl)
    params = build_params(fg, wl)
    derived = fg.derive_common(params, (wl["w"], wl["h"]))
    planes = host_planes(rgb, wl["mode"])
    lam_host = [fg.lambda_plane(fg.normalize_plane(pl)[0], derived.inv_e_pi_r2) for pl in planes]
    lam_dev = [torch.from_numpy(l).cuda() for l in lam_host]
    ow, oh = derived.output_width, derived.output_height
    outs = [torch.empty((oh, ow), dtype=torch.float32, device="cuda") for _ in planes]
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    offs = np.ascontiguousarray(derived.offsets if wl["algo"] == "grain" else derived.offsets_input, np.float32)
    fn = L.fg_render_grainwise_async if wl["algo"] == "grain" else L.fg_render_pixelwise_async
    # grain: tile costs, tile order, persistent tiles, popcount; pixel: cell table, then the per-sample
    # kernel, or the emptiness bitmask + sparse and fat block passes, or lean + fat block passes; epilogue
    launches_per_plane = 4 if wl["algo"] == "grain" else fg.pixelwise_kernel_count(params, derived)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    ev = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in planes] for _ in range(steps)]

    def step(i=None):
        flush.fill_(1.0)
        for c in range(len(planes)):
            if i is not None:
                ev[i][c][0].record(stream)
            rc = fn(lam_dev[c].data_ptr(), params.c, derived._c, offs.ctypes.data, outs[c].data_ptr(), sp)
            if rc != 0:
                raise RuntimeError(L.fg_last_error_message().decode())
            if i is not None:
                ev[i][c][1].record(stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if clocks:
        clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for i in range(steps):
        step(i)
    t_end.record(stream)
    torch.cuda.synchronize()
    launch_ms = [sum(ev[i][c][0].elapsed_time(ev[i][c][1]) for i in range(steps)) / steps
                 for c in range(len(planes))]  # mean duration of plane c's render call
    elapsed = t_start.elapsed_time(t_end) / 1e3
    if dist:
        elapsed = replica_max(dist, elapsed, "cuda")
    clk = clocks.stop() if clocks else None

    samples_per_frame = ow * oh * len(planes) * wl["n"]
    value = replica_value(samples_per_frame, steps, world, elapsed)
    ms_per_step = elapsed / steps * 1e3

    # ---- end to end through the public entry point, pinned host buffers
    e2e_steps = e2e_steps or steps
    pin_in = torch.from_numpy(rgb).pin_memory()
    pin_out = torch.empty((oh, ow, 3), dtype=torch.uint8).pin_memory()
    st = fg._StatsC()
    e2e_fn = lambda: L.fg_render_image(pin_in.data_ptr(), wl["w"], wl["h"], ctypes.byref(params.c), pin_out.data_ptr(),
                                       ctypes.byref(st), None, sp)
    for _ in range(min(warmup, 3)):
        assert e2e_fn() == 0, L.fg_last_error_message()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        assert e2e_fn() == 0
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = 4 * wl["w"] * wl["h"] * len(planes) + (16 if wl["algo"] == "grain" else 8) * wl["n"]
    if wl["mode"] == "luma":
        h2d += 8 * wl["w"] * wl["h"]
    d2h = 3 * ow * oh

    if rank != 0:
        return None

    line = {"metric": "MC samples/s", "value": value, "unit": "samples/s", "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64-rng/f32", "data": "synthetic (seeded, generated in bench.py)",
            "config": {"workload": wl_name, "description": wl["desc"], "frame_samples": samples_per_frame,
                       "ms_per_frame": ms_per_step, "l2": "256 MiB flush write before every step",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": samples_per_frame / e2e_s, "unit": "samples/s", "ms_per_frame": e2e_s * 1e3,
                    "steps": e2e_steps, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "fg_render_image: pinned f32 RGB in -> pinned u8 RGB out"},
            "gpu_launches": steps * len(planes) * launches_per_plane,
            "clocks": clk}

    # ---- roofline of the dominant kernel and the CPU baseline
    sm_count = torch.cuda.get_device_properties(0).multi_processor_count
    f_mhz = (clk or {}).get("sm_mhz") or 2070.0
    peak = sm_count * 128 * f_mhz * 1e6  # lane-ops/s
    counts = None
    if cpu:
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        if wl["algo"] == "grain":
            cpu_v, cpu_t, desc, counts = cpu_grain_baseline(oracle, planes, wl, threads)
        else:
            cpu_v, cpu_t, desc, _ = cpu_pixel_baseline(oracle, planes, wl, threads,
                                                        rows=None if wl["w"] <= 256 else threads)
        line["cpu_baseline"] = {"value": cpu_v, "unit": "samples/s", "cores": threads, "kind": "port",
                                "sample": desc, "seconds": cpu_t}
    peak_basis = f"{sm_count} SMs x 128 lanes x {f_mhz:.0f} MHz (sampled)"
    if counts and wl["algo"] == "grain":
        ops = [grainwise_lane_ops(c, wl, ow * oh) for c in counts]
        ach = sum(o / (ms / 1e3) for o, ms in zip(ops, launch_ms)) / len(ops)
        line["roofline"] = {"bound": "sm_issue", "achieved": ach / 1e12, "peak": peak / 1e12, "unit": "Tlane-op/s",
                            "frac": ach / peak, "traffic": GRAINWISE_DRAM_BYTES_PER_OUT_PX * ow * oh,
                            "traffic_basis": "ncu dram bytes of grainwise_persistent_kernel on a 512^2 -> 1024^2 "
                                             "plane of the grain-wise blob frame, scaled by output pixels",
                            "kernel": "grainwise_persistent_kernel (launch_ms: the whole plane)", "launch_ms": launch_ms,
                            "lane_ops_per_launch": ops, "counts": counts, "peak_basis": peak_basis}
    if wl["algo"] == "pixel" and launches_per_plane == 3:
        ops = [pixelwise_regen_lane_ops(lh, wl, derived, ow * oh) for lh in lam_host]
        ach = sum(o["total"] / (ms / 1e3) for o, ms in zip(ops, launch_ms)) / len(ops)
        line["roofline"] = {"bound": "sm_issue", "achieved": ach / 1e12, "peak": peak / 1e12, "unit": "Tlane-op/s",
                            "frac": ach / peak, "traffic": None,
                            "kernel": "pixelwise_regen_kernel (launch_ms: the whole plane)", "launch_ms": launch_ms,
                            "lane_ops_per_launch": [o["total"] for o in ops], "model_terms": ops[0],
                            "peak_basis": peak_basis}
    elif wl["algo"] == "pixel":
        ops = [pixelwise_lane_ops(lh, wl, derived, ow * oh) for lh in lam_host]
        ach = sum(o["total"] / (ms / 1e3) for o, ms in zip(ops, launch_ms)) / len(ops)
        line["roofline"] = {"bound": "sm_issue", "achieved": ach / 1e12, "peak": peak / 1e12, "unit": "Tlane-op/s",
                            "frac": ach / peak,
                            "traffic": PIXELWISE_DRAM_BYTES_PER_OUT_PX * ow * oh,
                            "traffic_basis": "ncu dram bytes of cell_mask_kernel + pixelwise_sparse_kernel on the "
                                             "1024^2 flat plane of the large frame's parameters, scaled by "
                                             "output pixels",
                            "kernel": "cell_mask_kernel + pixelwise_sparse_kernel + pixelwise_deferred_kernel "
                                      "(launch_ms: the whole render call of a plane)", "launch_ms": launch_ms,
                            "lane_ops_per_launch": [o["total"] for o in ops], "model_terms": ops[0],
                            "peak_basis": peak_basis}
    return line


def profile_once(wl_name):
    """Render plane 0 of a plain workload twice (one warm-up render, then the captured one): the small
    case for ncu captures."""
    import torch
    import film_grain_gb300 as fg
    wl = WORKLOADS[wl_name]
    L = fg.lib()
    params = build_params(fg, wl)
    derived = fg.derive_common(params, (wl["w"], wl["h"]))
    plane = host_planes(make_input(wl), wl["mode"])[0]
    lam = torch.from_numpy(fg.lambda_plane(fg.normalize_plane(plane)[0], derived.inv_e_pi_r2)).cuda()
    out = torch.empty((derived.output_height, derived.output_width), dtype=torch.float32, device="cuda")
    offs = np.ascontiguousarray(derived.offsets if wl["algo"] == "grain" else derived.offsets_input, np.float32)
    fn = L.fg_render_grainwise_async if wl["algo"] == "grain" else L.fg_render_pixelwise_async
    for _ in range(2):
        if fn(lam.data_ptr(), params.c, derived._c, offs.ctypes.data, out.data_ptr(),
              torch.cuda.current_stream().cuda_stream) != 0:
            raise RuntimeError(L.fg_last_error_message().decode())
    torch.cuda.synchronize()
    log(f"profile-once: {wl_name} plane 0 rendered twice")


def profile_once_surrogate():
    """The shipped network on a 1024^2 x 3 blob frame, twice: the small case for ncu captures."""
    import torch
    import film_grain_gb300 as fg
    from film_grain_gb300 import surrogate as sg, workloads
    net = sg.load_default()
    planes = host_planes(workloads.blobs_rgb(1024, 1024, 1), "rgb")
    u = torch.from_numpy(np.stack([fg.normalize_plane(p)[0] for p in planes])).cuda()
    radius = torch.full((3,), 0.025, dtype=torch.float32, device="cuda")
    for _ in range(2):
        net.infer(u, radius, seed=7)
    torch.cuda.synchronize()
    log("profile-once: surrogate on 1024^2 x 3 rendered twice")


def reference_line(args, wl_name):
    """--impl reference: the CPU oracle on the host cores, each step one bounded band of the frame."""
    import oracle
    oracle.build()
    wl = WORKLOADS[wl_name]
    threads = os.cpu_count() or 1
    rgb = make_input(wl)
    planes = host_planes(rgb, wl["mode"])
    vals = []
    desc = ""
    for i in range(args.warmup + args.steps):
        if wl["algo"] == "grain":
            v, _, desc, _ = cpu_grain_baseline(oracle, planes, wl, threads, count=False)
        else:
            v, _, desc, _ = cpu_pixel_baseline(oracle, planes, wl, threads, rows=None if wl["w"] <= 256 else threads)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    return {"impl": "reference", "metric": "MC samples/s", "value": value, "unit": "samples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64-rng/f32", "data": "synthetic (seeded)",
            "config": {"workload": wl_name, "description": wl["desc"]},
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                             "sample": desc + "; each step one sample"},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


DEFAULT_WORKLOAD = "pixel_rgb_4096"
# The other benchmark configurations, measured in the default one-GPU run beside the headline.
SIDE_WORKLOADS = ("pixel_luma_256", "grain_rgb_1024", "batch_sweep_64", "surrogate_rgb_4096")


def side_configs(steps, warmup, cpu):
    out = {}
    for name in SIDE_WORKLOADS:
        t0 = time.perf_counter()
        try:
            if name == "batch_sweep_64":
                out[name] = batch_line(steps, warmup, 1)
            elif name == "surrogate_rgb_4096":
                out[name] = surrogate_line(steps, warmup, 1, cpu=cpu)
            else:
                out[name] = plain_line(name, steps, warmup, cpu=cpu)
        except Exception as e:  # reported in the line, never silently dropped
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = time.perf_counter() - t0
        log(f"side config {name}: {out[name]['wall_s']:.1f} s")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + ["batch_sweep_64", "surrogate_rgb_4096"])
    ap.add_argument("--retrain", action="store_true",
                    help="surrogate_rgb_4096: train the network in this run instead of loading the shipped weights")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations measured beside the default workload")
    ap.add_argument("--config-steps", type=int, default=5, help="timed steps of each side configuration")
    ap.add_argument("--profile-once", action="store_true",
                    help="render plane 0 once after one warm-up render and exit (a small case for ncu captures)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if args.workload in ("batch_sweep_64", "surrogate_rgb_4096"):
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": f"{args.workload} has no reference counterpart"}))
            return
        if rank == 0:
            print(json.dumps(reference_line(args, args.workload)), flush=True)
        return

    import torch
    from film_grain_gb300 import build as fgbuild
    fgbuild.build()
    torch.cuda.set_device(local_rank)
    if args.profile_once:
        if args.workload == "surrogate_rgb_4096":
            profile_once_surrogate()
        elif args.workload != "batch_sweep_64":
            profile_once(args.workload)
        return
    if args.workload == "batch_sweep_64":
        line = batch_line(args.steps, args.warmup, world)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    if args.workload == "surrogate_rgb_4096":
        line = surrogate_line(args.steps, args.warmup, world, retrain=args.retrain, cpu=not args.no_cpu_baseline)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    big = WORKLOADS[args.workload]["w"] * WORKLOADS[args.workload]["h"] >= 4096 * 4096
    line = plain_line(args.workload, args.steps, args.warmup, rank, world, dist, cpu=not args.no_cpu_baseline,
                      e2e_steps=min(args.steps, 5) if big else None)
    if rank == 0 and world == 1 and args.workload == DEFAULT_WORKLOAD and not args.no_configs:
        line["configs"] = side_configs(max(1, args.config_steps), 3, cpu=not args.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
