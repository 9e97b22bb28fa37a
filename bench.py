"""Benchmark of the fused render-path training step (forward + MSE + backward).

Workload (dense 256^3 fp32 RGBA grid of 16 Gaussian blobs, box [-1.5,1.5]^3; 100 cameras of
800x800 at radius 4 on the upper hemisphere, FOV 0.691 rad, whose target images are rendered
from a second seeded ground-truth grid; 8192 random rays per step spread camera-major over
the cameras, near 2, far 6, 256 stratified samples per ray, trilinear lookup). Synthetic
seeded data stands in for the NeRF-synthetic scenes.

A step = zero the dense gradient (on a side stream, by clearing the cells the buffer's
previous step wrote) + one fused kernel that generates the rays from the resident cameras
and images, samples, looks up, composites, takes the MSE gradient and scatters dL/dcell. `value` is rays/s with everything resident in HBM; `e2e` is the same
metric through FusedTrainStep.step_rays with the ray batch (origins, dirs, targets)
copied from pinned host memory every step and the loss copied back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the reference's algorithm on the host CPU (the oracle's
restatement of it in PyTorch ops, all host threads) on the same workload: every step is
the full 8192-ray batch. Under torchrun with N > 1 each rank trains on its own ray batch
with a replicated grid and the gradients are summed with one all-reduce per step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import scenes  # noqa: E402  (seeded synthetic scene builder)

WORKLOAD = dict(workload="train step, 256^3 fp32 grid, 100 cams 800x800 with targets rendered "
                         "from a seeded ground-truth grid, 8192 rays x 256 stratified samples, "
                         "trilinear", grid=256, cameras=100, image=800, rays=8192, samples=256,
                mode="trilinear", near=2.0, far=6.0, blobs=16, rgb="sigmoid",
                camera_angle_x=0.691, grid_seed=1, camera_seed=2, ground_truth_seed=4)
# the precision form: 512^3 BF16 cells, 64 blobs, uniform RGB, 65536 rays from 200 cameras
# of 800x800, 512 samples, compensated log-sum transmittance
PRECISION = dict(workload="precision form, 512^3 grid (64 blobs, uniform RGB), 200 cams 800x800 "
                          "with targets rendered from a seeded ground-truth grid, 65536 rays x 512 "
                          "stratified samples, trilinear, log-sum transmittance", grid=512,
                 cameras=200, image=800, rays=65536, samples=512, mode="trilinear", near=2.0,
                 far=6.0, blobs=64, rgb="uniform", camera_angle_x=0.691, grid_seed=21,
                 camera_seed=22, ground_truth_seed=23)
NCU_TRAFFIC_BYTES = 145_588_480 + 12_452_096  # DRAM read + write, one launch
METRIC = "train rays/sec (fwd+bwd)"
# samples per chunk of the fused step (0: the library's choice)
CHUNK = 0
# how a gradient buffer is re-zeroed for its next step: "marked" clears the 4-cell units
# its previous step wrote (the step's kernel marks them); "fill" writes the whole buffer.
# On one GPU the bench reads no gradient and adds nothing into it, so both give the same
# steps. Ranks of a multi-GPU run sum their gradients in place (all-reduce), which writes
# cells no local step marked, so they fill.
ZEROING = "marked"


def zeroing_for(world):
    return ZEROING if world == 1 else "fill"


# CUDA events bracket every KERNEL_EVENT_EVERY-th launch of the fused kernel in a timed
# region. Events around every launch add ~3 us to each step (0.0925 against 0.0893 ms at
# the headline workload) and, by leaving gaps in which the side-stream gradient clear runs
# alone, understate the kernel's time inside a real step (0.089 against 0.093 ms).
KERNEL_EVENT_EVERY = 4


def timed_launches(step, steps, launch):
    """Runs launch(i) for i < steps with the fused kernel's events on a sample of them;
    returns the (start, end) event pairs."""
    events = []
    for i in range(steps):
        step.kernel_events = events if i % KERNEL_EVENT_EVERY == 0 else None
        launch(i)
    step.kernel_events = None
    return events


def mean_kernel_ms(events):
    return sum(a.elapsed_time(b) for a, b in events) / max(1, len(events))


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def scene_grids(W):
    """(trained grid, ground-truth grid) of a workload, float32 on the CPU, seeded."""
    grid = scenes.make_grid_fast(W["grid"], W["blobs"], W["grid_seed"], rgb=W["rgb"])
    gt = scenes.make_grid_fast(W["grid"], W["blobs"], W["ground_truth_seed"], rgb=W["rgb"])
    return grid, gt


def build_scene(pg, dev, W):
    """The trained grid, the cameras and their target images ([C,H,W,4] fp32, resident:
    1 GiB at 100 x 800^2), rendered on the GPU from the ground-truth grid along each
    pixel's ray with the step's sampling."""
    grid, gt = scene_grids(W)
    grid = grid.to(dev)
    T = torch.from_numpy(scenes.make_cameras(W["cameras"], seed=W["camera_seed"])).to(dev)
    S = W["samples"]
    imgs = pg.inference.render_camera_images(
        gt.to(dev), T, W["image"], W["image"], W["camera_angle_x"], W["near"],
        (W["far"] - W["near"]) / S, S, 3.0 / W["grid"], mode=W["mode"])
    return grid, T, imgs


class Clocks:
    """nvidia-smi sampler for the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def unique_cells(pg, grid, T, imgs, W, seed, delta, pd):
    """Per-unit figures of the algorithmic byte count, from the kernels' own index math on
    one step's rays (trilinear): (distinct cells read by in-bounds samples, as the
    reference reads them; distinct cells of the live samples, in bounds with
    transmittance > 0, which no exact implementation can skip; the in-bounds and live
    shares of the samples)."""
    S, side = W["samples"], W["grid"]
    idx, inb, coords = pg.render.camera_sample_indices(
        grid, T, imgs, W["camera_angle_x"], W["rays"], seed, W["near"], delta, S, pd,
        mode="trilinear", stratified=True, seed=7, return_coords=True)
    lin = (idx[..., 0] * side + idx[..., 1]) * side + idx[..., 2]
    all_cells = int(torch.unique(lin[inb.unsqueeze(-1).expand_as(lin)]).numel())
    with torch.no_grad():
        vals = pg.trilinear_interpolation(coords.reshape(-1, 3), idx.reshape(-1, 8, 3),
                                          grid.float(), clip=True)
    alpha = vals[:, 3].reshape(inb.shape) * inb
    trans = torch.cumprod(torch.cat([torch.ones_like(alpha[:, :1]), 1 - alpha[:, :-1]], 1), 1)
    live = inb & (trans > 0)
    live_cells = int(torch.unique(lin[live.unsqueeze(-1).expand_as(lin)]).numel())
    shares = float(inb.float().mean()), float(live.float().mean())
    del idx, lin, coords, vals
    return all_cells, live_cells, shares[0], shares[1]


def reference_cpu_steps(W, steps, warmup, budget_s=None):
    """The reference's training step on the host cores: the oracle's restatement of
    scripts/train.py:142-156, 181 in torch CPU ops (fp32 autograd, all host threads) on the
    full workload: every step is one fwd+bwd of W["rays"] camera rays (counter-hash pixel
    positions, as the GPU arm draws them) x W["samples"] stratified samples on the seeded
    grid, with targets rendered by the oracle from the ground-truth grid along the same
    rays (untimed). `warmup` untimed steps, then `steps` timed ones (fewer when budget_s of
    timed work runs out first, at least 2). Returns (median seconds per timed step, timed
    steps, threads)."""
    from oracle import torch_port as tp
    torch.set_num_threads(os.cpu_count() or 1)
    grid, gt = scene_grids(W)
    T = torch.from_numpy(scenes.make_cameras(W["cameras"], seed=W["camera_seed"]))
    pd = 3.0 / W["grid"]
    S, R = W["samples"], W["rays"]
    delta = (W["far"] - W["near"]) / S
    gmin = tp.grid_min(grid.shape, pd)
    jit = tp.jitter_for(7, R, S)
    frame = torch.zeros(1, W["image"], W["image"], 4).expand(W["cameras"], -1, -1, -1)
    times = []
    for i in range(warmup + steps):
        o, d, _ = tp.camera_batch(T, W["camera_angle_x"], frame, R, 1000 + i, W["near"])
        with torch.no_grad():
            target = tp.render(gt, o, d, S, delta, gmin, pd, W["mode"], True, jit)
        g = grid.detach().requires_grad_(True)
        t0 = time.perf_counter()
        loss = tp.train_loss(g, o, d, target, S, delta, gmin, pd, W["mode"], True, jit)
        loss.backward()
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
            if budget_s is not None and len(times) >= 2 and sum(times) >= budget_s:
                break
    return statistics.median(times), len(times), torch.get_num_threads()


def cpu_reference_rate(W, budget_s=15.0):
    """cpu_baseline: the reference's step on the host cores (reference_cpu_steps), one
    warm-up step and up to 20 timed ones within budget_s."""
    sec, n, threads = reference_cpu_steps(W, 20, 1, budget_s)
    return dict(value=W["rays"] / sec, unit="rays/s", cores=threads, kind="port",
                sample=f"the full workload ({W['rays']} rays x {W['samples']} stratified samples, "
                       f"{W['grid']}^3, {W['mode']}) per step, fwd+bwd, median of {n} steps after "
                       "1 warm-up; oracle restatement in torch CPU ops, fp32, all host threads")


def torch_gpu_rate(W, grid, T, imgs, dev, steps=10, warmup=2):
    """The reference's algorithm as plain torch ops on the same GPU (oracle port with
    CUDA tensors): `warmup` untimed steps, then `steps` steps timed with CUDA events, the
    SM clocks sampled around them."""
    from oracle import torch_port as tp
    pd = 3.0 / W["grid"]
    S = W["samples"]
    R = W["rays"]
    delta = (W["far"] - W["near"]) / S
    gmin = tp.grid_min(grid.shape, pd).to(dev)
    o, d, target = tp.camera_batch(T.cpu(), W["camera_angle_x"], imgs.cpu(), R, 4242, W["near"])
    o, d, target = o.to(dev), d.to(dev), target.to(dev)
    jit = tp.jitter_for(7, R, S).to(dev)

    def one():
        g = grid.detach().requires_grad_(True)
        loss = tp.train_loss(g, o, d, target, S, delta, gmin, pd, W["mode"], True, jit)
        loss.backward()

    for _ in range(warmup):
        one()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev.index) as clk:
        e0.record()
        for _ in range(steps):
            one()
        e1.record()
        torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    return dict(value=R / (ms / 1e3), unit="rays/s", ms_per_step=ms, kind="port",
                clocks=clk.summary(),
                sample=f"{R} rays x {S} samples, same scene, {steps} steps after {warmup} warm-up")


def storage_leg(pg, grid, T, imgs, W, dev, dtype, steps, warmup, mode=None, zeroing=None):
    """Same workload with the grid stored as `dtype` (fp32 arithmetic and gradients), or
    with another lookup mode: rays/s of the whole step and the fused kernel's time."""
    S, R = W["samples"], W["rays"]
    g = grid.to(dtype)
    step = pg.FusedTrainStep(g, 3.0 / W["grid"], S, (W["far"] - W["near"]) / S,
                             mode=mode or W["mode"], stratified=True, seed=7, overlap_zero=True,
                             chunk_samples=CHUNK, zeroing=zeroing or ZEROING)
    stream = torch.cuda.current_stream(dev)
    for i in range(warmup):
        step.step_cameras(T, imgs, W["camera_angle_x"], R, 5000 + i, near=W["near"])
    torch.cuda.synchronize(dev)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    events = timed_launches(step, steps, lambda i: step.step_cameras(
        T, imgs, W["camera_angle_x"], R, 6000 + i, near=W["near"]))
    t1.record(stream)
    torch.cuda.synchronize(dev)
    ms = t0.elapsed_time(t1) / steps
    kern = mean_kernel_ms(events)
    return {"value": R / (ms / 1e3), "unit": "rays/s", "ms_per_step": ms, "kernel_ms": kern,
            "storage": str(dtype).replace("torch.", ""), "note": "same workload, fp32 arithmetic "
            "and gradients, cells stored in this type"}


def drop_in_leg(pg, grid, T, imgs, W, dev, steps, warmup):
    """scripts/train.py:129-156 with the reference's imports swapped for this package's
    drop-in functions: the unfused path, one kernel per reference function (ray
    generation, sample points, normalisation, nearest lookup with the clip fused, masked
    compositing, torch's MSE, autograd backward through the hand-written scatters). Same
    cameras and grid, 82 rays per camera x 100 cameras, 256 samples, nearest lookup (the
    lookup train.py uses)."""
    S = W["samples"]
    per_cam = W["rays"] // W["cameras"]
    pd = 3.0 / W["grid"]
    delta = (W["far"] - W["near"]) / S
    grid_indices, _, _, _ = pg.generate_grid(W["grid"], W["grid"], W["grid"], pd, device=dev)
    g = grid.clone().requires_grad_(True)
    stream = torch.cuda.current_stream(dev)

    def one():
        g.grad = None
        samples, target, _, _ = pg.sample_camera_rays_batched(T, W["camera_angle_x"], imgs, per_cam, S,
                                                              delta, False, False, device=dev)
        n = pg.normalize_samples_for_indecies(grid_indices, samples, pd)
        vals, mask = pg.get_nearest_voxels(n, g, clip=True)
        vals = vals * mask.unsqueeze(-1)
        px = pg.compute_alpha_weighted_pixels(vals.reshape(T.shape[0], per_cam, S, 4))
        loss = torch.nn.functional.mse_loss(px.reshape(-1, 4), target)
        loss.backward()
        return loss

    for _ in range(warmup):
        one()
    torch.cuda.synchronize(dev)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        one()
    t1.record(stream)
    torch.cuda.synchronize(dev)
    ms = t0.elapsed_time(t1) / steps
    rays = per_cam * W["cameras"]
    return {"value": rays / (ms / 1e3), "unit": "rays/s", "ms_per_step": ms, "rays": rays,
            "note": "the reference's train.py step composed from the drop-in functions "
                    "(import swap only), nearest lookup, torch.rand ray draws, autograd"}


def random_access_ceiling(pg, dev, reads=1 << 24, reps=5):
    """The GPU's rate for independent random 32 B sectors out of a 256 MiB buffer (16 B
    loads, and float4 atomic adds), each launch after a 256 MiB write that evicts L2:
    the ceiling for gathers and scatters with no reuse, as the render kernels do."""
    from plenoxels_gb300 import _lib, probes
    lib = _lib.load()
    plib = probes.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    nbytes = 256 << 20
    table = torch.zeros(nbytes // 4, device=dev)
    flush = torch.empty(nbytes // 4, device=dev)
    sink = torch.zeros(1, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = {}
    for kind in ("reads", "atomics"):
        n = reads if kind == "reads" else reads // 4
        ms = []
        for rep in range(reps + 1):
            _lib.check(lib.pgb_fill_zero(flush.data_ptr(), nbytes, stream), "pgb_fill_zero")
            e0.record()
            if kind == "reads":
                st = plib.pgb_probe_random_reads(table.data_ptr(), nbytes, n, 17 + rep, sink.data_ptr(), stream)
            else:
                st = plib.pgb_probe_random_atomics(table.data_ptr(), nbytes, n, 17 + rep, stream)
            e1.record()
            _lib.check(st, "pgb_probe_random_" + kind)
            torch.cuda.synchronize(dev)
            if rep:
                ms.append(e0.elapsed_time(e1))
        best[kind] = n / (min(ms) / 1e3) / 1e9
    del table, flush
    return {"read_gsectors_per_s": best["reads"], "read_sector_gbs": best["reads"] * 32,
            "atomic_gupdates_per_s": best["atomics"],
            "probe": "2^24 random 16 B loads / 2^22 random float4 atomic adds over 256 MiB, "
                     "L2 evicted before each launch, best of 5"}


def batched_leg(pg, dev, steps=30, seed=11, num_scenes=64):
    """Batched form: 64 scenes (sides from {32,64,128,256}), 5 % occupied cells, BF16
    cells, rays per scene log-uniform in [1k, 64k], 512 samples per ray, early
    termination at T < 1e-4, one persistent launch per step replayed from a CUDA graph.
    Returns aggregate rays/s and per-step latency percentiles."""
    from plenoxels_gb300.batch import BatchedTrainStep, Scene
    g = torch.Generator(device=dev).manual_seed(seed)
    rng = np.random.default_rng(seed)
    scs, origins, dirs, targets, owners = [], [], [], [], []
    S = 512
    for i in range(num_scenes):
        side = int(rng.choice([32, 64, 128, 256]))
        pd = 3.0 / side
        ax = (torch.arange(side, device=dev, dtype=torch.float32) - math.ceil(side / 2) + 1) * pd
        dens = torch.zeros(side, side, side, device=dev)
        for _ in range(8):
            c = torch.rand(3, generator=g, device=dev) * 2 - 1
            a = 5 + 15 * torch.rand((), generator=g, device=dev)
            d2 = ((ax - c[0]) ** 2)[:, None, None] + ((ax - c[1]) ** 2)[None, :, None] + \
                ((ax - c[2]) ** 2)[None, None, :]
            dens += a * torch.exp(-d2 / (2 * 0.3 ** 2))
        sub = dens.flatten()[torch.randint(0, dens.numel(), (1 << 20,), generator=g, device=dev)]
        occ = dens > torch.quantile(sub, 0.95)
        cells = torch.cat([torch.rand(side, side, side, 3, generator=g, device=dev),
                           dens.unsqueeze(-1)], -1)
        cells[~occ] = 0.0
        scs.append(Scene(cells.to(torch.bfloat16).contiguous(), occ, pd, S, 4.0 / S))
        n = int(round(math.exp(rng.uniform(math.log(1000), math.log(64000)))))
        per_cam = -(-n // 4)
        T = torch.from_numpy(scenes.make_cameras(4, seed * 1000 + i)).to(dev)
        imgs = torch.rand(4, 32, 32, 4, generator=g, device=dev)
        uv = torch.rand(4, per_cam, 2, generator=g, device=dev)
        dd, px = pg.generate_rays_batched(imgs, per_cam, T, 0.691, device=dev, ray_uv=uv)
        oo = torch.repeat_interleave(T[:, :3, 3], per_cam, 0) + 2.0 * dd
        origins.append(oo[:n]); dirs.append(dd[:n]); targets.append(px[:n])
        owners.append(torch.full((n,), i, dtype=torch.int32, device=dev))
        del dens
    R = sum(o.shape[0] for o in origins)
    step = BatchedTrainStep(scs, R, term_threshold=1e-4)
    step.set_rays(torch.cat(origins), torch.cat(dirs), torch.cat(targets), torch.cat(owners))
    tiles = step.autotune(reps=3, brick_sizes=(0, 1, 2))
    step.capture()
    for _ in range(3):
        step.step()
    torch.cuda.synchronize(dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        a.record()
        step.step()
        b.record()
    torch.cuda.synchronize(dev)
    ms = sorted(a.elapsed_time(b) for a, b in ev)
    p50 = ms[len(ms) // 2]
    p99 = ms[min(len(ms) - 1, int(math.ceil(0.99 * len(ms))) - 1)]
    cells = sum(int(sc.cells.shape[0]) ** 3 for sc in scs)
    occ_cells = sum(int(sc.occupancy.sum()) for sc in scs)
    return {"value": R / (statistics.median(ms) / 1e3), "unit": "rays/s", "rays_per_step": R,
            "scenes": len(scs), "cells": cells, "occupied_cells": occ_cells, "samples": S,
            "p50_ms": p50, "p99_ms": p99,
            "tiles": {f"K{k}_t{t}" + ("_merge" if m else ""): v for (k, t, m), v in tiles.items()},
            "chosen_tile": f"K{step.tiles[0]}_t{step.tiles[1]}" + ("_merge" if step.tiles[2] else ""),
            "chosen_brick_cells": 1 << step.brick_log2,
            "note": "BF16 cells, occupancy-masked fp32 gradients, early termination at T<1e-4, "
                    "CUDA-graph replay of zeroing + one persistent launch + the ordered loss sum; same rays every step"}


def full_step_leg(pg, grid, T, imgs, W, dev, steps, warmup):
    """The whole reference training step (scripts/train.py:142-184) at its default weights
    (lr 0.0075, tv 1e-5, beta 5e-3): fused render + MSE + beta + backward, TV gradient,
    Adam + |grad| accumulator + gradient clear. Also the Adam pass's achieved bandwidth."""
    from plenoxels_gb300.train import Trainer
    S, R = W["samples"], W["rays"]
    g = grid.clone()
    tr = Trainer(g, 3.0 / W["grid"], S, (W["far"] - W["near"]) / S, 0.0075, tv=1e-5, beta=5e-3,
                 mode=W["mode"], stratified=True, seed=7)
    stream = torch.cuda.current_stream(dev)
    for i in range(warmup):
        tr.step_cameras(T, imgs, W["camera_angle_x"], R, 7000 + i, near=W["near"])
    torch.cuda.synchronize(dev)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for i in range(steps):
        tr.step_cameras(T, imgs, W["camera_angle_x"], R, 8000 + i, near=W["near"])
    t1.record(stream)
    torch.cuda.synchronize(dev)
    ms = t0.elapsed_time(t1) / steps
    # the Adam pass alone: reads param, grad, both moments and the accumulator, writes all
    # five back (the gradient as zeros): 10 x 16 B per cell
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    for _ in range(steps):
        tr.opt.step(tr.render.grad)
    a1.record(stream)
    torch.cuda.synchronize(dev)
    adam_ms = a0.elapsed_time(a1) / steps
    adam_bytes = grid.numel() // 4 * 160
    # the TV loss reduction + the Adam pass with the TV stencil fused (what a step runs)
    bufs = [tr.grid, tr._spare if tr._spare is not None else torch.empty_like(tr.grid)]
    a0.record(stream)
    for i in range(steps):
        tr.opt.step_tv(tr.render.grad, 1e-5, bufs[(i + 1) % 2])
    a1.record(stream)
    torch.cuda.synchronize(dev)
    adam_tv_ms = a0.elapsed_time(a1) / steps
    peak, _ = _peaks()
    return {"value": R / (ms / 1e3), "unit": "rays/s", "ms_per_step": ms,
            "adam_ms": adam_ms, "adam_gbs": adam_bytes / (adam_ms / 1e3) / 1e9,
            "adam_frac_of_measured_peak": adam_bytes / (adam_ms / 1e3) / 1e9 / peak,
            "tv_and_fused_adam_tv_ms": adam_tv_ms,
            "note": "render + MSE + beta (5e-3) + backward, TV (1e-5) loss and gradient (the "
                    "gradient's stencil evaluated inside the Adam pass), Adam (lr 0.0075) with "
                    "|grad| accumulation; dense fp32 grid of 256^3"}


def run_reference_arm(args, W):
    """--impl reference: the reference's training step on the host cores (the oracle's
    torch restatement, fp32 autograd, all threads), each step the full workload of
    W["rays"] rays; W untimed steps, then K timed ones."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sec, n, cores = reference_cpu_steps(W, args.steps, args.warmup)
    value = W["rays"] / sec
    sample = (f"the full workload ({W['rays']} rays x {W['samples']} stratified samples, "
              f"{W['grid']}^3, {W['mode']}) per step, fwd+bwd, median of {n} steps after "
              f"{args.warmup} warm-up; oracle restatement in torch CPU ops, fp32, all host threads")
    line = {"metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference", "config": dict(W),
            "cpu_baseline": {"value": value, "unit": "rays/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def precision_leg(pg, dev, steps, warmup):
    """The precision form: a 512^3 grid of 64 blobs with BF16 cells, 65536 rays per step
    from 200 cameras of 800x800, 512 stratified samples, compensated log-sum
    transmittance; the same step with fp32 cells beside it, and both with the product
    transmittance. Rays/s of the whole step (gradient zeroing + fused launch) and the
    fused kernel's time, for each form."""
    P = PRECISION
    grid, T, imgs = build_scene(pg, dev, P)
    S, R = P["samples"], P["rays"]
    out = {"workload": P["workload"]}
    forms = [("bf16_logsum", torch.bfloat16, "logsum"), ("f32_logsum", torch.float32, "logsum"),
             ("bf16_product", torch.bfloat16, "product"), ("f32_product", torch.float32, "product")]
    stream = torch.cuda.current_stream(dev)
    for name, dt, trans in forms:
        g = grid.to(dt)
        st = pg.FusedTrainStep(g, 3.0 / P["grid"], S, (P["far"] - P["near"]) / S, mode=P["mode"],
                               stratified=True, seed=7, overlap_zero=True, transmittance=trans,
                               chunk_samples=CHUNK, zeroing=ZEROING)
        for i in range(warmup):
            st.step_cameras(T, imgs, P["camera_angle_x"], R, 5000 + i, near=P["near"])
        torch.cuda.synchronize(dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        events = timed_launches(st, steps, lambda i: st.step_cameras(
            T, imgs, P["camera_angle_x"], R, 6000 + i, near=P["near"]))
        t1.record(stream)
        torch.cuda.synchronize(dev)
        ms = t0.elapsed_time(t1) / steps
        kern = mean_kernel_ms(events)
        out[name] = {"value": R / (ms / 1e3), "unit": "rays/s", "ms_per_step": ms, "kernel_ms": kern}
        del st, g
    out["bf16_over_f32_logsum"] = out["bf16_logsum"]["value"] / out["f32_logsum"]["value"]
    out["bf16_over_f32_product"] = out["bf16_product"]["value"] / out["f32_product"]["value"]
    del grid, imgs
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-baselines", action="store_true", help="skip the CPU and torch-GPU legs")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched multi-scene leg")
    ap.add_argument("--no-precision", action="store_true", help="skip the 512^3 precision-form leg")
    ap.add_argument("--batched-only", action="store_true", help="run only the batched leg")
    ap.add_argument("--batched-scenes", type=int, default=64, help="scenes of the batched leg")
    args = ap.parse_args()
    W = dict(WORKLOAD)

    if args.impl == "reference":
        run_reference_arm(args, W)
        return

    import plenoxels_gb300 as pg
    import plenoxels_gb300.render  # noqa: F401

    if args.batched_only:
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        torch.cuda.set_device(dev)
        print(json.dumps({"batched_form": batched_leg(pg, dev, num_scenes=args.batched_scenes)}))
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    S, R = W["samples"], W["rays"]
    pd = 3.0 / W["grid"]
    delta = (W["far"] - W["near"]) / S
    grid, T, imgs = build_scene(pg, dev, W)
    from plenoxels_gb300.distributed import allreduce_gradient
    # weak scaling: R rays per rank, each rank's MSE weighted by its share of R * world
    step = pg.FusedTrainStep(grid, pd, S, delta, mode=W["mode"], stratified=True, seed=7,
                             loss_weight=1.0 / world, overlap_zero=True, chunk_samples=CHUNK,
                             zeroing=zeroing_for(world))
    stream = torch.cuda.current_stream(dev)

    def train(i):
        step.step_cameras(T, imgs, W["camera_angle_x"], R, 1000 * rank + i, near=W["near"])
        allreduce_gradient(step.grad)

    for i in range(args.warmup):
        train(i)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()

    # timed region: K steps (gradient zeroing + fused kernel), events around each kernel
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def load(seconds, first):
        # the same fused step (no collective: ranks may run different counts), untimed, so
        # nvidia-smi samples the clocks under this load around the timed region
        i, end = first, time.perf_counter() + seconds
        while time.perf_counter() < end:
            for _ in range(64):
                step.step_cameras(T, imgs, W["camera_angle_x"], R, 1000 * rank + i, near=W["near"])
                i += 1
            torch.cuda.synchronize(dev)

    with Clocks(dev.index) as clk:
        load(0.4, 10_000)
        if world > 1:
            torch.distributed.barrier()
        launches0 = pg.launch_count()
        t0.record(stream)
        kern_events = timed_launches(step, args.steps, lambda i: train(args.warmup + i))
        t1.record(stream)
        torch.cuda.synchronize(dev)
        launches = pg.launch_count() - launches0
        load(0.3, 20_000)
    ms_total = t0.elapsed_time(t1)
    kern_ms = mean_kernel_ms(kern_events)
    if world > 1:
        tt = torch.tensor([ms_total], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(tt)
        torch.distributed.barrier()
    ms_step = ms_total / args.steps
    value = world * R / (ms_step / 1e3)

    # e2e: host ray batches through the public API (pinned H2D each step, loss D2H). A
    # batch is one pinned block [origins R*3 | dirs R*3 | target R*4], so a step's inputs
    # are one copy; the step reads contiguous views of the device copy
    nb = 4
    host = []
    uv_gen = torch.Generator(device=dev).manual_seed(7000 + rank)  # the same rays every run
    for b in range(nb):
        uv = torch.rand(W["cameras"], R // W["cameras"] + 1, 2, device=dev, generator=uv_gen)
        dirs, pixels = pg.generate_rays_batched(imgs, R // W["cameras"] + 1, T, W["camera_angle_x"],
                                                device=dev, ray_uv=uv)
        cam_pos = torch.repeat_interleave(T[:, :3, 3], R // W["cameras"] + 1, 0)
        o = cam_pos + W["near"] * dirs
        block = torch.cat([x[:R].reshape(-1) for x in (o, dirs, pixels)]).cpu().pin_memory()
        host.append(block)

    def views(block):
        return block[:3 * R].view(R, 3), block[3 * R:6 * R].view(R, 3), block[6 * R:].view(R, 4)

    # two device input blocks: step i+1's batch is copied on a copy stream while step i
    # runs, as a training loop would pipeline it; every copy is inside the timed region
    bufs = [torch.empty(10 * R, device=dev) for _ in range(2)]
    buf_views = [views(x) for x in bufs]
    copy_stream = torch.cuda.Stream(device=dev)
    # each step's losses land in its own row of a pinned host buffer: the kernel writes them
    # there (the GPU addresses pinned host memory), so the read-back needs no copy call
    loss_host = torch.zeros(args.steps + args.warmup + 1, 2, dtype=torch.float32).pin_memory()
    h2d = host[0].numel() * host[0].element_size()
    copied = [torch.cuda.Event(), torch.cuda.Event()]  # block b holds its batch
    free = [torch.cuda.Event(), torch.cuda.Event()]    # the step that last read block b has run
    used = [False, False]

    def pipelined(i, first_wait=None):
        b = i % 2
        with torch.cuda.stream(copy_stream):
            if first_wait is not None:
                copy_stream.wait_event(first_wait)
            if used[b]:
                copy_stream.wait_event(free[b])
            bufs[b].copy_(host[i % nb], non_blocking=True)
            copied[b].record(copy_stream)
        return b

    def run(i, b):
        stream.wait_event(copied[b])
        step.step_rays(*buf_views[b], loss_out=loss_host[i])
        allreduce_gradient(step.grad)
        free[b].record(stream)
        used[b] = True

    nxt = pipelined(0)
    for i in range(args.warmup):
        cur = nxt
        if i + 1 < args.warmup:
            nxt = pipelined(i + 1)
        run(i, cur)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    nxt = pipelined(args.warmup, first_wait=e0)
    for i in range(args.warmup, args.warmup + args.steps):
        cur = nxt
        if i + 1 < args.warmup + args.steps:
            nxt = pipelined(i + 1)
        run(i, cur)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    read_back = loss_host[args.warmup:args.warmup + args.steps, 0]
    assert bool(torch.isfinite(read_back).all()) and bool((read_back > 0).all()), \
        "every timed step's loss must reach the host"
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        tt = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(tt)
    e2e = {"value": world * R / (e2e_ms / 1e3), "unit": "rays/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": 4, "ms_per_step": e2e_ms}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # roofline of the fused kernel: algorithmic bytes per launch / its measured duration.
    # traffic: dram__bytes_read.sum + dram__bytes_write.sum of one launch of this kernel on
    # this workload under ncu
    U, U_live, inb_frac, live_frac = unique_cells(pg, grid, T, imgs, W, 1000 * rank + args.warmup,
                                                  delta, pd)
    # U: distinct cells of the step's in-bounds samples (the cells the reference's
    # algorithm reads); U_live: those of the live samples only (T > 0), the cells no exact
    # implementation can skip
    alg_bytes = U * 16 + U * 16 + R * 60
    alg_live = U_live * 16 + U_live * 16 + R * 60
    peak, peak_kind = _peaks()
    achieved = alg_bytes / (kern_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": NCU_TRAFFIC_BYTES,
                "traffic_unit": "bytes per launch (ncu capture of this workload)",
                "kernel": "render_kernel<trilinear,train>",
                "kernel_ms": kern_ms,
                "kernel_ms_sample": f"CUDA events around every {KERNEL_EVENT_EVERY}th launch of the "
                                    f"timed region ({len(kern_events)} launches)",
                "unique_cells": U, "algorithmic_bytes": alg_bytes,
                "unique_cells_definition": "distinct cells read by the step's in-bounds samples "
                                           "(all 8 corners), as the reference's algorithm reads them",
                "unique_cells_live": U_live, "algorithmic_bytes_live": alg_live,
                "frac_live": alg_live / (kern_ms / 1e3) / 1e9 / peak,
                "live_definition": "cells of the live samples only (in bounds, transmittance > 0): "
                                   "samples behind an opaque one have weight 0 and gradient 0, and "
                                   "the kernel stops reading a ray after the chunk where T reaches 0",
                "in_bounds_sample_share": inb_frac, "live_sample_share": live_frac,
                "peak_kind": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured" else "fallback 6.8 TB/s",
                "issued_gather_bytes": int(R * S * inb_frac * 8 * 16)}
    line = {"metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": dict(W, l2="inputs larger than L2: 256 MiB grid read and 256 MiB gradient "
                                 "zeroed + scattered every step, 1 GiB of target images",
                           chunk_samples=CHUNK, gradient_zeroing=zeroing_for(world),
                           parallelism=f"dp{world}" if world > 1 else "single"),
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "clocks": clk.summary()}
    rnd = random_access_ceiling(pg, dev)
    roofline["random_access_ceiling"] = rnd
    # DRAM sector traffic of one launch (ncu) at the measured kernel time, against the
    # random-sector read rate: above 1 means the kernel's sectors have more locality
    # (z-adjacent corners, consecutive samples) than independent random ones
    roofline["traffic_gbs_at_kernel_time"] = NCU_TRAFFIC_BYTES / (kern_ms / 1e3) / 1e9
    roofline["traffic_vs_random_read_ceiling"] = roofline["traffic_gbs_at_kernel_time"] / rnd["read_sector_gbs"]
    line["bf16_storage"] = storage_leg(pg, grid, T, imgs, W, dev, torch.bfloat16, args.steps,
                                       args.warmup)
    nearest = storage_leg(pg, grid, T, imgs, W, dev, torch.float32, args.steps, args.warmup,
                          mode="nearest")
    nearest.pop("storage")
    nearest["note"] = ("same workload with nearest-cell lookup (the lookup scripts/train.py "
                       "trains with); fp32 cells")
    line["nearest_lookup"] = nearest
    dense = storage_leg(pg, grid, T, imgs, W, dev, torch.float32, args.steps, args.warmup,
                        zeroing="fill")
    dense.pop("storage")
    dense["note"] = ("same workload with the whole 256 MiB gradient buffer written with zeros "
                     "before each step instead of its marked units; fp32 cells")
    line["dense_fill_zeroing"] = dense
    line["drop_in_path"] = drop_in_leg(pg, grid, T, imgs, W, dev, args.steps, args.warmup)
    line["full_training_step"] = full_step_leg(pg, grid, T, imgs, W, dev, args.steps, args.warmup)
    if not args.no_baselines:
        line["torch_gpu_baseline"] = torch_gpu_rate(W, grid, T, imgs, dev)
    del step, grid, imgs
    torch.cuda.empty_cache()
    if not args.no_precision:
        line["precision_form"] = precision_leg(pg, dev, args.steps, args.warmup)
    if not args.no_batched:
        line["batched_form"] = batched_leg(pg, dev)
    if not args.no_baselines:
        line["cpu_baseline"] = cpu_reference_rate(W)
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
