"""Batched form of the fused training step: many scenes, one persistent launch per step.

Each scene is a dense [X,Y,Z,4] grid (BF16 or fp32 cells) plus a per-cell occupancy mask;
unoccupied cells are zero and are not parameters: the step writes gradient only to
occupied cells (the rest of each gradient buffer stays zero). A dilated brick mask built from the occupancy lets the kernel skip samples
whose eight trilinear corners are all unoccupied, exactly. Rays of all scenes go through
one ray queue; rays stop early once their transmittance drops below a threshold.

``BatchedTrainStep`` owns fixed device buffers for the rays, so a step can be captured in
a CUDA graph and replayed (``capture()``); ``autotune()`` picks the tile configuration
(samples per chunk, rays per block) by timing the candidates on the actual batch.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import torch

from . import _lib
from ._lib import PgbScene, check, ptr, require_cuda
from .grid_functions import grid_origin

# Empty-space bricks of 2^BRICK_LOG2 cells a side. At 0 the dilated mask is exact per
# cell (a sample is skipped iff its 8 corners are unoccupied); on the 64-scene workload
# the step measured 7.9 / 8.3 / 9.5 / 11.6 ms for bricks of 1 / 2 / 4 / 8 cells.
BRICK_LOG2 = 0


@dataclass
class Scene:
    """One scene of a batch. cells: [X,Y,Z,4] (bfloat16 or float32, zero where not
    occupied); occupancy: bool [X,Y,Z]; num_samples and delta_step sample its rays."""
    cells: torch.Tensor
    occupancy: torch.Tensor
    points_distance: float
    num_samples: int
    delta_step: float
    grid_min: tuple | None = None
    grad: torch.Tensor = field(default=None, repr=False)
    bricks: torch.Tensor = field(default=None, repr=False)
    occupancy_bits: torch.Tensor = field(default=None, repr=False)

    def prepare(self, brick_log2=BRICK_LOG2):
        require_cuda(self.cells, self.occupancy)
        if self.cells.dim() != 4 or self.cells.shape[-1] != 4 or not self.cells.is_contiguous():
            raise ValueError("scene cells must be a contiguous [X,Y,Z,4] tensor")
        if tuple(self.occupancy.shape) != tuple(self.cells.shape[:3]):
            raise ValueError("occupancy must be [X,Y,Z]")
        lib = _lib.load()
        dev = self.cells.device
        s = torch.cuda.current_stream(dev).cuda_stream
        X, Y, Z = (int(v) for v in self.cells.shape[:3])
        G = X * Y * Z
        bits = torch.empty((G + 31) // 32, dtype=torch.int32, device=dev)
        occ = self.occupancy.contiguous().to(torch.uint8)
        check(lib.pgb_pack_mask(ptr(occ), G, ptr(bits), s), "scene occupancy")
        self.occupancy_bits = bits
        B = [-(-d // (1 << brick_log2)) for d in (X, Y, Z)]
        self.bricks = torch.empty((B[0] * B[1] * B[2] + 31) // 32, dtype=torch.int32, device=dev)
        check(lib.pgb_build_bricks(ptr(bits), _lib.dims3((X, Y, Z)), brick_log2, ptr(self.bricks), s),
              "scene bricks")
        if self.grad is None:
            self.grad = torch.zeros(self.cells.shape, dtype=torch.float32, device=dev)
        if self.grid_min is None:
            self.grid_min = grid_origin(self.cells.shape, self.points_distance)
        desc = PgbScene()
        desc.cells = ptr(self.cells)
        desc.bricks = ptr(self.bricks)
        desc.occupancy = ptr(self.occupancy_bits)
        desc.grad_cells = ptr(self.grad)
        desc.dims[:] = [X, Y, Z]
        desc.brick_log2 = brick_log2
        desc.brick_dims[:] = B
        desc.origin[:] = [float(v) for v in self.grid_min]
        desc.points_distance = float(self.points_distance)
        desc.num_samples = int(self.num_samples)
        desc.delta_step = float(self.delta_step)
        return desc


# (samples per lane K, threads per block, merge): merge = 1 sums a warp's updates of the
# same cell before the atomics (trilinear)
TILE_CANDIDATES = [(1, 256, 0), (1, 256, 1), (2, 256, 0), (2, 256, 1), (2, 128, 0), (4, 256, 0),
                   (4, 128, 0), (8, 256, 0)]


class BatchedTrainStep:
    """Forward + MSE + backward over all rays of all scenes in one persistent launch.

    rays are given as device tensors origins [R,3], dirs [R,3], target [R,4] (float32)
    and ray_scene [R] (int32 scene index); set_rays() copies them into the step's fixed
    buffers (capacity max_rays), so a captured graph replays on new rays."""

    def __init__(self, scenes, max_rays, mode="trilinear", clip=True, term_threshold=1e-4,
                 stratified=False, seed=0, loss_weight=1.0, tiles=None, brick_log2=BRICK_LOG2):
        if not scenes:
            raise ValueError("a batch needs at least one scene")
        dtypes = {sc.cells.dtype for sc in scenes}
        if len(dtypes) != 1 or next(iter(dtypes)) not in (torch.float32, torch.bfloat16):
            raise TypeError("all scenes must share one cell dtype, float32 or bfloat16")
        self.scenes = list(scenes)
        self.dtype = _lib.STORAGE_CODES[next(iter(dtypes))]
        self.mode = {"nearest": _lib.PGB_NEAREST, "trilinear": _lib.PGB_TRILINEAR}[mode]
        self.clip = bool(clip)
        self.term_threshold = float(term_threshold)
        self.stratified = bool(stratified)
        self.seed = int(seed)
        self.loss_weight = float(loss_weight)
        self.max_samples = max(int(sc.num_samples) for sc in scenes)
        if tiles is None:
            tiles = (next((k for k in (2, 4, 8) if 32 * 32 * k >= self.max_samples), 8), 256, 0)
        self.tiles = self._tile(tiles)
        dev = scenes[0].cells.device
        self.device = dev
        if self.max_samples > 32 * 32 * 8:
            raise NotImplementedError("at most 8192 samples per ray in the batched form")
        if not self._tile_fits(self.tiles):
            raise ValueError(f"tile {self.tiles} cannot cover {self.max_samples} samples per ray")
        self.brick_log2 = None
        self._set_bricks(brick_log2)
        self.max_cells = max(int(sc.cells.shape[0] * sc.cells.shape[1] * sc.cells.shape[2]) for sc in scenes)
        lib = _lib.load()
        self.max_rays = int(max_rays)
        self.origins = torch.zeros(self.max_rays, 3, device=dev)
        self.dirs = torch.zeros(self.max_rays, 3, device=dev)
        self.target = torch.zeros(self.max_rays, 4, device=dev)
        self.ray_scene = torch.zeros(self.max_rays, dtype=torch.int32, device=dev)
        self.num_rays = 0
        self.workspace = torch.zeros(lib.pgb_batch_workspace_bytes(self.max_rays), dtype=torch.uint8,
                                     device=dev)
        self.loss = torch.zeros((), device=dev)
        self.rgba = None
        self.graph = None

    @staticmethod
    def _tile(tile):
        """(K, threads, merge) from a 2- or 3-tuple (merge defaults to 0)."""
        t = tuple(int(v) for v in tile)
        return t if len(t) == 3 else (t[0], t[1], 0)

    def _tile_fits(self, tile):
        # a ray spans at most 32 chunks of 32 * K samples
        return 32 * 32 * int(tile[0]) >= self.max_samples

    def _set_bricks(self, brick_log2):
        """(Re)builds every scene's dilated brick mask at 2^brick_log2 cells a side and the
        device table of scene descriptors."""
        if brick_log2 == self.brick_log2:
            return
        descs = (PgbScene * len(self.scenes))(*[sc.prepare(brick_log2) for sc in self.scenes])
        raw = bytes(memoryview(descs).cast("B"))
        self.scene_table = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.device)
        self.brick_log2 = int(brick_log2)

    def set_rays(self, origins, dirs, target, ray_scene):
        R = origins.shape[0]
        if R > self.max_rays:
            raise ValueError(f"{R} rays exceed the step's capacity of {self.max_rays}")
        if self.graph is not None and R != self.num_rays:
            raise ValueError("a captured step replays a fixed ray count; re-capture to change it")
        self.origins[:R].copy_(origins, non_blocking=True)
        self.dirs[:R].copy_(dirs, non_blocking=True)
        self.target[:R].copy_(target, non_blocking=True)
        self.ray_scene[:R].copy_(ray_scene, non_blocking=True)
        self.num_rays = R

    def _run(self, tiles=None):
        lib = _lib.load()
        s = torch.cuda.current_stream(self.device).cuda_stream
        check(lib.pgb_batch_zero_grads(ptr(self.scene_table), len(self.scenes), self.max_cells, s),
              "batched step")
        K, threads, merge = self._tile(tiles or self.tiles)
        check(lib.pgb_batch_train(ptr(self.scene_table), len(self.scenes), self.dtype, self.mode,
                                  1 if self.clip else 0, ptr(self.origins), ptr(self.dirs),
                                  ptr(self.target), ptr(self.ray_scene), self.num_rays,
                                  self.term_threshold, 1 if self.stratified else 0, self.seed,
                                  self.loss_weight, ptr(self.rgba), ptr(self.loss),
                                  ptr(self.workspace), K, threads, merge, s), "batched step")
        return self.loss

    def step(self):
        """One training step over the current rays (graph replay once captured)."""
        if self.graph is not None:
            self.graph.replay()
            return self.loss
        return self._run()

    def capture(self):
        """Captures zeroing + the persistent launch in a CUDA graph (after one eager run
        has configured the kernels)."""
        self._run()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                self._run()
        torch.cuda.current_stream(self.device).wait_stream(side)
        self.graph = g
        return g

    def autotune(self, candidates=TILE_CANDIDATES, reps=5, brick_sizes=None):
        """Times each (samples-per-lane, threads-per-block, merge) tile on the current rays, for
        each empty-space brick size 2^L in brick_sizes (default: the current one), and keeps
        the fastest; returns {tile: ms} at the chosen brick size (self.brick_log2)."""
        if self.graph is not None:
            raise RuntimeError("autotune before capture")
        best = None
        for L in (brick_sizes or (self.brick_log2,)):
            self._set_bricks(L)
            times = {}
            for tile in (self._tile(t) for t in candidates if self._tile_fits(t)):
                self._run(tile)
                torch.cuda.synchronize(self.device)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    self._run(tile)
                e1.record()
                torch.cuda.synchronize(self.device)
                times[tile] = e0.elapsed_time(e1) / reps
            tile = min(times, key=times.get)
            if best is None or times[tile] < best[2]:
                best = (L, tile, times[tile], times)
        self._set_bricks(best[0])
        self.tiles = best[1]
        return best[3]
