"""The reference's training step (scripts/train.py:104-184) on the fused kernels.

Per step: rays from the cameras and images (in-kernel) or given, forward + MSE + beta
loss + backward in one launch (FusedTrainStep), the TV gradient (two passes) when
enabled, and one Adam pass that also accumulates |grad| and clears the gradient.

With the TV term on the full grid (no pooling), the TV gradient is not a pass of its own:
Adam evaluates its stencil while updating (FusedAdam.step_tv), which needs the update
written to a second grid buffer. The trainer then alternates two buffers, and
``trainer.grid`` is always the current one (fuse_tv=False keeps one buffer, updated in
place, at the cost of the separate TV gradient pass).

Progressive growing (scripts/train.py:91-123): while the schedule's receptive field r is
above 1, the step renders the grid average-pooled with window r and stride max(1, r//4)
(pitch points_distance * stride, origin at the coordinate of cell r//2), and the pooled
gradient is spread back onto the full grid by the pooling's adjoint, which rewrites the
whole full gradient. The TV term applies once r < 19, to the grid being rendered.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr
from .grid_functions import pool_shape
from .optim import FusedAdam
from .render import FusedTrainStep

DEFAULT_FIELDS = list(range(93, 2, -2))  # scripts/train.py:91
STEPS_PER_FIELD = 5                       # scripts/train.py:92


class Trainer:
    def __init__(self, grid, points_distance, num_samples, delta_step, lr, tv=0.0, beta=0.0,
                 mode="nearest", betas=(0.9, 0.999), eps=1e-8, stratified=False, seed=0,
                 progressive_growing=False, fields=None, steps_per_field=STEPS_PER_FIELD,
                 fuse_tv=True):
        self.grid = grid
        self.fuse_tv = bool(fuse_tv)
        self._spare = None  # the second grid buffer of the fused TV + Adam pass
        self.points_distance = float(points_distance)
        self.cfg = dict(num_samples=num_samples, delta_step=delta_step, mode=mode,
                        stratified=stratified, seed=seed, beta=beta)
        self.render = FusedTrainStep(grid, points_distance, **self.cfg)
        self.opt = FusedAdam(grid, lr, betas, eps)
        self.tv = float(tv)
        self.beta = float(beta)
        self.progressive = bool(progressive_growing)
        self.fields = list(DEFAULT_FIELDS if fields is None else fields)
        self.steps_per_field = int(steps_per_field)
        self.step_index = 0
        self._pooled = {}  # field -> (pooled grid, its FusedTrainStep, stride, scratch)
        self.losses = torch.zeros(3, device=grid.device)  # mse, tv, beta of the last step

    def field(self, i):
        """Receptive field of step i (scripts/train.py:108); 0 once the schedule ends."""
        k = i // self.steps_per_field
        return self.fields[k] if k < len(self.fields) else 0

    def _pooled_step(self, r):
        if r not in self._pooled:
            stride = max(1, r // 4)
            start = int(r / 2)
            od, nbytes = pool_shape(self.grid.shape, r, stride)
            pooled = torch.empty(*od, 4, dtype=torch.float32, device=self.grid.device)
            scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=self.grid.device)
            # the min of grid_grid_original[start::stride, ...] (scripts/train.py:114-116)
            gmin = tuple(float(np.float32(start - math.ceil(s / 2) + 1) * np.float32(self.points_distance))
                         for s in self.grid.shape[:3])
            step = FusedTrainStep(pooled, self.points_distance * stride, grid_min=gmin, **self.cfg)
            self._pooled[r] = (pooled, step, stride, scratch)
        return self._pooled[r]

    def _run(self, launch):
        r = self.field(self.step_index) if self.progressive else 0
        lib = _lib.load()
        s = torch.cuda.current_stream(self.grid.device).cuda_stream
        full_grad = self.render.grad
        if r > 1:
            pooled, step, stride, scratch = self._pooled_step(r)
            dims = _lib.dims3(self.grid.shape)
            check(lib.pgb_avg_pool3d_fwd(ptr(self.grid), dims, r, stride, ptr(scratch), ptr(pooled), s),
                  "pooled grid")
            launch(step, True)
            render_step, tv_grid, tv_grad = step, pooled, step.grad
        else:
            # the Adam pass left the gradient zeroed: accumulate into it directly
            launch(self.render, False)
            render_step, tv_grid, tv_grad = self.render, self.grid, full_grad
        self.losses[0] = render_step.losses[0]
        self.losses[2] = render_step.losses[1] if self.beta != 0.0 else 0.0
        self.losses[1] = 0.0
        if self.tv > 0.0 and r < 19 and self.fuse_tv and r <= 1:
            # TV on the full grid: its gradient is evaluated inside the Adam pass, which
            # writes the new grid to the spare buffer; the buffers then swap roles
            if self._spare is None:
                self._spare = torch.empty_like(self.grid)
            old = self.grid
            self.losses[1] = self.opt.step_tv(full_grad, self.tv, self._spare)
            self.grid, self._spare = self._spare, old
            self.render.grid = self.grid
            self.step_index += 1
            return self.losses
        if self.tv > 0.0 and r < 19:
            self.losses[1] = self.opt.add_tv(tv_grad, self.tv, grid=tv_grid)
        if r > 1:
            check(lib.pgb_avg_pool3d_bwd(ptr(render_step.grad), _lib.dims3(self.grid.shape), r,
                                         stride, ptr(scratch), ptr(full_grad), s), "pooled grid")
        self.opt.step(full_grad)
        self.step_index += 1
        return self.losses

    def step_cameras(self, transforms, images, camera_angle_x, num_rays, ray_seed, near=0.0):
        return self._run(lambda st, zero: st.step_cameras(transforms, images, camera_angle_x,
                                                          num_rays, ray_seed, near=near,
                                                          zero_grad=zero))

    def step_rays(self, origins, dirs, target):
        return self._run(lambda st, zero: st.step_rays(origins, dirs, target, zero_grad=zero))
