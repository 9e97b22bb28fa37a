"""The reference's training step (scripts/train.py:104-184) on the fused kernels.

Per step: rays from the cameras and images (in-kernel), forward + MSE + beta loss +
backward in one launch (FusedTrainStep), the TV gradient (two passes) when enabled, and
one Adam pass that also accumulates |grad| and clears the gradient for the next step.
Progressive growing (the pooled coarse-to-fine grids of :108-123) is not part of this
trainer; it trains the full grid as the reference does once the schedule has ended.
"""
from __future__ import annotations

import torch

from .optim import FusedAdam
from .render import FusedTrainStep


class Trainer:
    def __init__(self, grid, points_distance, num_samples, delta_step, lr, tv=0.0, beta=0.0,
                 mode="nearest", betas=(0.9, 0.999), eps=1e-8, stratified=False, seed=0):
        self.render = FusedTrainStep(grid, points_distance, num_samples, delta_step, mode=mode,
                                     stratified=stratified, seed=seed, beta=beta)
        self.opt = FusedAdam(grid, lr, betas, eps)
        self.tv = float(tv)
        self.beta = float(beta)
        self.losses = torch.zeros(3, device=grid.device)  # mse, tv, beta of the last step

    def step_cameras(self, transforms, images, camera_angle_x, num_rays, ray_seed, near=0.0):
        # the Adam pass left the gradient zeroed: accumulate into it directly
        self.render.step_cameras(transforms, images, camera_angle_x, num_rays, ray_seed, near=near,
                                 zero_grad=False)
        return self._finish()

    def step_rays(self, origins, dirs, target):
        self.render.step_rays(origins, dirs, target, zero_grad=False)
        return self._finish()

    def _finish(self):
        grad = self.render.grad
        self.losses[0] = self.render.losses[0]
        self.losses[2] = self.render.losses[1] if self.beta != 0.0 else 0.0
        if self.tv > 0.0:
            self.losses[1] = self.opt.add_tv(grad, self.tv)
        self.opt.step(grad)
        return self.losses
