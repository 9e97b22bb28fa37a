"""The optimiser side of the reference's training step (scripts/train.py) for one dense
fp32 grid: torch.optim.Adam (:89, :182), the TV loss (:44-65, :163-168) and the |grad|
accumulator (:184), as streaming kernels that also clear the gradient for the next step.
"""
from __future__ import annotations

import torch

from . import _lib
from ._lib import check, ptr, require_cuda


class FusedAdam:
    """torch.optim.Adam (no weight decay, no amsgrad) over one dense [X,Y,Z,4] fp32 grid.

    step(grad) applies one update from grad, adds |grad| to ``abs_grad`` (the reference's
    ``grid_cells_full_grad``) and zeroes grad, all in one pass, so the next training
    step can accumulate into grad without a separate fill."""

    def __init__(self, grid, lr, betas=(0.9, 0.999), eps=1e-8, accumulate_abs_grad=True):
        require_cuda(grid)
        if grid.dtype != torch.float32 or not grid.is_contiguous() or grid.numel() % 4 != 0:
            raise TypeError("FusedAdam takes a contiguous float32 grid")
        self.grid = grid
        self.lr = float(lr)
        self.betas = (float(betas[0]), float(betas[1]))
        self.eps = float(eps)
        self.exp_avg = torch.zeros_like(grid)
        self.exp_avg_sq = torch.zeros_like(grid)
        self.abs_grad = torch.zeros_like(grid) if accumulate_abs_grad else None
        self.step_count = 0
        lib = _lib.load()
        self._tv_ws = torch.zeros(lib.pgb_tv_workspace_bytes(), dtype=torch.uint8, device=grid.device)
        self.tv_sumsq = torch.zeros((), dtype=torch.float64, device=grid.device)

    def add_tv(self, grad, weight, grid=None):
        """Adds the gradient of weight * tv_loss(grid) (scripts/train.py:163-165) to grad;
        returns the term's value as a device scalar. grid defaults to the optimised grid
        (the pooled grid while progressive growing runs)."""
        grid = self.grid if grid is None else grid
        lib = _lib.load()
        s = torch.cuda.current_stream(grid.device).cuda_stream
        dims = _lib.dims3(grid.shape)
        check(lib.pgb_tv_sumsq(ptr(grid), dims, ptr(self.tv_sumsq), ptr(self._tv_ws), s), "tv loss")
        check(lib.pgb_tv_grad(ptr(grid), dims, ptr(self.tv_sumsq), float(weight), ptr(grad), s),
              "tv loss")
        return float(weight) * self.tv_sumsq.sqrt()

    @torch.no_grad()
    def step(self, grad=None, zero_grad=True):
        grad = self.grid.grad if grad is None else grad
        if grad is None or grad.shape != self.grid.shape or grad.dtype != torch.float32:
            raise ValueError("step needs the grid's float32 gradient")
        self.step_count += 1
        s = torch.cuda.current_stream(self.grid.device).cuda_stream
        check(_lib.load().pgb_adam_step(ptr(self.grid), ptr(grad), ptr(self.exp_avg),
                                        ptr(self.exp_avg_sq), ptr(self.abs_grad), self.grid.numel(),
                                        self.lr, self.betas[0], self.betas[1], self.eps,
                                        self.step_count, 1 if zero_grad else 0, s), "adam step")

    @torch.no_grad()
    def step_tv(self, grad, weight, out, zero_grad=True):
        """add_tv on the optimised grid followed by step, in two passes instead of three:
        the TV loss value (one reduction over the grid), then Adam on grad + the TV gradient
        with the stencil evaluated in the update pass. The updated grid is written to
        ``out`` (a buffer of the grid's shape, not the grid itself: a cell's neighbours are
        read while cells are updated), which becomes ``self.grid``; the previous grid
        tensor is left holding the pre-step values. Returns weight * tv_loss as a device
        scalar."""
        g = self.grid
        if out.shape != g.shape or out.dtype != g.dtype or not out.is_contiguous() or out.data_ptr() == g.data_ptr():
            raise ValueError("out must be a separate contiguous float32 buffer of the grid's shape")
        if grad is None or grad.shape != g.shape or grad.dtype != torch.float32:
            raise ValueError("step_tv needs the grid's float32 gradient")
        lib = _lib.load()
        s = torch.cuda.current_stream(g.device).cuda_stream
        dims = _lib.dims3(g.shape)
        check(lib.pgb_tv_sumsq(ptr(g), dims, ptr(self.tv_sumsq), ptr(self._tv_ws), s), "tv loss")
        self.step_count += 1
        check(lib.pgb_adam_tv_step(ptr(g), ptr(out), ptr(grad), ptr(self.exp_avg), ptr(self.exp_avg_sq),
                                   ptr(self.abs_grad), dims, ptr(self.tv_sumsq), float(weight), self.lr,
                                   self.betas[0], self.betas[1], self.eps, self.step_count,
                                   1 if zero_grad else 0, s), "adam + tv step")
        self.grid = out
        return float(weight) * self.tv_sumsq.sqrt()
