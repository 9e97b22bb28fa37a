"""Ray-sharded data parallelism for the fused training step.

Rays are independent, so each rank renders its own share of the step's rays against a
replicated grid, and the only exchange is the gradient. Each rank weights its MSE by its
share of the global ray count, so the summed gradient and the summed loss equal the
single-process ones (scripts/train.py:156 takes the mean over all rays of the step).

Two ways to finish a step across ranks:
- allreduce_gradient: one sum all-reduce of the dense gradient, then every rank runs the
  same optimiser step on the whole grid (replicated optimiser state);
- ShardedGridUpdate: reduce-scatter of the gradient, so each rank holds the summed
  gradient of 1/N of the cells, an optimiser step on that shard only (optimiser state for
  1/N of the grid), and an all-gather of the updated shards into every rank's grid. It
  moves the same bytes as the all-reduce (an all-reduce is a reduce-scatter followed by an
  all-gather) and divides the optimiser pass and its memory by N.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard_rays(num_rays: int, rank: int, world_size: int) -> tuple[int, int]:
    """(start, count) of this rank's contiguous share of num_rays rays."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside world of size {world_size}")
    base, extra = divmod(int(num_rays), world_size)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def loss_weight(local_rays: int, global_rays: int) -> float:
    """Weight of a rank's mean-over-its-rays loss in the global mean."""
    return float(local_rays) / float(global_rays) if global_rays > 0 else 0.0


def allreduce_gradient(grad: torch.Tensor, group=None) -> torch.Tensor:
    """Sums the ranks' gradients in place (NCCL for CUDA tensors, gloo for CPU ones)."""
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
    return grad


def grid_shard(numel: int, rank: int, world_size: int) -> tuple[int, int]:
    """(start, length) in floats of rank's shard of a flat grid of numel floats: equal
    shards of whole cells (4 floats, so a shard keeps the 16-byte alignment of the
    vectorised kernels), the last ones shorter or empty when numel does not divide."""
    cells = numel // 4
    per = -(-cells // world_size)
    start = min(rank * per, cells)
    end = min(start + per, cells)
    return 4 * start, 4 * (end - start)


class ShardedGridUpdate:
    """The optimiser step of a replicated dense grid, sharded over the ranks of `group`.

    step(grad) reduce-scatters the ranks' dense gradients so that this rank holds the
    sum over ranks for its shard of the cells (grid_shard), applies the local optimiser to
    that shard, and all-gathers the updated shards, after which every rank's grid holds
    the same updated values. make_optimizer(shard) receives this rank's shard of the grid
    (a contiguous flat fp32 view into the grid's storage) and returns an object whose
    step(grad_shard) updates it in place from the summed gradient of the shard: on GPUs,
    plenoxels_gb300.FusedAdam. Optimiser state then exists only for the shard.

    Per step and rank this moves 2 (N-1)/N times the gradient's bytes, as an all-reduce
    does; the optimiser pass reads and writes 1/N of the grid."""

    def __init__(self, grid: torch.Tensor, make_optimizer, group=None):
        if grid.dtype != torch.float32 or not grid.is_contiguous() or grid.numel() % 4 != 0:
            raise ValueError("ShardedGridUpdate takes a contiguous float32 grid of whole cells")
        self.group = group
        self.world = dist.get_world_size(group) if dist.is_initialized() else 1
        self.rank = dist.get_rank(group) if dist.is_initialized() else 0
        self.grid = grid
        n = grid.numel()
        self.per = 4 * (-(-(n // 4) // self.world))  # padded shard length in floats
        self.start, self.length = grid_shard(n, self.rank, self.world)
        self.padded = self.per * self.world != n
        flat = grid.view(-1)
        dev = grid.device
        self.grad_shard = torch.zeros(self.per, dtype=torch.float32, device=dev)
        self._own = torch.zeros(self.per, dtype=torch.float32, device=dev)
        if self.padded:
            self._send = torch.zeros(self.per * self.world, dtype=torch.float32, device=dev)
            self._gather = torch.zeros(self.per * self.world, dtype=torch.float32, device=dev)
        self.shard = flat[self.start:self.start + self.length]
        self.opt = make_optimizer(self.shard) if self.length > 0 else None

    def step(self, grad: torch.Tensor) -> torch.Tensor:
        """One update from this rank's dense gradient (same shape as the grid). Returns
        the grid."""
        if grad.shape != self.grid.shape or grad.dtype != torch.float32:
            raise ValueError("step needs a float32 gradient of the grid's shape")
        n = self.grid.numel()
        flat_g = grad.contiguous().view(-1)
        if self.padded:
            self._send[:n].copy_(flat_g)
            send = self._send
        else:
            send = flat_g
        if self.world > 1:
            dist.reduce_scatter_tensor(self.grad_shard, send, op=dist.ReduceOp.SUM, group=self.group)
        else:
            self.grad_shard.copy_(send[:self.per])
        if self.opt is not None:
            self.opt.step(self.grad_shard[:self.length])
        if self.world > 1:
            # the own shard goes through a buffer of its own, so the collective's input
            # never aliases its output
            self._own[:self.length].copy_(self.shard)
            if self.padded:
                dist.all_gather_into_tensor(self._gather, self._own, group=self.group)
                self.grid.view(-1).copy_(self._gather[:n])
            else:
                dist.all_gather_into_tensor(self.grid.view(-1), self._own, group=self.group)
        return self.grid
