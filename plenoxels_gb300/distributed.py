"""Ray-sharded data parallelism for the fused training step.

Rays are independent, so each rank renders its own share of the step's rays against a
replicated grid; the only exchange is one sum all-reduce of the dense gradient per step.
Each rank weights its MSE by its share of the global ray count, so the summed gradient
and the summed loss equal the single-process ones (scripts/train.py:156 takes the mean
over all rays of the step).
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
