"""The data-parallel design on CPU gloo ranks: each rank takes its shard of the rays,
weights its loss by its share, computes the gradient (oracle, CPU) and the ranks sum
gradients with one all-reduce; the result equals the single-process gradient."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from plenoxels_gb300.distributed import allreduce_gradient, loss_weight, shard_rays


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _scene():
    import scenes
    from oracle import torch_port as tp
    side, S, R = 16, 32, 37  # ragged: 37 rays over the ranks
    grid = torch.from_numpy(scenes.make_grid(side, 2, 5, amp=(0.2, 1.5)))
    T = torch.from_numpy(scenes.make_cameras(2, 6))
    imgs = torch.from_numpy(scenes.make_images(2, 8, 8, 7))
    o, d, tgt = tp.camera_batch(T, 0.691, imgs, R, 8, 2.0)
    return grid, o, d, tgt, side, S


def _rank_main(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import torch_port as tp
    grid, o, d, tgt, side, S = _scene()
    start, count = shard_rays(o.shape[0], rank, world)
    pd = 3.0 / side
    g = grid.clone().requires_grad_(True)
    loss = tp.train_loss(g, o[start:start + count], d[start:start + count], tgt[start:start + count],
                         S, 4.0 / S, tp.grid_min(grid.shape, pd), pd)
    (loss * loss_weight(count, o.shape[0])).backward()
    grad = allreduce_gradient(g.grad)
    lsum = torch.tensor([float(loss) * loss_weight(count, o.shape[0])])
    dist.all_reduce(lsum)
    if rank == 0:
        np.save(out + ".grad.npy", grad.numpy())
        np.save(out + ".loss.npy", lsum.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_shard_rays_covers_every_ray_once():
    for R in (0, 1, 7, 8192, 8193):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                s, c = shard_rays(R, r, world)
                seen.extend(range(s, s + c))
            assert seen == list(range(R))


def test_two_rank_gradient_equals_single_process(tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from oracle import torch_port as tp
    out = str(tmp_path / "r")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    grid, o, d, tgt, side, S = _scene()
    pd = 3.0 / side
    g = grid.clone().requires_grad_(True)
    loss = tp.train_loss(g, o, d, tgt, S, 4.0 / S, tp.grid_min(grid.shape, pd), pd)
    loss.backward()
    grad = np.load(out + ".grad.npy")
    assert np.abs(grad - g.grad.numpy()).max() <= 1e-6 * np.abs(g.grad.numpy()).max()
    np.testing.assert_allclose(np.load(out + ".loss.npy")[0], float(loss), rtol=1e-6)


class _TorchAdamShard:
    """Test-side local optimiser for ShardedGridUpdate on CPU ranks: torch.optim.Adam
    (the reference's optimiser, scripts/train.py:89) over the rank's shard."""

    def __init__(self, shard):
        self.shard = shard
        self.param = torch.nn.Parameter(shard.detach().clone())
        self.opt = torch.optim.Adam([self.param], lr=0.0075, foreach=False)

    def step(self, grad):
        self.param.grad = grad.clone()
        self.opt.step()
        with torch.no_grad():
            self.shard.copy_(self.param)


def _sharded_rank_main(rank, world, port, out, shape, steps):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from plenoxels_gb300.distributed import ShardedGridUpdate
    g = torch.Generator().manual_seed(0)
    grid = torch.rand(shape, generator=g)  # replicated: the same seed on every rank
    upd = ShardedGridUpdate(grid, _TorchAdamShard)
    for i in range(steps):
        # each rank's own gradient (seeded by rank and step)
        gr = torch.Generator().manual_seed(1000 * i + rank)
        upd.step(torch.randn(shape, generator=gr) * 10.0 ** (-i))
    np.save(out + f".rank{rank}.npy", grid.numpy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,shape", [(2, (6, 5, 4, 4)), (3, (7, 5, 3, 4))])
def test_sharded_update_equals_single_process_adam(tmp_path, world, shape):
    """Reduce-scatter -> Adam on each rank's shard -> all-gather equals one process
    running Adam on the summed gradient, on every rank, bit for bit (the shards cover
    every cell once; the 7x5x3 grid does not divide into 3 equal shards)."""
    steps = 3
    out = str(tmp_path / "s")
    mp.start_processes(_sharded_rank_main, args=(world, _free_port(), out, shape, steps),
                       nprocs=world, start_method="spawn")
    g = torch.Generator().manual_seed(0)
    p = torch.nn.Parameter(torch.rand(shape, generator=g))
    opt = torch.optim.Adam([p], lr=0.0075, foreach=False)
    for i in range(steps):
        total = torch.zeros(shape)
        for r in range(world):
            gr = torch.Generator().manual_seed(1000 * i + r)
            total += torch.randn(shape, generator=gr) * 10.0 ** (-i)
        p.grad = total
        opt.step()
    for r in range(world):
        got = np.load(out + f".rank{r}.npy")
        np.testing.assert_allclose(got, p.detach().numpy(), rtol=0, atol=1e-7)


def test_grid_shards_cover_every_cell_once():
    from plenoxels_gb300.distributed import grid_shard
    for numel in (4, 16, 4 * 105, 4 * 256 ** 3):
        for world in (1, 2, 3, 8):
            seen = 0
            for r in range(world):
                s, n = grid_shard(numel, r, world)
                assert s % 4 == 0 and n % 4 == 0 and s == seen
                seen += n
            assert seen == numel
