"""The fused training step under ray-sharded data parallelism, on the GPU.

Two processes share the one GPU. Each runs the product FusedTrainStep on its contiguous
share of the rays with its MSE weighted by its share of the global ray count
(distributed.shard_rays / loss_weight) and its offset in the batch's stratification
stream (first_ray). Their gradients and losses are summed over a
gloo group on CPU copies, and the sums must equal one process running the same step on
all rays (scripts/train.py:156 takes the mean over all rays). No kernel waits on another
process: the only exchange is the host-side sum after each process's step has finished.

Tolerances: loss within 1e-6 relative, gradient within 1e-5 of its largest entry (atomic
accumulation order differs between the runs)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _scene():
    import scenes
    from oracle import torch_port as tp
    side, S, R = 32, 96, 301  # ragged: 301 rays over the ranks
    grid = torch.from_numpy(scenes.make_grid(side, 3, 51, amp=(0.3, 3.0), negative_frac=0.02))
    T = torch.from_numpy(scenes.make_cameras(3, 52))
    imgs = torch.from_numpy(scenes.make_images(3, 16, 16, 53))
    o, d, tgt = tp.camera_batch(T, 0.691, imgs, R, 54, 2.0)
    return grid, o, d, tgt, side, S


def _step(grid, o, d, tgt, side, S, weight, mode, first_ray=0):
    import plenoxels_gb300 as pg
    st = pg.FusedTrainStep(grid.cuda(), 3.0 / side, S, 4.0 / S, mode=mode, stratified=True,
                           seed=5, loss_weight=weight)
    loss = st.step_rays(o.cuda(), d.cuda(), tgt.cuda(), first_ray=first_ray)
    torch.cuda.synchronize()
    return float(loss), st.grad.cpu()


def _rank_main(rank, world, port, out, mode):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from plenoxels_gb300.distributed import allreduce_gradient, loss_weight, shard_rays
    torch.cuda.set_device(0)
    grid, o, d, tgt, side, S = _scene()
    start, count = shard_rays(o.shape[0], rank, world)
    sl = slice(start, start + count)
    loss, grad = _step(grid, o[sl], d[sl], tgt[sl], side, S, loss_weight(count, o.shape[0]), mode,
                       first_ray=start)
    allreduce_gradient(grad)
    lsum = torch.tensor([loss], dtype=torch.float64)
    dist.all_reduce(lsum)
    if rank == 0:
        np.save(out + ".grad.npy", grad.numpy())
        np.save(out + ".loss.npy", lsum.numpy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("mode", ["trilinear", "nearest"])
def test_two_process_fused_step_equals_single_process(tmp_path, mode):
    out = str(tmp_path / "r")
    mp.start_processes(_rank_main, args=(2, _free_port(), out, mode), nprocs=2,
                       start_method="spawn")
    grid, o, d, tgt, side, S = _scene()
    loss, grad = _step(grid, o, d, tgt, side, S, 1.0, mode)
    got = np.load(out + ".grad.npy")
    ref = grad.numpy()
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    np.testing.assert_allclose(np.load(out + ".loss.npy")[0], loss, rtol=1e-6)
