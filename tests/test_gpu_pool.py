"""Coarse-to-fine pooling (src/grid_functions.py:173-181) and the progressive-growing
training steps (scripts/train.py:91-123) against torch's avg_pool3d and the reference's
loop. Pooled values within 1e-5 relative (separable sums in another order), the adjoint
within 1e-5 of its largest entry, loss trajectories within 1e-4 relative."""
import math

import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes
from oracle import torch_port as tp
from plenoxels_gb300.train import Trainer

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.mark.parametrize("shape,r,s", [((32, 32, 32, 4), 9, 2), ((40, 33, 27, 4), 7, 1),
                                       ((64, 64, 64, 4), 31, 7), ((20, 20, 20, 4), 3, None)])
def test_average_pool_matches_avg_pool3d(shape, r, s):
    torch.manual_seed(0)
    grid = torch.rand(shape, device=DEV)
    ref_in = grid.clone().requires_grad_(True)
    ref = tp.average_pool3d_grid(ref_in, r, s)
    g = grid.clone().requires_grad_(True)
    out = pg.average_pool3d_grid(g, r, s)
    assert out.shape == ref.shape
    np.testing.assert_allclose(out.detach().cpu().numpy(), ref.detach().cpu().numpy(), rtol=1e-5, atol=1e-6)
    w = torch.randn_like(ref)
    (ref * w).sum().backward()
    (out * w).sum().backward()
    scale = float(ref_in.grad.abs().max())
    assert float((g.grad - ref_in.grad).abs().max()) <= 1e-5 * scale


def test_progressive_growing_steps_follow_the_reference_loop():
    side, S, R = 32, 64, 300
    grid0 = torch.from_numpy(scenes.make_grid(side, 3, 91, amp=(0.2, 1.5)))
    T = torch.from_numpy(scenes.make_cameras(4, 92))
    imgs = torch.from_numpy(scenes.make_images(4, 8, 8, 93))
    pd0, delta, lr, tv, beta = scenes.points_distance(side), 4.0 / S, 0.0075, 1e-5, 5e-3
    fields, per = [21, 17, 9, 5, 3], 1
    coords = tp.grid_world_coords(grid0.shape, pd0)
    ref = grid0.clone().requires_grad_(True)
    topt = torch.optim.Adam([ref], lr=lr)
    grid = grid0.to(DEV)
    trainer = Trainer(grid, pd0, S, delta, lr, tv=tv, beta=beta, mode="nearest",
                      progressive_growing=True, fields=fields, steps_per_field=per)
    for i in range(7):  # five pooled fields, then two full-grid steps
        o, d, tgt = tp.camera_batch(T, 0.691, imgs, R, 120 + i, 2.0)
        r = fields[i // per] if i // per < len(fields) else 0
        topt.zero_grad()
        if r > 1:  # scripts/train.py:110-118
            stride = max(1, r // 4)
            start = int(r / 2)
            gmin = coords[start::stride, start::stride, start::stride].reshape(-1, 3).min(0)[0]
            cells = tp.average_pool3d_grid(ref, r, stride)
            pd = pd0 * stride
        else:
            gmin, cells, pd = coords.reshape(-1, 3).min(0)[0], ref, pd0
        px, vals = tp.render_samples(cells, o, d, S, delta, gmin, pd, "nearest")
        mse = torch.nn.functional.mse_loss(px, tgt)
        tvl = tv * tp.tv_loss(cells) if r < 19 else torch.zeros(())
        bl = beta * tp.beta_loss(vals[..., -1])
        (mse + tvl + bl).backward()
        topt.step()
        losses = trainer.step_rays(o.to(DEV), d.to(DEV), tgt.to(DEV)).cpu()
        np.testing.assert_allclose(losses.numpy(), [float(mse), float(tvl), float(bl)], rtol=1e-4,
                                   atol=1e-9)
    diff = (grid.cpu() - ref.detach()).abs()
    assert float(diff.max()) <= 7 * lr
    assert float((diff > 1e-5).float().mean()) < 0.01
