"""The reference's own CPU-runnable configuration through the fused kernels: a dense 64^3
grid (RGB = sigmoid(N(0,1)), opacity = ReLU of 3 Gaussian blobs of amplitude 5..20), one
camera at radius 4 with a 64x64 image (every pixel one even-spread ray), near 2, far 6,
128 samples, nearest lookup, white background, MSE against a target rendered from a
second seeded grid, one forward + backward step. Checked against the oracle (fp32
autograd): loss and pixels within 1e-5 relative, gradient within 1e-4 of its largest
entry, and with the background term's adjoint through alpha."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes
from oracle import torch_port as tp

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _scene_64cube():
    side, res, S, near, far = 64, 64, 128, 2.0, 6.0
    grid = torch.from_numpy(scenes.make_grid(side, 3, 1000))
    truth = torch.from_numpy(scenes.make_grid(side, 3, 2000))
    T = torch.from_numpy(scenes.make_cameras(1, 3000))
    imgs = torch.zeros(1, res, res, 4)
    d, _ = tp.camera_rays(T, 0.691, imgs, tp.even_uv(1, res))
    o = T[:, :3, 3].expand(res * res, 3) + near * d
    pd = scenes.points_distance(side)
    delta = (far - near) / S
    gmin = tp.grid_min(grid.shape, pd)
    white = (1.0, 1.0, 1.0)
    target = tp.render(truth, o, d, S, delta, gmin, pd, "nearest", background=white)
    return grid, o, d, target, S, delta, pd, gmin, white


@pytest.mark.parametrize("background", [True, False])
def test_white_background_step_matches_oracle(background):
    grid, o, d, target, S, delta, pd, gmin, white = _scene_64cube()
    bg = white if background else None
    g = grid.clone().requires_grad_(True)
    px_ref = tp.render(g, o, d, S, delta, gmin, pd, "nearest", background=bg)
    loss_ref = torch.nn.functional.mse_loss(px_ref, target)
    loss_ref.backward()
    # autograd path (render_rays) and the fused step must both agree
    gg = grid.to(DEV).requires_grad_(True)
    px = pg.render_rays(gg, o.to(DEV), d.to(DEV), delta, S, pd, mode="nearest", background=bg)
    np.testing.assert_allclose(px.detach().cpu().numpy(), px_ref.detach().numpy(), rtol=1e-5, atol=2e-6)
    torch.nn.functional.mse_loss(px, target.to(DEV)).backward()
    scale = float(g.grad.abs().max())
    assert float((gg.grad.cpu() - g.grad).abs().max()) <= 1e-4 * scale
    step = pg.FusedTrainStep(grid.to(DEV), pd, S, delta, mode="nearest", background=bg)
    loss = step.step_rays(o.to(DEV), d.to(DEV), target.to(DEV))
    np.testing.assert_allclose(float(loss), float(loss_ref), rtol=1e-5)
    assert float((step.grad.cpu() - g.grad).abs().max()) <= 1e-4 * scale
