"""Full-image inference render (src/visualization.py:111-154) against the oracle's
composition of the reference's functions: the uint8 image may differ by one level where
255 * rgba lies within the fp32 compositing error of a rounding boundary."""
import numpy as np
import pytest
import torch

import scenes
from oracle import torch_port as tp
import plenoxels_gb300 as pg
from plenoxels_gb300.inference import visulize_3d_in_2d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("do_threshold", [False, True])
def test_image_matches_reference_composition(do_threshold):
    side, S, res = 32, 128, 40
    pd, delta = scenes.points_distance(side), 6.0 / S
    grid = torch.from_numpy(scenes.make_grid(side, 3, 81, amp=(0.2, 2.0), negative_frac=0.05))
    T = torch.from_numpy(scenes.make_cameras(1, 82))
    imgs = torch.zeros(1, res, res, 4)
    data = {"grid": grid, "param": {"points_distance": pd, "delta_step": delta}}
    img = visulize_3d_in_2d(data, T.cuda(), 0.691, imgs.cuda(), None, do_threshold, 0.3, res * res, S)
    # oracle: scripts' composition on the reference's functions
    g = grid.clip(0.0, 1.0)
    if do_threshold:
        g[..., -1][g[..., -1] < 0.3] = 0.0
    d, _ = tp.camera_rays(T, 0.691, imgs, tp.even_uv(1, res))
    o = T[:, :3, 3].expand(res * res, 3)
    px = tp.render(g, o, d, S, delta, tp.grid_min(g.shape, pd), pd, "nearest", clip=False)
    ref = (px.numpy() * 255).round().clip(0, 255).astype(np.uint8).reshape(res, res, 4).transpose(1, 0, 2)
    diff = np.abs(img.astype(int) - ref.astype(int))
    assert diff.max() <= 1 and (diff > 0).mean() < 1e-3
    assert img.shape == (res, res, 4) and img.dtype == np.uint8


def test_camera_images_are_the_renders_of_each_pixels_ray():
    """render_camera_images: pixel (row, col) of camera c is the composited ray of the
    uniforms (col / H, row / W) from that camera, started at near along its direction."""
    import scenes
    from oracle import torch_port as tp
    side, S, H, near = 24, 64, 12, 2.0
    grid = torch.from_numpy(scenes.make_grid(side, 3, 81, amp=(0.3, 3.0), negative_frac=0.02))
    T = torch.from_numpy(scenes.make_cameras(2, 82))
    pd, delta = scenes.points_distance(side), 4.0 / S
    imgs = pg.inference.render_camera_images(grid.cuda(), T.cuda(), H, H, 0.691, near, delta, S, pd)
    assert imgs.shape == (2, H, H, 4)
    rows = torch.arange(H, device="cuda", dtype=torch.float32)
    cols = torch.arange(H, device="cuda", dtype=torch.float32)
    uv = torch.stack([(cols / H).expand(H, H), (rows / H)[:, None].expand(H, H)], -1).reshape(1, H * H, 2).cpu()
    for c in range(2):
        d, _ = tp.camera_rays(T[c:c + 1], 0.691, torch.zeros(1, H, H, 4), uv)
        o = T[c, :3, 3] + near * d
        ref = tp.render(grid, o, d, S, delta, tp.grid_min(grid.shape, pd), pd, "trilinear")
        np.testing.assert_allclose(imgs[c].reshape(-1, 4).cpu().numpy(), ref.numpy(), rtol=1e-5, atol=2e-6)
