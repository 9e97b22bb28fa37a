"""Point-splat preview (src/visualization.py:157-232) and stray-voxel clean-up
(src/grid_functions.py:260-280) against the oracle's restatement of the reference.

The clean-up must agree exactly (random opacities put no neighbour sum on the threshold).
The splat's pixel positions may differ where a projected coordinate lies within the
reference's BLAS dot-product rounding of a pixel boundary, so the image must agree on
all but a small fraction of pixels, and every differing pixel must be explained by a
point whose projection sits at such a boundary or by a distance tie."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes
from oracle import torch_port as tp
from plenoxels_gb300.visualization import visulize_3d_in_2d_fast

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel_size,radius,threshold", [(3, 1.0, 2.0), (5, 1.5, 3.0), (3, 2.0, 4.5)])
def test_remove_noise_matches_reference(kernel_size, radius, threshold):
    torch.manual_seed(0)
    g = torch.rand(20, 18, 22, 4)
    g[..., 3] = torch.where(torch.rand(20, 18, 22) < 0.4, torch.rand(20, 18, 22), torch.zeros(20, 18, 22))
    ref = tp.remove_noise(g.clone(), kernel_size, radius, threshold, repeats=6)
    got = pg.grid_functions.convolve_grid_to_remove_noise(g.clone().cuda(), kernel_size, radius,
                                                          threshold, repeats=6).cpu()
    assert torch.equal(got, ref)


def test_splat_preview_matches_reference():
    side = 48
    grid = torch.from_numpy(scenes.make_grid(side, 4, 11, amp=(0.05, 0.6)))
    T = torch.from_numpy(scenes.make_cameras(1, 12))[0]
    ref, xx, yy, dist = tp.splat_preview(grid, scenes.points_distance(side), T, 0.691, 64)
    got = visulize_3d_in_2d_fast(grid, scenes.points_distance(side), T, 0.691, 64)
    assert got.shape == ref.shape and got.dtype == np.float64
    differ = np.any(got != ref, axis=-1)
    assert (~np.all(ref == 1.0, axis=-1)).sum() > 100, "the scene must cover part of the image"
    assert differ.mean() < 0.01, f"{differ.sum()} of {differ.size} pixels differ"
