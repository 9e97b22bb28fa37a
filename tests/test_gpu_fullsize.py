"""The headline workload at its full size, checked against the oracle: a 256^3 fp32 grid of
16 blobs, 100 cameras of 800x800 at radius 4 whose targets are rendered from a second
seeded ground-truth grid, 8192 in-kernel camera rays per step, 256 stratified samples,
trilinear, near 2 / far 6 (the workload bench.py times, built the same way). Every ray's
cell indices bit-exact, RGBA within 1e-5 relative, the whole-step loss within 1e-5 and the
dense 256^3 gradient within 1e-4 of its largest entry; then a second step on new rays."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes
from oracle import torch_port as tp

pytestmark = pytest.mark.gpu
DEV = "cuda"
SIDE, BLOBS, CAMS, RES, R, S, NEAR, FAR, FOV = 256, 16, 100, 800, 8192, 256, 2.0, 6.0, 0.691


@pytest.fixture(scope="module")
def workload():
    grid = scenes.make_grid_fast(SIDE, BLOBS, 1)
    T = torch.from_numpy(scenes.make_cameras(CAMS, seed=2))
    gt = scenes.make_grid_fast(SIDE, BLOBS, 4)
    imgs = pg.inference.render_camera_images(gt.to(DEV), T.to(DEV), RES, RES, FOV, NEAR,
                                             (FAR - NEAR) / S, S, scenes.points_distance(SIDE))
    return grid, T, imgs.cpu()


@pytest.mark.parametrize("ray_seed", [1005, 2006])
def test_full_size_step_matches_oracle(workload, ray_seed):
    grid, T, imgs = workload
    pd = scenes.points_distance(SIDE)
    delta = (FAR - NEAR) / S
    gmin = tp.grid_min(grid.shape, pd)
    jit = tp.jitter_for(7, R, S)
    o, d, target = tp.camera_batch(T, FOV, imgs, R, ray_seed, NEAR)
    # oracle (CPU, fp32 autograd)
    g_ref = grid.clone().requires_grad_(True)
    px_ref = tp.render(g_ref, o, d, S, delta, gmin, pd, "trilinear", True, jit)
    loss_ref = torch.nn.functional.mse_loss(px_ref, target)
    loss_ref.backward()
    idx_ref, inb_ref = tp.sample_indices(o, d, S, delta, gmin, pd, grid.shape, "trilinear", jit)
    # CUDA: rays generated in-kernel from the resident cameras, as the bench step does
    gd, Td, imgsd = grid.to(DEV), T.to(DEV), imgs.to(DEV)
    idx, inb = pg.render.camera_sample_indices(gd, Td, imgsd, FOV, R, ray_seed, NEAR, delta, S, pd,
                                               mode="trilinear", stratified=True, seed=7)
    assert torch.equal(inb.cpu(), inb_ref.reshape(R, S))
    assert torch.equal(idx.cpu().reshape(-1), idx_ref.reshape(-1))
    del idx, inb, idx_ref, inb_ref
    step = pg.FusedTrainStep(gd, pd, S, delta, mode="trilinear", stratified=True, seed=7)
    rgba = torch.empty(R, 4, device=DEV)
    loss = step.step_cameras(Td, imgsd, FOV, R, ray_seed, near=NEAR, rgba_out=rgba)
    torch.cuda.synchronize()
    np.testing.assert_allclose(rgba.cpu().numpy(), px_ref.detach().numpy(), rtol=1e-5, atol=2e-6)
    np.testing.assert_allclose(float(loss), float(loss_ref), rtol=1e-5)
    ref = g_ref.grad
    err = float((step.grad.cpu() - ref).abs().max())
    assert err <= 1e-4 * float(ref.abs().max()), err


def test_full_size_drop_in_step_matches_oracle(workload):
    """The same workload through the import-swap path (scripts/train.py:129-156 composed
    from the drop-in functions, nearest lookup, autograd backward) with the oracle's rays:
    normalised coordinates bit-exact, RGBA within 1e-5 relative, the dense gradient within
    1e-4 of its largest entry."""
    grid, T, imgs = workload
    pd = scenes.points_distance(SIDE)
    delta = (FAR - NEAR) / S
    gmin = tp.grid_min(grid.shape, pd)
    o, d, target = tp.camera_batch(T, FOV, imgs, R, 3007, NEAR)
    g_ref = grid.clone().requires_grad_(True)
    px_ref = tp.render(g_ref, o, d, S, delta, gmin, pd, "nearest", True, None)
    torch.nn.functional.mse_loss(px_ref, target).backward()
    # drop-in path on the GPU, fed the same rays: sample points, normalisation, lookup
    gi, _, _, _ = pg.generate_grid(SIDE, SIDE, SIDE, pd, device=DEV)
    od, dd = o.to(DEV), d.to(DEV)
    k = torch.arange(1, S + 1, device=DEV, dtype=torch.float32)
    samples = (od.unsqueeze(1) + dd.unsqueeze(1) * (delta * k).unsqueeze(-1)).reshape(-1, 3)
    n = pg.normalize_samples_for_indecies(gi, samples, pd)
    n_ref = tp.normalize(tp.sample_positions(o, d, S, delta, None), gmin, pd)
    assert torch.equal(n.cpu(), n_ref)
    g = grid.to(DEV).requires_grad_(True)
    vals, mask = pg.get_nearest_voxels(n, g, clip=True)
    px = pg.compute_alpha_weighted_pixels((vals * mask.unsqueeze(-1)).reshape(1, R, S, 4)).reshape(R, 4)
    np.testing.assert_allclose(px.detach().cpu().numpy(), px_ref.detach().numpy(), rtol=1e-5, atol=2e-6)
    torch.nn.functional.mse_loss(px, target.to(DEV)).backward()
    ref = g_ref.grad
    err = float((g.grad.cpu() - ref).abs().max())
    assert err <= 1e-4 * float(ref.abs().max()), err
