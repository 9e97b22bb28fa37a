"""Drop-in operators on the GPU against outputs of the reference itself (tests/golden).

Tolerances: ray directions, sample positions, normalised coordinates, voxel indices,
masks and looked-up values are compared bit for bit; composited RGBA within 1e-5
relative; grid gradients within 1e-4 of the largest gradient entry (atomic accumulation
order differs from the reference's sequential index_put)."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
from conftest import load_golden

pytestmark = pytest.mark.gpu

PATH_CASES = ["ref_nearest", "ref_trilinear", "ref_trilinear_saturated", "ref_even_spread",
              "ref_edge_nearest", "ref_edge_trilinear"]
DEV = "cuda"


def _t(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    return t if dtype is None else t.to(dtype)


def _grad_close(got, ref, rel=1e-4):
    scale = np.abs(ref).max()
    err = np.abs(got - ref).max()
    assert err <= rel * scale + 1e-9, f"max grad error {err:.3e} vs scale {scale:.3e}"


def _drop_in_step(d):
    side = int(d["side"])
    pd = float(d["points_distance"])
    coords, cells, _, _ = pg.generate_grid(side, side, side, points_distance=pd, device=DEV)
    with torch.no_grad():
        cells.copy_(_t(d["grid"]))
    T = _t(d["transforms"])
    imgs = _t(d["imgs"])
    C, R, S = T.shape[0], int(d["rays_per_cam"]), int(d["num_samples"])
    even = bool(int(d["even_spread"]))
    uv = None if even else _t(d["uv"])
    samples, pixels, cam_pos, dirs = pg.sample_camera_rays_batched(
        T, float(d["camera_angle_x"]), imgs, R, S, float(d["delta"]), even, False, device=DEV,
        ray_uv=uv)
    n = pg.normalize_samples_for_indecies(coords, samples, pd)
    if str(d["mode"]) == "nearest":
        vals, mask = pg.get_nearest_voxels(n, cells, clip=True)
        idx = torch.round(n).to(torch.long)
        pg.fix_out_of_bounds(idx, cells)
    else:
        idx = pg.get_grid_points_indices(n)
        pg.fix_out_of_bounds(idx.view(-1, 3), cells)
        vals = pg.trilinear_interpolation(n, idx, cells, clip=True)
        mask = pg.find_out_of_bound(n, cells)
    vals = vals * mask.unsqueeze(-1)
    px = pg.compute_alpha_weighted_pixels(vals.reshape(C, R, S, 4)).reshape(C * R, 4)
    loss = torch.nn.functional.mse_loss(px, pixels)
    loss.backward()
    return dict(dirs=dirs, pixels=pixels, samples=samples, normalized=n, index=idx, mask=mask,
                vals=vals, rgba=px, loss=loss, grad=cells.grad, cam_pos=cam_pos)


@pytest.mark.parametrize("case", PATH_CASES)
def test_drop_in_path_matches_reference(case):
    d = load_golden(case)
    o = _drop_in_step(d)
    for key in ["dirs", "pixels", "samples", "normalized", "index", "mask", "vals"]:
        got = o[key].detach().cpu().numpy()
        np.testing.assert_array_equal(got, d[key], err_msg=f"{case}:{key}")
    np.testing.assert_allclose(o["rgba"].detach().cpu().numpy(), d["rgba"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(float(o["loss"].detach()), float(d["loss"]), rtol=1e-5)
    _grad_close(o["grad"].cpu().numpy(), d["grad"])


@pytest.mark.parametrize("case", PATH_CASES)
def test_fused_path_matches_reference(case):
    """render_rays (one kernel) on the reference's rays: same indices, same pixels."""
    d = load_golden(case)
    side = int(d["side"])
    pd = float(d["points_distance"])
    R = d["dirs"].shape[0]
    C = d["transforms"].shape[0]
    S = int(d["num_samples"])
    origins = np.repeat(d["transforms"][:, :3, 3], R // C, axis=0)
    grid = _t(d["grid"]).requires_grad_(True)
    o, dr = _t(origins), _t(d["dirs"])
    idx, inb = pg.render_sample_indices(grid, o, dr, float(d["delta"]), S, pd, mode=str(d["mode"]))
    ref_idx = d["index"].reshape(idx.shape)
    np.testing.assert_array_equal(idx.cpu().numpy(), ref_idx)
    np.testing.assert_array_equal(inb.cpu().numpy().reshape(-1), d["mask"])
    rgba = pg.render_rays(grid, o, dr, float(d["delta"]), S, pd, mode=str(d["mode"]))
    np.testing.assert_allclose(rgba.detach().cpu().numpy(), d["rgba"], rtol=1e-5, atol=1e-6)
    loss = torch.nn.functional.mse_loss(rgba, _t(d["pixels"]))
    loss.backward()
    _grad_close(grid.grad.cpu().numpy(), d["grad"])


def test_fused_train_step_matches_reference():
    d = load_golden("ref_trilinear_saturated")
    pd = float(d["points_distance"])
    R = d["dirs"].shape[0]
    C = d["transforms"].shape[0]
    origins = _t(np.repeat(d["transforms"][:, :3, 3], R // C, axis=0))
    grid = _t(d["grid"]).requires_grad_(True)
    step = pg.FusedTrainStep(grid, pd, int(d["num_samples"]), float(d["delta"]), mode="trilinear")
    rgba = torch.empty(R, 4, device=DEV)
    for _ in range(2):  # the workspace must come back clean after each launch
        loss = step.step_rays(origins, _t(d["dirs"]), _t(d["pixels"]), rgba_out=rgba)
        np.testing.assert_allclose(float(loss), float(d["loss"]), rtol=1e-5)
        np.testing.assert_allclose(rgba.cpu().numpy(), d["rgba"], rtol=1e-5, atol=1e-6)
        _grad_close(step.grad.cpu().numpy(), d["grad"])
    assert grid.grad is step.grad


def test_composite_matches_reference():
    d = load_golden("ref_composite")
    x = _t(d["samples"]).requires_grad_(True)
    out = pg.compute_alpha_weighted_pixels(x)
    out.backward(_t(d["dout"]))
    np.testing.assert_allclose(out.detach().cpu().numpy(), d["out"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(x.grad.cpu().numpy(), d["dsamples"], rtol=1e-4, atol=1e-5)


def test_generate_grid_matches_reference_layout():
    d = load_golden("ref_nearest")
    side = int(d["side"])
    coords, cells, mesh, gg = pg.generate_grid(side, side, side, float(d["points_distance"]), device=DEV)
    assert cells.requires_grad and cells.is_leaf and float(cells.abs().sum()) == 0.0
    np.testing.assert_array_equal(coords.min(0)[0].cpu().numpy(), d["grid_min"])
    assert mesh.dtype == torch.int64 and tuple(mesh[1, 2, 3].tolist()) == (1, 2, 3)
    assert coords.data_ptr() == gg.data_ptr()


def test_collect_cells_matches_reference():
    """collect_cell_information_via_indices (src/grid_functions.py:154-170) against the
    reference's own output: gathered corner values and the float-coordinate mask bit for
    bit, and the autograd gradient of the gathered values."""
    d = load_golden("ref_collect_cells")
    grid = _t(d["grid"]).requires_grad_(True)
    vals, mask = pg.collect_cell_information_via_indices(_t(d["normalized"]), grid)
    vals.backward(_t(d["dvals"]))
    np.testing.assert_array_equal(vals.detach().cpu().numpy(), d["vals"])
    np.testing.assert_array_equal(mask.cpu().numpy(), d["mask"])
    _grad_close(grid.grad.cpu().numpy(), d["grad"])
