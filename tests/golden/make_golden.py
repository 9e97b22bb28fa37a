"""Generates the golden fixtures in this folder by running the REFERENCE's own functions
(DanJbk/Plenoxels) on seeded synthetic inputs, on CPU.

Run where a checkout of the reference exists, naming its root directory:
    PLENOXELS_REFERENCE=<path to the reference checkout> python tests/golden/make_golden.py

The reference imports PIL through src/data_processing.py:3 only to read PNG files, and
src/visualization.py imports matplotlib and plotly only for its plots; stub modules stand
in for them (no reference file is modified, and no stubbed function is called). Each
fixture stores the inputs, the reference's outputs and the reference autograd gradient.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("PLENOXELS_REFERENCE")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("set PLENOXELS_REFERENCE to the root of a DanJbk/Plenoxels checkout")
sys.path.insert(0, os.path.dirname(HERE))  # tests/
sys.modules.setdefault("PIL", types.ModuleType("PIL"))
sys.modules["PIL"].Image = None
# plotting modules of src/visualization.py:1-6 (only its plot functions use them)
for _name in ("matplotlib", "matplotlib.pyplot", "matplotlib.colors", "plotly",
              "plotly.graph_objs", "plotly.io"):
    sys.modules.setdefault(_name, types.ModuleType(_name))
sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
sys.modules["matplotlib"].colors = sys.modules["matplotlib.colors"]
sys.modules["plotly"].graph_objs = sys.modules["plotly.graph_objs"]
sys.modules["plotly"].io = sys.modules["plotly.io"]
sys.path.insert(0, REF)

import scenes  # noqa: E402
from src.grid_functions import (collect_cell_information_via_indices,  # noqa: E402
                                convolve_grid_to_remove_noise, fix_out_of_bounds,
                                find_out_of_bound, generate_grid, get_grid_points_indices,
                                get_nearest_voxels, trilinear_interpolation)
from src.ray_sampling import (compute_alpha_weighted_pixels, normalize_samples_for_indecies,  # noqa: E402
                              sample_camera_rays_batched)
from src.visualization import visulize_3d_in_2d_fast  # noqa: E402


def _np(t):
    return t.detach().cpu().numpy()


def reference_step(grid_np, transforms, imgs, rays_per_cam, num_samples, delta, side, mode,
                   uv_seed, even_spread=False):
    """One step of scripts/train.py:130-181 on the reference's functions, with the
    lookup chosen by mode; returns a dict of inputs and outputs."""
    pd = scenes.points_distance(side)
    grid_coords, cells, _, _ = generate_grid(side, side, side, points_distance=pd, device="cpu")
    with torch.no_grad():
        cells.copy_(torch.from_numpy(grid_np))
    T = torch.from_numpy(transforms)
    I = torch.from_numpy(imgs)
    C = T.shape[0]
    uv = None
    if not even_spread:
        torch.manual_seed(uv_seed)
        uv = torch.rand(C, rays_per_cam, 2)
        torch.manual_seed(uv_seed)
    samples, pixels, cam_pos, dirs = sample_camera_rays_batched(
        transform_matrices=T, camera_angle_x=0.691, imgs=I, number_of_rays=rays_per_cam,
        num_samples=num_samples, delta_step=delta, even_spread=even_spread, camera_ray=False,
        device="cpu")
    R = dirs.shape[0] // C
    n = normalize_samples_for_indecies(grid_coords, samples, pd)
    if mode == "nearest":
        vals, mask = get_nearest_voxels(n, cells.clip(0, 1))
        idx = torch.round(n).to(torch.long)
        fix_out_of_bounds(idx, cells)
    else:
        idx = get_grid_points_indices(n)
        fix_out_of_bounds(idx.view(-1, 3), cells)
        vals = trilinear_interpolation(n, idx, cells.clip(0, 1))
        mask = find_out_of_bound(n, cells)
    vals = vals * mask.unsqueeze(-1)
    px = compute_alpha_weighted_pixels(vals.reshape(C, R, num_samples, 4)).reshape(C * R, 4)
    loss = torch.nn.functional.mse_loss(px, pixels)
    loss.backward()
    out = dict(grid=grid_np, transforms=transforms, imgs=imgs, side=side, points_distance=pd,
               rays_per_cam=R, num_samples=num_samples, delta=delta, camera_angle_x=0.691,
               even_spread=int(even_spread), mode=mode,
               samples=_np(samples), pixels=_np(pixels), dirs=_np(dirs), normalized=_np(n),
               grid_min=_np(grid_coords.min(0)[0]), index=_np(idx), mask=_np(mask),
               vals=_np(vals), rgba=_np(px), loss=_np(loss), grad=_np(cells.grad))
    if uv is not None:
        out["uv"] = _np(uv)
    return out


def composite_case(seed):
    rng = np.random.default_rng(seed)
    s = rng.random((2, 5, 40, 4)).astype(np.float32)
    s[..., 3] = np.where(rng.random((2, 5, 40)) < 0.1, 1.0, s[..., 3] * 0.3)  # saturation
    s[0, 0, :, 3] = 0.0  # fully transparent ray
    s[1, 4, 0, 3] = 1.0  # opaque first sample
    x = torch.from_numpy(s).requires_grad_(True)
    out = compute_alpha_weighted_pixels(x)
    g = torch.from_numpy(rng.standard_normal(out.shape).astype(np.float32))
    out.backward(g)
    return dict(samples=s, out=_np(out), dout=_np(g), dsamples=_np(x.grad))


def edge_case(mode):
    """Axis-aligned rays on a power-of-two pitch: nearest rounding ties at .5, trilinear
    integer coordinates and upper-face wrap, samples before and beyond the box, alpha
    saturation after the clip."""
    side = 8
    grid = scenes.make_grid(side, 2, seed=7, amp=(0.5, 3.0), negative_frac=0.1)
    pd = 0.25  # box [-0.75, 1.0]
    T = np.stack([scenes.look_at(np.array(p, dtype=np.float64)) for p in
                  ([0.0, 0.0, 3.0], [3.0, 0.0, 0.01], [0.01, 3.0, 0.0])])
    imgs = scenes.make_images(3, 4, 4, seed=8)
    grid_coords, cells, _, _ = generate_grid(side, side, side, points_distance=pd, device="cpu")
    with torch.no_grad():
        cells.copy_(torch.from_numpy(grid))
    Tt = torch.from_numpy(T)
    samples, pixels, _, dirs = sample_camera_rays_batched(
        transform_matrices=Tt, camera_angle_x=0.691, imgs=torch.from_numpy(imgs),
        number_of_rays=9, num_samples=56, delta_step=0.125, even_spread=True, camera_ray=False,
        device="cpu")
    n = normalize_samples_for_indecies(grid_coords, samples, pd)
    if mode == "nearest":
        vals, mask = get_nearest_voxels(n, cells.clip(0, 1))
        idx = torch.round(n).to(torch.long)
        fix_out_of_bounds(idx, cells)
    else:
        idx = get_grid_points_indices(n)
        fix_out_of_bounds(idx.view(-1, 3), cells)
        vals = trilinear_interpolation(n, idx, cells.clip(0, 1))
        mask = find_out_of_bound(n, cells)
    vals = vals * mask.unsqueeze(-1)
    px = compute_alpha_weighted_pixels(vals.reshape(3, 9, 56, 4)).reshape(27, 4)
    loss = torch.nn.functional.mse_loss(px, pixels)
    loss.backward()
    return dict(grid=grid, transforms=T, imgs=imgs, side=side, points_distance=pd, rays_per_cam=9,
                num_samples=56, delta=0.125, camera_angle_x=0.691, even_spread=1, mode=mode,
                samples=_np(samples), pixels=_np(pixels), dirs=_np(dirs), normalized=_np(n),
                grid_min=_np(grid_coords.min(0)[0]), index=_np(idx), mask=_np(mask),
                vals=_np(vals), rgba=_np(px), loss=_np(loss), grad=_np(cells.grad))


def collect_cells_case(seed):
    """collect_cell_information_via_indices (src/grid_functions.py:154-170) on a non-cubic
    grid: coordinates inside, on integer values, in (dim-1, dim) (upper-face wrap),
    negative and beyond the grid, and the autograd gradient of its gathered values."""
    rng = np.random.default_rng(seed)
    dims = (7, 5, 6)
    grid = rng.uniform(-0.2, 1.2, dims + (4,)).astype(np.float32)
    n = rng.uniform(-1.5, 1.0, (160, 3)) * np.array(dims) + np.array(dims) * 0.25
    n[:20] = np.round(n[:20])                                 # integer coordinates
    n[20:40] = np.array(dims) - rng.uniform(0.0, 1.0, (20, 3))  # upper faces
    n[40] = [-0.5, 2.5, 3.0]                                  # negative fraction
    n = n.astype(np.float32)
    B = torch.from_numpy(grid.copy()).requires_grad_(True)
    vals, mask = collect_cell_information_via_indices(torch.from_numpy(n.copy()), B)
    dout = rng.standard_normal(vals.shape).astype(np.float32)
    vals.backward(torch.from_numpy(dout))
    return dict(grid=grid, normalized=n, vals=_np(vals), mask=_np(mask), dvals=dout,
                grad=_np(B.grad))


def remove_noise_case(seed):
    """convolve_grid_to_remove_noise (src/grid_functions.py:270-280) for three kernels."""
    rng = np.random.default_rng(seed)
    grid = rng.random((20, 18, 22, 4)).astype(np.float32)
    keep = rng.random((20, 18, 22)) < 0.4
    grid[..., 3] = np.where(keep, rng.random((20, 18, 22)), 0.0).astype(np.float32)
    out = dict(grid=grid)
    for i, (k, r, t) in enumerate([(3, 1.0, 2.0), (5, 1.5, 3.0), (3, 2.0, 4.5)]):
        g = torch.from_numpy(grid.copy())
        res = convolve_grid_to_remove_noise(g, kernel_size=k, radius=r, threshold=t, repeats=6)
        out[f"params_{i}"] = np.array([k, r, t])
        out[f"out_{i}"] = _np(res)
    return out


def splat_case(seed):
    """visulize_3d_in_2d_fast (src/visualization.py:157-232) of a 48^3 blob grid."""
    side = 48
    grid = scenes.make_grid(side, 4, seed, amp=(0.05, 0.6))
    grid[grid[..., 3] <= 0.1] = 0.0  # cells the preview never draws: zeros compress
    T = scenes.make_cameras(2, seed + 1)
    out = dict(grid=grid, transforms=T, points_distance=scenes.points_distance(side),
               camera_angle_x=0.691, size_y=64)
    for c in range(T.shape[0]):
        img = visulize_3d_in_2d_fast(torch.from_numpy(grid), scenes.points_distance(side),
                                     torch.from_numpy(T[c]), 0.691, 64)
        out[f"img_{c}"] = np.asarray(img)
    return out


def main():
    torch.set_num_threads(1)
    cases = {}
    cams = scenes.make_cameras(2, seed=11)
    imgs = scenes.make_images(2, 16, 16, seed=12)
    g_soft = scenes.make_grid(16, 3, seed=13, amp=(0.2, 2.0), negative_frac=0.05)
    cases["ref_nearest"] = reference_step(g_soft, cams, imgs, 24, 48, 0.125, 16, "nearest", 101)
    cases["ref_trilinear"] = reference_step(g_soft, cams, imgs, 24, 48, 0.125, 16, "trilinear", 102)
    g_hard = scenes.make_grid(24, 3, seed=14)  # amplitudes 5..20: alpha saturates after clip
    cams3 = scenes.make_cameras(3, seed=15)
    imgs3 = scenes.make_images(3, 20, 20, seed=16)
    cases["ref_trilinear_saturated"] = reference_step(g_hard, cams3, imgs3, 16, 96, 0.0625, 24,
                                                      "trilinear", 103)
    cases["ref_even_spread"] = reference_step(g_soft, cams, imgs, 36, 40, 0.15, 16, "nearest", 0,
                                              even_spread=True)
    cases["ref_edge_nearest"] = edge_case("nearest")
    cases["ref_edge_trilinear"] = edge_case("trilinear")
    cases["ref_composite"] = composite_case(21)
    cases["ref_collect_cells"] = collect_cells_case(31)
    cases["ref_remove_noise"] = remove_noise_case(32)
    cases["ref_splat"] = splat_case(33)
    for name, d in cases.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(f"{path}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
