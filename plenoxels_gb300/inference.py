"""Checkpoint format and full-image rendering of a trained grid.

save_checkpoint/load_checkpoint read and write the reference's checkpoint dict
(scripts/train.py:197-210; read back by scripts/compare_inference_to_image.py:41-50 and
scripts/visulize_grid.py:23-27): {"grid", "grid_grad", "param": {device, number_of_rays,
num_samples, delta_step, even_spread, camera_ray, points_distance, gridsize}} saved with
torch.save, tensors on the CPU.

visulize_3d_in_2d renders one camera's image as src/visualization.py:111-154 does (grid
clipped to [0,1], optional opacity threshold, side x side even-spread rays from the camera
position, nearest lookup, compositing, uint8 RGBA transposed) in one fused forward launch
and one conversion kernel.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, require_cuda
from .grid_functions import grid_origin
from .ray_sampling import generate_rays_batched
from .render import _rays_desc

PARAM_KEYS = ("device", "number_of_rays", "num_samples", "delta_step", "even_spread",
              "camera_ray", "points_distance", "gridsize")


def save_checkpoint(path, grid, grid_grad, param):
    """Writes the reference's checkpoint dict; param must hold the reference's keys."""
    missing = [k for k in PARAM_KEYS if k not in param]
    if missing:
        raise KeyError(f"checkpoint param lacks {missing}")
    torch.save({"grid": grid.detach().cpu(),
                "grid_grad": grid_grad.detach().cpu() if grid_grad is not None else None,
                "param": dict(param)}, path)


def load_checkpoint(path, device="cuda"):
    """Reads a checkpoint written by the reference or save_checkpoint; the grid and its
    gradient are moved to `device`."""
    data = torch.load(path, map_location="cpu", weights_only=False)
    out = dict(data)
    out["grid"] = data["grid"].to(device)
    if data.get("grid_grad") is not None:
        out["grid_grad"] = data["grid_grad"].to(device)
    return out


@torch.no_grad()
def visulize_3d_in_2d(grid_cells_data, transform_matrices, camera_angle_x, imgs, grid_indices,
                      do_threshold, transparency_threshold, number_of_rays, num_samples, device="cuda"):
    """src/visualization.py:111-154: uint8 [res,res,4] image (numpy), res = sqrt(rays)."""
    grid = grid_cells_data["grid"].detach().to(device).contiguous()
    require_cuda(grid, transform_matrices, imgs)
    if transform_matrices.shape[0] != 1:
        raise ValueError("visulize_3d_in_2d renders one camera (the reference reshapes to 1 x R)")
    param = grid_cells_data["param"]
    pd, delta = float(param["points_distance"]), float(param["delta_step"])
    side = int(np.round(np.sqrt(number_of_rays)))
    R = side * side
    dirs, _ = generate_rays_batched(imgs, R, transform_matrices, camera_angle_x, even_spread=True,
                                    device=device)
    origins = transform_matrices[:, :3, 3].expand(R, 3).contiguous()
    if grid_indices is not None:
        gmin = tuple(float(x) for x in grid_indices.reshape(-1, 3).min(0)[0].tolist())
    else:
        gmin = grid_origin(grid.shape, pd)
    floor = float(transparency_threshold) if do_threshold else 0.0
    gdesc = _lib.make_grid(grid, gmin, pd, _lib.PGB_NEAREST, True, alpha_floor=floor)
    rdesc = _rays_desc(origins, dirs, R, num_samples, delta, False, 0, 0.0)
    rgba = torch.empty(R, 4, dtype=torch.float32, device=grid.device)
    lib = _lib.load()
    s = torch.cuda.current_stream(grid.device).cuda_stream
    check(lib.pgb_render_fwd(gdesc, rdesc, ptr(rgba), s), "visulize_3d_in_2d")
    image = torch.empty(side, side, 4, dtype=torch.uint8, device=grid.device)
    check(lib.pgb_rgba_to_image(ptr(rgba), side, ptr(image), s), "visulize_3d_in_2d")
    return image.cpu().numpy()


@torch.no_grad()
def render_camera_images(grid, transforms, height, width, camera_angle_x, near, delta_step,
                         num_samples, points_distance, mode="trilinear", grid_min=None,
                         stratified=False, seed=0):
    """Premultiplied RGBA images [C, height, width, 4] (float32, on the grid's device) of
    a grid seen from each camera: pixel (row, col) is the composited ray of the uniforms
    u = col / height, v = row / width, the ray that generate_rays_batched
    (src/ray_sampling.py:195-264) maps back to that pixel, started `near` along its
    direction and sampled as the training step samples. One fused forward launch per
    camera. Square images only, as the reference indexes them. No counterpart in the
    reference beyond the per-ray forward it composes (it trains against photographs)."""
    require_cuda(grid, transforms)
    if height != width:
        raise ValueError("render_camera_images renders square images")
    from .render import render_rays
    dev = grid.device
    C, H, W = transforms.shape[0], int(height), int(width)
    rows = torch.arange(H, device=dev, dtype=torch.float32)
    cols = torch.arange(W, device=dev, dtype=torch.float32)
    uv = torch.stack([(cols / H).expand(H, W), (rows / W)[:, None].expand(H, W)], -1).reshape(1, H * W, 2)
    blank = torch.zeros(1, H, W, 4, device=dev)
    out = torch.empty(C, H, W, 4, dtype=torch.float32, device=dev)
    g = grid.detach().contiguous()
    for c in range(C):
        T = transforms[c:c + 1].contiguous()
        dirs, _ = generate_rays_batched(blank, H * W, T, camera_angle_x, device=dev, ray_uv=uv)
        origins = (T[0, :3, 3] + near * dirs).contiguous()
        rgba = render_rays(g, origins, dirs, delta_step, num_samples, points_distance, grid_min,
                           mode=mode, stratified=stratified, seed=seed)
        out[c] = rgba.reshape(H, W, 4)
    return out
