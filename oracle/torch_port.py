"""ORACLE — test infrastructure, not part of the product.

A restatement, in PyTorch tensor ops, of the reference's render path (DanJbk/Plenoxels,
paths below relative to that repository). It is the checker for the CUDA kernels and the
timed CPU baseline; only tests, the smoke check and the benchmark's baseline legs use it.

It evaluates the same ATen ops in the same order as the reference, so on CPU its fp32
results are bit-identical to the reference's (pinned by tests/golden, which holds
outputs of the reference itself). Every function is dtype-generic: called with float64
tensors it is the fp64 oracle.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .hash import stratified_jitter, camera_uniforms


# ----------------------------------------------------------------------- grid layout
def grid_world_coords(shape, points_distance: float, dtype=torch.float32, device="cpu"):
    """World coordinates [X,Y,Z,3] of every cell: (i - ceil(s/2) + 1) * pd.
    src/grid_functions.py:198-211 (generate_grid)."""
    axes = [torch.arange(s, device=device) for s in shape[:3]]
    grids = torch.meshgrid(*axes, indexing="ij")
    cols = []
    for g, s in zip(grids, shape[:3]):
        c = g.to(dtype) - float(np.ceil(s / 2)) + 1
        cols.append(c * points_distance)
    return torch.stack(cols, dim=-1)


def grid_min(shape, points_distance: float, dtype=torch.float32):
    """Per-axis min of the coordinate table as a [3] tensor (the value :13 subtracts)."""
    return torch.stack([
        (torch.tensor(1 - math.ceil(s / 2), dtype=dtype) * points_distance) for s in shape[:3]])


# ----------------------------------------------------------------------- rays
def _plain_norm3(v):
    """sqrt((x*x + y*y) + z*z) over the last dim of [N,3], each op rounded separately."""
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    return ((x * x + y * y) + z * z).sqrt()


def camera_rays(transforms, camera_angle_x, imgs, uv):
    """Directions and target pixels of camera rays from uniforms uv [C,R,2].
    src/ray_sampling.py:212-264 (generate_rays_batched), same op order."""
    C, R = uv.shape[0], uv.shape[1]
    x_axis = transforms[:, :3, 0]
    y_axis = transforms[:, :3, 1]
    z_axis = -transforms[:, :3, 2]
    # torch's norm over these strided views rounds every op on x86 (where the golden
    # fixtures were made from the reference) but contracts to FMAs on aarch64; the
    # explicit form below is the x86 rounding on every platform
    aspect = _plain_norm3(x_axis) / _plain_norm3(y_axis)
    ray = uv.clone()
    pix = uv.clone()
    ray[:, :, 0] = camera_angle_x * (ray[:, :, 0] - 0.5)
    ray[:, :, 1] = -((camera_angle_x * (1 / aspect)).unsqueeze(1) * (ray[:, :, 1] - 0.5))
    pix[:, :, 0] = (imgs.shape[1] * pix[:, :, 0]).round().clamp(max=imgs.shape[1] - 1)
    pix[:, :, 1] = (imgs.shape[2] * pix[:, :, 1]).round().clamp(max=imgs.shape[2] - 1)
    pix = pix.to(torch.long).reshape(C * R, 2)
    cam = torch.repeat_interleave(torch.arange(C, device=uv.device), R, 0)
    target = imgs[cam, pix[:, 1], pix[:, 0]]
    u = ray[:, :, 0].unsqueeze(-1).expand(C, R, 3)
    v = ray[:, :, 1].unsqueeze(-1).expand(C, R, 3)
    d = (u * x_axis.unsqueeze(1).expand(C, R, 3) + v * y_axis.unsqueeze(1).expand(C, R, 3)
         + z_axis.unsqueeze(1).expand(C, R, 3))
    d = d / d.norm(dim=2).unsqueeze(-1)
    return d.reshape(C * R, 3), target


def even_uv(num_cameras: int, side: int, device="cpu"):
    """uv of the even-spread rays: cartesian_prod(linspace(0,1,side), same), per camera.
    src/ray_sampling.py:220-223."""
    l = torch.linspace(0, end=1, steps=side, device=device)
    return torch.cartesian_prod(l, l).repeat([num_cameras, 1, 1])


def camera_batch(transforms, camera_angle_x, imgs, num_rays: int, seed: int, near: float):
    """The in-kernel camera ray batch: rays camera-major (ray r -> camera r*C//R), pixel
    uniforms from the counter hash, origin moved to near along the ray. Returns
    (origins [R,3], dirs [R,3], target [R,4])."""
    C = transforms.shape[0]
    cam = (np.arange(num_rays, dtype=np.int64) * C) // max(num_rays, 1)
    u, v = camera_uniforms(seed, num_rays)
    dirs = torch.empty(num_rays, 3, dtype=torch.float32)
    target = torch.empty(num_rays, 4, dtype=torch.float32)
    for c in range(C):
        sel = np.nonzero(cam == c)[0]
        if len(sel) == 0:
            continue
        uv = torch.from_numpy(np.stack([u[sel], v[sel]], -1)).unsqueeze(0)
        d, t = camera_rays(transforms[c:c + 1].cpu(), camera_angle_x, imgs[c:c + 1].cpu(), uv)
        dirs[torch.from_numpy(sel)] = d
        target[torch.from_numpy(sel)] = t
    pos = transforms[:, :3, 3].cpu()[torch.from_numpy(cam)]
    origins = pos + near * dirs
    return origins, dirs, target


# ----------------------------------------------------------------------- sampling
def sample_positions(origins, dirs, num_samples: int, delta_step: float, jitter=None):
    """[R*S,3] sample points o + d * (delta * k), k = 1..S, sample-minor.
    src/ray_sampling.py:161-167. jitter [R,S] (stratified harness) gives
    t = delta * (k - j)."""
    R = origins.shape[0]
    # k in the rays' dtype: for fp32 this is exactly the reference's int64 arange promoted
    # to the default fp32 dtype; for fp64 it keeps t in fp64
    k = torch.arange(num_samples + 1, device=origins.device)[1:].to(origins.dtype)
    if jitter is None:
        t = (delta_step * k).repeat(R).unsqueeze(1)
    else:
        t = (delta_step * (k.unsqueeze(0) - jitter.to(origins.device))).reshape(-1, 1)
    o = torch.repeat_interleave(origins, num_samples, 0)
    d = torch.repeat_interleave(dirs, num_samples, 0)
    return o + d * t


def normalize(samples, gmin, points_distance: float):
    """src/ray_sampling.py:12-13 with the min precomputed."""
    return (samples - gmin) / points_distance


# ----------------------------------------------------------------------- lookup
def in_bounds(idx, shape):
    """src/grid_functions.py:47-63 find_out_of_bound."""
    X, Y, Z = shape[:3]
    return ((idx[:, 0] < X) & (idx[:, 0] >= 0) & (idx[:, 1] < Y) & (idx[:, 1] >= 0)
            & (idx[:, 2] < Z) & (idx[:, 2] >= 0))


def wrap_(idx, shape):
    """src/grid_functions.py:66-79 fix_out_of_bounds (in place, floor modulo)."""
    X, Y, Z = shape[:3]
    idx[:, 0] %= X
    idx[:, 1] %= Y
    idx[:, 2] %= Z
    return idx


def nearest_lookup(n, grid):
    """src/grid_functions.py:103-114: values at round(n) (wrapped) and the int mask."""
    idx = torch.round(n).to(torch.long)
    mask = in_bounds(idx, grid.shape)
    wrap_(idx, grid.shape)
    return grid[idx[:, 0], idx[:, 1], idx[:, 2]], mask, idx


def corner_indices(n):
    """src/grid_functions.py:220-246: [N,8,3] corners, x/y/z in {ceil, floor}."""
    c = [torch.ceil(n[:, a]).unsqueeze(1) for a in range(3)]
    f = [torch.floor(n[:, a]).unsqueeze(1) for a in range(3)]
    pts = [torch.cat([x, y, z], 1).unsqueeze(1)
           for x in (c[0], f[0]) for y in (c[1], f[1]) for z in (c[2], f[2])]
    return torch.cat(pts, 1).type(torch.long)


def collect_cells(n, grid):
    """src/grid_functions.py:154-170 collect_cell_information_via_indices: the in-bounds
    mask of the float coordinates, then the 8 corners flattened to [N*8,3], wrapped in
    place and gathered. Returns (values [N*8,4], mask [N])."""
    mask = in_bounds(n, grid.shape)
    corners = corner_indices(n).reshape(-1, 3)
    wrap_(corners, grid.shape)
    return grid[corners[:, 0], corners[:, 1], corners[:, 2]], mask


def trilinear_blend(n, corners, grid):
    """src/grid_functions.py:7-44 trilinear_interpolation, same op order."""
    fr = torch.frac(n)
    s0 = grid[corners[:, 4:, 0], corners[:, 4:, 1], corners[:, 4:, 2]]
    s1 = grid[corners[:, :4, 0], corners[:, :4, 1], corners[:, :4, 2]]
    w = fr[:, 0].unsqueeze(-1).unsqueeze(-1)
    out = (s1 * w) + (s0 * (1 - w))
    w = fr[:, 1].unsqueeze(-1).unsqueeze(-1)
    out = (out[:, :2] * w) + (out[:, 2:] * (1 - w))
    w = fr[:, 2].unsqueeze(-1)
    return (out[:, 0] * w) + (out[:, 1] * (1 - w))


def trilinear_lookup(n, grid):
    """The trilinear path as the reference's functions compose (no caller exists in the
    reference): corners -> in-place wrap on a [N*8,3] view -> blend -> float mask."""
    corners = corner_indices(n)
    wrap_(corners.view(-1, 3), grid.shape)
    vals = trilinear_blend(n, corners, grid)
    mask = in_bounds(n, grid.shape)
    return vals, mask, corners


# ----------------------------------------------------------------------- compositing
def composite(samples):
    """src/ray_sampling.py:172-192 compute_alpha_weighted_pixels on [C,R,S,4]."""
    alpha = samples[..., -1]
    padded = torch.cat([torch.zeros_like(alpha[..., :1]), alpha], dim=2)
    trans = (1 - padded[..., :-1]).cumprod(dim=2)
    w = (alpha * trans).unsqueeze(-1)
    rgb = (samples[..., :-1] * w).sum(2)
    a = w.sum(dim=2)
    return torch.cat([rgb, a], dim=2)


# ----------------------------------------------------------------------- full path
def render(grid, origins, dirs, num_samples: int, delta_step: float, gmin, points_distance: float,
           mode: str = "trilinear", clip: bool = True, jitter=None, background=None):
    """rgba [R,4] of rays through the grid: scripts/train.py:142-153 with the lookup
    chosen by mode; background (harness term, e.g. white) composites rgb over it.
    Differentiable in grid through torch autograd."""
    R = origins.shape[0]
    pts = sample_positions(origins, dirs, num_samples, delta_step, jitter)
    n = normalize(pts, gmin, points_distance)
    g = grid.clip(0, 1) if clip else grid
    if mode == "nearest":
        vals, mask, _ = nearest_lookup(n, g)
    elif mode == "trilinear":
        vals, mask, _ = trilinear_lookup(n, g)
    else:
        raise ValueError(mode)
    vals = vals * mask.unsqueeze(-1)
    px = composite(vals.reshape(1, R, num_samples, 4)).reshape(R, 4)
    if background is not None:
        bg = torch.as_tensor(background, dtype=px.dtype)
        px = torch.cat([px[:, :3] + (1 - px[:, 3:]) * bg, px[:, 3:]], 1)
    return px


def train_loss(grid, origins, dirs, target, num_samples, delta_step, gmin, points_distance,
               mode="trilinear", clip=True, jitter=None, background=None):
    """mse_loss(render, target), scripts/train.py:156."""
    px = render(grid, origins, dirs, num_samples, delta_step, gmin, points_distance, mode, clip,
                jitter, background)
    return torch.nn.functional.mse_loss(px, target)


def sample_indices(origins, dirs, num_samples, delta_step, gmin, points_distance, shape,
                   mode="trilinear", jitter=None):
    """The wrapped cell indices the path reads and the in-bounds flags, per sample."""
    pts = sample_positions(origins, dirs, num_samples, delta_step, jitter)
    n = normalize(pts, gmin, points_distance)
    if mode == "nearest":
        idx = torch.round(n).to(torch.long)
        mask = in_bounds(idx, shape)
        wrap_(idx, shape)
        return idx, mask
    corners = corner_indices(n)
    wrap_(corners.view(-1, 3), shape)
    return corners, in_bounds(n, shape)


def jitter_for(seed: int, num_rays: int, num_samples: int, dtype=torch.float32):
    """Stratification offsets j[r, s] of the counter hash."""
    return torch.from_numpy(stratified_jitter(seed, num_rays, num_samples)).to(dtype)


# ----------------------------------------------------------------------- training losses
def tv_loss(grid):
    """scripts/train.py:44-65: sqrt of the summed squared neighbour differences along
    the three axes (the reference names them x, y, z but differences dims 1, 2, 0)."""
    gx = (grid[:, :-1, :, :] - grid[:, 1:, :, :]).pow(2)
    gy = (grid[:, :, :-1, :] - grid[:, :, 1:, :]).pow(2)
    gz = (grid[:-1, :, :, :] - grid[1:, :, :, :]).pow(2)
    return torch.sqrt(gx.sum() + gy.sum() + gz.sum())


def beta_loss(alpha, eps=1e-4):
    """scripts/train.py:170-177 without the weight: mean of log(a + eps) - log(1 - a + eps)
    over the sampled (masked) opacities."""
    return (torch.log(alpha + eps) - torch.log(1 - alpha + eps)).mean()


def render_samples(grid, origins, dirs, num_samples, delta_step, gmin, points_distance,
                   mode="nearest", clip=True, jitter=None):
    """(rgba [R,4], masked sample values [R,S,4]): the path of render() keeping the
    per-sample values the beta loss reads (scripts/train.py:146-151)."""
    R = origins.shape[0]
    pts = sample_positions(origins, dirs, num_samples, delta_step, jitter)
    n = normalize(pts, gmin, points_distance)
    g = grid.clip(0, 1) if clip else grid
    vals, mask, _ = nearest_lookup(n, g) if mode == "nearest" else trilinear_lookup(n, g)
    vals = (vals * mask.unsqueeze(-1)).reshape(1, R, num_samples, 4)
    return composite(vals).reshape(R, 4), vals


def average_pool3d_grid(tensor, receptive_field_size=3, stride=None):
    """src/grid_functions.py:173-181: avg_pool3d of the channels-last grid."""
    x = tensor.permute(3, 0, 1, 2).unsqueeze(0)
    r = (receptive_field_size,) * 3
    return torch.nn.functional.avg_pool3d(x, r, stride=stride).squeeze(0).permute(1, 2, 3, 0)


def remove_noise(grid_cells, kernel_size=3, radius=1.0, threshold=2, repeats=20):
    """src/grid_functions.py:260-280: filled-ball conv3d of alpha, clear cells below the
    threshold, repeated (in place)."""
    k = np.linspace(-(kernel_size // 2), kernel_size // 2, kernel_size)
    x, y, z = np.meshgrid(k, k, k)
    d = np.sqrt(x * x + y * y + z * z)
    w = np.where(d <= radius, 1, 0)
    w[kernel_size // 2, kernel_size // 2, kernel_size // 2] = 0
    w = torch.from_numpy(w).float().unsqueeze(0).unsqueeze(0)
    w = w / w.max()
    for _ in range(repeats):
        out = torch.nn.functional.conv3d(grid_cells[..., -1].unsqueeze(0), w, padding="same")[0]
        grid_cells[out < threshold] = 0
    return grid_cells


def splat_preview(grid, points_distance, transform_matrix, camera_angle_x, size_y):
    """src/visualization.py:157-232 (visulize_3d_in_2d_fast), same ops. Returns the image
    and, per drawn point (points inside the field of view), a dict of its pixel (xx, yy),
    its unrounded pixel coordinates (fx = xs * x_norm, fy = size_y * y_norm), its
    normalised coordinates (xn, yn) and its distance from the camera."""
    rot = transform_matrix[:3, :3]
    pos = transform_matrix[:3, 3]
    yz = transform_matrix[:3, 0]
    xz = transform_matrix[:3, 1]
    aspect = yz.norm(dim=0) / xz.norm(dim=0)
    cond = grid[..., 3] > 0.1
    pts = np.argwhere(cond)
    colors = grid[cond]
    half = (torch.tensor(grid.shape[:3]) / 2).unsqueeze(1).ceil()
    pts = ((pts - half) + 1)
    pts = (pts * points_distance).T
    ctp = pts - pos
    a = torch.matmul(ctp, yz)
    b = torch.matmul(ctp, xz)
    nm = ctp.norm(dim=1) * yz.norm()
    ax, ay = a / nm, b / nm
    xn = 0.5 + ay / -camera_angle_x
    yn = 0.5 + ax / (camera_angle_x / aspect)
    ok = (xn < 1.0).logical_and(xn >= 0.0).logical_and(yn < 1.0).logical_and(yn >= 0.0)
    xn, yn, colors, ctp = xn[ok], yn[ok], colors[ok], ctp[ok]
    ys = size_y
    xs = int(ys * aspect)
    fx, fy = xs * xn, ys * yn
    xx = fx.round().clamp(min=0, max=xs - 1).type(torch.long)
    yy = fy.round().clamp(min=0, max=ys - 1).type(torch.long)
    dist = ctp.norm(dim=1)
    order = torch.argsort(-dist)
    img = np.ones([xs, ys, 3])
    img[xx[order], yy[order]] = colors[order][:, :3]
    return img, dict(xx=xx, yy=yy, fx=fx, fy=fy, xn=xn, yn=yn, dist=dist)
