"""Drop-in for the ray half of the reference's ``src/ray_sampling.py`` on GB300.

Same names, arguments and return values as the reference, one kernel per step on the
current CUDA stream. Out of scope (no callers in the reference): get_camera_normal,
sample_positive_opacity, generate_rays and sample_camera_rays (the superseded per-camera
CPU loop).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, require_cuda, stream_of


def _f32(t, what):
    if t.dtype != torch.float32:
        raise TypeError(f"{what}: float32 tensor required, got {t.dtype}")
    return t.contiguous()


def normalize_samples_for_indecies(grid_indices, samples_interval, points_distance):
    """src/ray_sampling.py:12-13: (samples - grid_indices.min(0)) / points_distance, with
    the min as a reduction kernel and an IEEE division (bit-identical to the reference's
    CPU arithmetic)."""
    require_cuda(grid_indices, samples_interval)
    gi = _f32(grid_indices, "normalize_samples_for_indecies").reshape(-1, 3)
    sm = _f32(samples_interval, "normalize_samples_for_indecies")
    lib = _lib.load()
    s = stream_of(sm)
    gmin = torch.empty(3, dtype=torch.float32, device=sm.device)
    check(lib.pgb_coords_min(ptr(gi), gi.shape[0], ptr(gmin), s), "normalize_samples_for_indecies")
    out = torch.empty_like(sm)
    check(lib.pgb_normalize_samples(ptr(sm), sm.shape[0], ptr(gmin), float(points_distance),
                                    ptr(out), s), "normalize_samples_for_indecies")
    return out


def generate_rays_batched(imgs, number_of_rays, transform_matricies, camera_angle_x,
                          even_spread=False, device="cuda", ray_uv=None):
    """src/ray_sampling.py:195-264: (directions [C*R,3], target pixels [C*R,4]).

    The random pixel positions are drawn with torch.rand(C, R, 2) exactly as the
    reference draws them (same generator, same shape), unless ray_uv [C,R,2] supplies
    them. even_spread=True uses a side x side linspace grid (R must be a square)."""
    require_cuda(imgs, transform_matricies)
    T = _f32(transform_matricies, "generate_rays_batched")
    I = _f32(imgs, "generate_rays_batched")
    if I.dim() != 4 or I.shape[-1] != 4:
        raise ValueError(f"generate_rays_batched: imgs must be [C,H,W,4], got {tuple(I.shape)}")
    C = T.shape[0]
    R = int(number_of_rays)
    uv = None
    if even_spread:
        side = int(np.round(np.sqrt(R)))
        if side * side != R:
            raise ValueError(f"even_spread needs a square number of rays, got {R}")
    else:
        if ray_uv is None:
            ray_uv = torch.rand(C, R, 2, device=device)
        require_cuda(ray_uv)
        uv = _f32(ray_uv, "generate_rays_batched")
    dirs = torch.empty(C * R, 3, dtype=torch.float32, device=T.device)
    pixels = torch.empty(C * R, 4, dtype=torch.float32, device=T.device)
    # a pixel index can only leave the image for non-square images or caller-given uniforms
    # (torch.rand draws lie in [0,1)); only then is the status word read back
    checked = I.shape[1] != I.shape[2] or ray_uv is not None
    status = torch.zeros(1, dtype=torch.int32, device=T.device) if checked else None
    check(_lib.load().pgb_generate_rays(ptr(T), C, R, float(camera_angle_x), ptr(I), I.shape[1],
                                        I.shape[2], ptr(uv), 1 if even_spread else 0, ptr(dirs),
                                        ptr(pixels), ptr(status), stream_of(T)),
          "generate_rays_batched")
    if checked and int(status.item()) != 0:
        raise IndexError("generate_rays_batched: pixel index out of range of the images")
    return dirs, pixels


def sample_camera_rays_batched(transform_matrices, camera_angle_x, imgs, number_of_rays,
                               num_samples, delta_step, even_spread, camera_ray, device="cuda",
                               ray_uv=None):
    """src/ray_sampling.py:128-169: (samples_interval [C*R*S,3], pixels_to_rays [C*R,4],
    camera_positions [C,3], ray_directions [C*R,3]); samples at
    position + direction * (delta_step * k), k = 1..S."""
    if camera_ray:
        raise NotImplementedError(
            "camera_ray=True: the reference broadcasts a [1,C,3] direction against [N,1] "
            "offsets (src/ray_sampling.py:150-167), which has no consistent meaning")
    if even_spread:
        number_of_rays = int(np.round(np.sqrt(number_of_rays)) ** 2)
    dirs, pixels = generate_rays_batched(imgs, number_of_rays, transform_matrices, camera_angle_x,
                                         even_spread=even_spread, device=device, ray_uv=ray_uv)
    T = transform_matrices.contiguous()
    C = T.shape[0]
    S = int(num_samples)
    samples = torch.empty(C * number_of_rays * S, 3, dtype=torch.float32, device=T.device)
    check(_lib.load().pgb_sample_points(ptr(T), C, number_of_rays, ptr(dirs), S, float(delta_step),
                                        ptr(samples), stream_of(T)), "sample_camera_rays_batched")
    return samples, pixels, transform_matrices[:, :3, 3], dirs


class _Composite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, samples):
        lib = _lib.load()
        C, R, S, _ = samples.shape
        out = torch.empty(C, R, 4, dtype=samples.dtype, device=samples.device)
        code = _lib.PGB_F64 if samples.dtype == torch.float64 else _lib.PGB_F32
        check(lib.pgb_composite_fwd(ptr(samples), code, C * R, S, ptr(out), stream_of(samples)),
              "compute_alpha_weighted_pixels")
        ctx.save_for_backward(samples)
        return out

    @staticmethod
    def backward(ctx, d_out):
        (samples,) = ctx.saved_tensors
        lib = _lib.load()
        C, R, S, _ = samples.shape
        d_out = d_out.to(samples.dtype).contiguous()
        d_samples = torch.empty_like(samples)
        code = _lib.PGB_F64 if samples.dtype == torch.float64 else _lib.PGB_F32
        check(lib.pgb_composite_bwd(ptr(samples), code, C * R, S, ptr(d_out), ptr(d_samples),
                                    stream_of(samples)), "compute_alpha_weighted_pixels backward")
        return d_samples


def compute_alpha_weighted_pixels(samples):
    """src/ray_sampling.py:172-192: [C,R,S,4] samples -> [C,R,4] = (sum_k w_k rgb_k,
    sum_k w_k), w_k = alpha_k * prod_{j<k} (1 - alpha_j). The backward is the
    division-free suffix recurrence (exact where alpha == 1)."""
    require_cuda(samples)
    if samples.dim() != 4 or samples.shape[-1] != 4:
        raise ValueError(f"compute_alpha_weighted_pixels: expected [C,R,S,4], got {tuple(samples.shape)}")
    if samples.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"compute_alpha_weighted_pixels: float32/float64 required, got {samples.dtype}")
    return _Composite.apply(samples.contiguous())
