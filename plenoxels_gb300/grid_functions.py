"""Drop-in for the lookup half of the reference's ``src/grid_functions.py`` on GB300.

Same function names, arguments and return values as the reference; every function runs
one or more kernels of ``libplenoxels_gb300.so`` on the current CUDA stream. Inputs must
be CUDA tensors (there is no CPU path). Functions that the reference differentiates
(lookups of the grid) are ``torch.autograd.Function``s whose backward is a hand-written
scatter kernel.

Also provided: average_pool3d_grid (the coarse-to-fine pooling the training loop feeds
into the path) and convolve_grid_to_remove_noise (the stray-voxel clean-up applied before
viewing). Out of scope: voxel_average, get_receptive_field_voxels and the kernel helpers.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr, require_cuda, stream_of


def _device(device) -> torch.device:
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError(f"plenoxels_gb300 runs on CUDA devices only, got device={device!r}")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def generate_grid(sx, sy, sz, points_distance=0.5, info_size=4, device="cuda"):
    """src/grid_functions.py:184-217. Returns (grid_coords [G,3], grid_cells [X,Y,Z,info]
    zero leaf with requires_grad, meshgrid [X,Y,Z,3] int64, grid_grid [X,Y,Z,3])."""
    dev = _device(device)
    lib = _lib.load()
    coords = torch.empty(sx, sy, sz, 3, dtype=torch.float32, device=dev)
    mesh = torch.empty(sx, sy, sz, 3, dtype=torch.int64, device=dev)
    s = torch.cuda.current_stream(dev).cuda_stream
    check(lib.pgb_grid_coords(_lib.dims3((sx, sy, sz)), float(points_distance), ptr(coords),
                              ptr(mesh), s), "generate_grid")
    cells = torch.empty(sx, sy, sz, info_size, dtype=torch.float32, device=dev)
    check(lib.pgb_fill_zero(ptr(cells), cells.numel() * 4, s), "generate_grid")
    cells.requires_grad_(True)
    return coords.reshape(sx * sy * sz, 3), cells, mesh, coords


def grid_origin(shape, points_distance: float, dtype=torch.float32):
    """Per-axis minimum of generate_grid's coordinates, (1 - ceil(s/2)) * pd, rounded as
    the reference's tensor arithmetic rounds it (fp32 unless dtype is float64)."""
    if dtype == torch.float64:
        return tuple(float(np.float64(1 - math.ceil(s / 2)) * np.float64(points_distance))
                     for s in shape[:3])
    return tuple(float(np.float32(1 - math.ceil(s / 2)) * np.float32(points_distance))
                 for s in shape[:3])


def _grid_desc(grid, mode, clip=False):
    return _lib.make_grid(grid, (0.0, 0.0, 0.0), 1.0, mode, clip)


def _check_coords(n, grid, what):
    if n.dim() != 2 or n.shape[1] != 3:
        raise ValueError(f"{what}: expected [N,3] coordinates, got {tuple(n.shape)}")
    want = _lib.real_dtype(grid.dtype)
    if n.dtype != want:
        raise TypeError(f"{what}: coordinates must be {want} for a {grid.dtype} grid, got {n.dtype}")
    return n.contiguous()


class _NearestLookup(torch.autograd.Function):
    @staticmethod
    def forward(ctx, n, grid, clip):
        lib = _lib.load()
        N = n.shape[0]
        vals = torch.empty(N, 4, dtype=_lib.real_dtype(grid.dtype), device=n.device)
        mask = torch.empty(N, dtype=torch.bool, device=n.device)
        desc = _grid_desc(grid, _lib.PGB_NEAREST, clip)
        check(lib.pgb_nearest_gather(desc, ptr(n), N, ptr(vals), ptr(mask), None, stream_of(n)),
              "get_nearest_voxels")
        ctx.save_for_backward(n, grid)
        ctx.clip = clip
        ctx.mark_non_differentiable(mask)
        return vals, mask

    @staticmethod
    def backward(ctx, d_vals, _d_mask):
        n, grid = ctx.saved_tensors
        lib = _lib.load()
        grad = torch.empty(grid.shape, dtype=_lib.real_dtype(grid.dtype), device=grid.device)
        s = stream_of(grid)
        check(lib.pgb_fill_zero(ptr(grad), grad.numel() * grad.element_size(), s), "backward")
        if d_vals is not None:
            d_vals = d_vals.to(grad.dtype).contiguous()
            desc = _grid_desc(grid, _lib.PGB_NEAREST, ctx.clip)
            check(lib.pgb_nearest_scatter(desc, ptr(n), n.shape[0], ptr(d_vals), ptr(grad), s),
                  "get_nearest_voxels backward")
        return None, grad, None


def get_nearest_voxels(normalized_samples_for_indices, grid, receptive_field=1, clip=False):
    """src/grid_functions.py:103-114: (values of the nearest cells [N,4], in-bounds mask
    [N]). Indices round half to even and wrap periodically; values are not masked.
    receptive_field is accepted and ignored, as in the reference. clip=True fuses the
    grid.clip(0, 1) of scripts/train.py:146 into the gather."""
    require_cuda(normalized_samples_for_indices, grid)
    n = _check_coords(normalized_samples_for_indices, grid, "get_nearest_voxels")
    return _NearestLookup.apply(n, grid.contiguous(), bool(clip))


def find_out_of_bound(indecies, grid):
    """src/grid_functions.py:47-63: bool [N], True where 0 <= idx < dim on every axis."""
    require_cuda(indecies, grid)
    idx = indecies
    if idx.dtype == torch.float32:
        kind = _lib.PGB_INDEX_F32
    elif idx.dtype == torch.float64:
        kind = _lib.PGB_INDEX_F64
    else:
        kind = _lib.PGB_INDEX_I64
        idx = idx.to(torch.int64)
    idx = idx.contiguous()
    out = torch.empty(idx.shape[0], dtype=torch.bool, device=idx.device)
    check(_lib.load().pgb_in_bounds(ptr(idx), kind, idx.shape[0], _lib.dims3(grid.shape), ptr(out),
                                    stream_of(idx)), "find_out_of_bound")
    return out


def fix_out_of_bounds(indices, grid):
    """src/grid_functions.py:66-79: wraps int64 [N,3] indices in place (floor modulo) and
    returns the three column views."""
    require_cuda(indices, grid)
    if indices.dtype != torch.int64:
        raise TypeError(f"fix_out_of_bounds: int64 indices required, got {indices.dtype}")
    if not indices.is_contiguous():
        raise ValueError("fix_out_of_bounds: indices must be contiguous to be wrapped in place")
    check(_lib.load().pgb_wrap_indices(ptr(indices), indices.shape[0], _lib.dims3(grid.shape),
                                       stream_of(indices)), "fix_out_of_bounds")
    return indices[:, 0], indices[:, 1], indices[:, 2]


def get_grid_points_indices(normalized_samples_for_indecies):
    """src/grid_functions.py:220-246: int64 [N,8,3] corners, x/y/z in {ceil, floor}."""
    n = normalized_samples_for_indecies
    require_cuda(n)
    if n.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"get_grid_points_indices: float coordinates required, got {n.dtype}")
    n = n.contiguous()
    out = torch.empty(n.shape[0], 8, 3, dtype=torch.int64, device=n.device)
    code = _lib.PGB_F64 if n.dtype == torch.float64 else _lib.PGB_F32
    check(_lib.load().pgb_corner_indices(ptr(n), code, n.shape[0], ptr(out), stream_of(n)),
          "get_grid_points_indices")
    return out


def _raise_on_status(status, what):
    if int(status.item()) != 0:
        raise IndexError(f"{what}: index out of range of the grid")


class _CellGather(torch.autograd.Function):
    @staticmethod
    def forward(ctx, idx, grid):
        lib = _lib.load()
        M = idx.shape[0]
        out = torch.empty(M, 4, dtype=_lib.real_dtype(grid.dtype), device=idx.device)
        status = torch.zeros(1, dtype=torch.int32, device=idx.device)
        check(lib.pgb_gather_cells(_grid_desc(grid, _lib.PGB_NEAREST), ptr(idx), M, ptr(out),
                                   ptr(status), stream_of(idx)), "collect_cell_information_via_indices")
        _raise_on_status(status, "collect_cell_information_via_indices")
        ctx.save_for_backward(idx, grid)
        return out

    @staticmethod
    def backward(ctx, d_out):
        idx, grid = ctx.saved_tensors
        lib = _lib.load()
        grad = torch.empty(grid.shape, dtype=_lib.real_dtype(grid.dtype), device=grid.device)
        s = stream_of(grid)
        check(lib.pgb_fill_zero(ptr(grad), grad.numel() * grad.element_size(), s), "backward")
        d_out = d_out.to(grad.dtype).contiguous()
        check(lib.pgb_scatter_cells(_grid_desc(grid, _lib.PGB_NEAREST), ptr(idx), idx.shape[0],
                                    ptr(d_out), ptr(grad), None, s), "backward")
        return None, grad


def collect_cell_information_via_indices(normalized_samples_for_indices, B):
    """src/grid_functions.py:154-170: (cells at the 8 wrapped corners of every sample,
    [N*8,4]; float in-bounds mask [N])."""
    require_cuda(normalized_samples_for_indices, B)
    outofbounds = find_out_of_bound(normalized_samples_for_indices, B)
    corners = get_grid_points_indices(normalized_samples_for_indices).reshape(-1, 3)
    fix_out_of_bounds(corners, B)
    return _CellGather.apply(corners, B.contiguous()), outofbounds


class _Trilinear(torch.autograd.Function):
    @staticmethod
    def forward(ctx, n, corners, grid, clip):
        lib = _lib.load()
        N = n.shape[0]
        out = torch.empty(N, 4, dtype=_lib.real_dtype(grid.dtype), device=n.device)
        status = torch.zeros(1, dtype=torch.int32, device=n.device)
        desc = _grid_desc(grid, _lib.PGB_TRILINEAR, clip)
        check(lib.pgb_trilinear_gather(desc, ptr(n), ptr(corners), N, ptr(out), ptr(status),
                                       stream_of(n)), "trilinear_interpolation")
        _raise_on_status(status, "trilinear_interpolation")
        ctx.save_for_backward(n, corners, grid)
        ctx.clip = clip
        return out

    @staticmethod
    def backward(ctx, d_out):
        n, corners, grid = ctx.saved_tensors
        lib = _lib.load()
        grad = torch.empty(grid.shape, dtype=_lib.real_dtype(grid.dtype), device=grid.device)
        s = stream_of(grid)
        check(lib.pgb_fill_zero(ptr(grad), grad.numel() * grad.element_size(), s), "backward")
        d_out = d_out.to(grad.dtype).contiguous()
        desc = _grid_desc(grid, _lib.PGB_TRILINEAR, ctx.clip)
        check(lib.pgb_trilinear_scatter(desc, ptr(n), ptr(corners), n.shape[0], ptr(d_out),
                                        ptr(grad), None, s), "trilinear_interpolation backward")
        return None, None, grad, None


def trilinear_interpolation(normalized_samples_for_indecies, selected_points, grid_cells, clip=False):
    """src/grid_functions.py:7-44: [N,4] trilinear blend of the 8 given (already wrapped)
    corners with torch.frac weights, x then y then z. Differentiable in grid_cells (the
    reference never differentiates the coordinates). clip=True fuses grid.clip(0, 1)."""
    require_cuda(normalized_samples_for_indecies, selected_points, grid_cells)
    n = _check_coords(normalized_samples_for_indecies, grid_cells, "trilinear_interpolation")
    if selected_points.dtype != torch.int64 or tuple(selected_points.shape[1:]) != (8, 3):
        raise ValueError("trilinear_interpolation: selected_points must be int64 [N,8,3]")
    return _Trilinear.apply(n, selected_points.contiguous(), grid_cells.contiguous(), bool(clip))


def pool_shape(shape, window, stride):
    """(out_dims, scratch bytes) of average_pool3d_grid on a [X,Y,Z,4] grid."""
    od = (ctypes.c_int32 * 3)()
    nbytes = ctypes.c_int64(0)
    check(_lib.load().pgb_avg_pool3d_shape(_lib.dims3(shape), int(window), int(stride), od,
                                           ctypes.byref(nbytes)), "average_pool3d_grid")
    return (od[0], od[1], od[2]), int(nbytes.value)


class _AvgPool(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid, window, stride):
        od, nbytes = pool_shape(grid.shape, window, stride)
        scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=grid.device)
        out = torch.empty(*od, 4, dtype=torch.float32, device=grid.device)
        check(_lib.load().pgb_avg_pool3d_fwd(ptr(grid), _lib.dims3(grid.shape), window, stride,
                                             ptr(scratch), ptr(out), stream_of(grid)),
              "average_pool3d_grid")
        ctx.shape, ctx.window, ctx.stride = tuple(grid.shape), window, stride
        return out

    @staticmethod
    def backward(ctx, d_out):
        _, nbytes = pool_shape(ctx.shape, ctx.window, ctx.stride)
        d_out = d_out.to(torch.float32).contiguous()
        scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=d_out.device)
        d_in = torch.empty(ctx.shape, dtype=torch.float32, device=d_out.device)
        check(_lib.load().pgb_avg_pool3d_bwd(ptr(d_out), _lib.dims3(ctx.shape), ctx.window,
                                             ctx.stride, ptr(scratch), ptr(d_in),
                                             stream_of(d_out)), "average_pool3d_grid backward")
        return d_in, None, None


def average_pool3d_grid(tensor, receptive_field_size=3, stride=None):
    """src/grid_functions.py:173-181: [X,Y,Z,4] -> [Xo,Yo,Zo,4] average over cubic windows
    of receptive_field_size cells with the given stride (default: the window), no
    padding. Returns a contiguous tensor (the reference returns a permuted view of the
    same values). Differentiable."""
    require_cuda(tensor)
    if tensor.dim() != 4 or tensor.shape[-1] != 4 or tensor.dtype != torch.float32:
        raise ValueError("average_pool3d_grid takes a float32 [X,Y,Z,4] grid")
    r = int(receptive_field_size)
    s = r if stride is None else int(stride)
    return _AvgPool.apply(tensor.contiguous(), r, s)


@torch.no_grad()
def convolve_grid_to_remove_noise(grid_cells, kernel_size=3, radius=1.0, threshold=2, repeats=20):
    """src/grid_functions.py:270-280: `repeats` times, cells whose summed neighbour alpha
    over the filled ball (distance <= radius, centre excluded, zero padding) is below
    threshold are cleared, in place; returns grid_cells."""
    require_cuda(grid_cells)
    if grid_cells.dim() != 4 or grid_cells.shape[-1] != 4 or grid_cells.dtype != torch.float32:
        raise ValueError("convolve_grid_to_remove_noise takes a float32 [X,Y,Z,4] grid")
    if not grid_cells.is_contiguous():
        raise ValueError("convolve_grid_to_remove_noise works in place on a contiguous grid")
    sums = torch.empty(grid_cells.shape[:3], dtype=torch.float32, device=grid_cells.device)
    check(_lib.load().pgb_remove_noise(ptr(grid_cells), _lib.dims3(grid_cells.shape), int(kernel_size),
                                       float(radius), float(threshold), int(repeats), ptr(sums),
                                       stream_of(grid_cells)), "convolve_grid_to_remove_noise")
    return grid_cells
