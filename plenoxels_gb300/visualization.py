"""Drop-in for the point-splat preview of the reference's src/visualization.py:157-232
(visulize_3d_in_2d_fast), on the GPU. The plotting helpers of that file (matplotlib,
plotly) are presentation and are not provided."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check, ptr


@torch.no_grad()
def visulize_3d_in_2d_fast(grid, points_distance, transform_matrix, camera_angle_x, size_y,
                           device=None, alpha_min=0.1):
    """[xs, size_y, 3] float64 image (numpy): each cell with alpha > 0.1 projected to its
    pixel, the nearest one painting its RGB over a white background. xs = int(size_y *
    aspect) with the aspect of the camera's x and y axes."""
    dev = torch.device(device) if device is not None else (
        grid.device if grid.is_cuda else torch.device("cuda", torch.cuda.current_device()))
    if dev.type != "cuda":
        raise ValueError("visulize_3d_in_2d_fast runs on a CUDA device")
    g = grid.detach().to(dev, torch.float32).contiguous()
    T = (ctypes.c_float * 16)(*[float(v) for v in transform_matrix.detach().cpu().reshape(-1).tolist()])
    lib = _lib.load()
    xs = ctypes.c_int32(0)
    check(lib.pgb_splat_size(T, int(size_y), ctypes.byref(xs)), "visulize_3d_in_2d_fast")
    keys = torch.empty(xs.value * int(size_y), dtype=torch.int64, device=dev)
    img = torch.empty(xs.value, int(size_y), 3, dtype=torch.float32, device=dev)
    check(lib.pgb_splat_preview(ptr(g), _lib.dims3(g.shape), float(points_distance), T,
                                float(camera_angle_x), int(size_y), float(alpha_min), ptr(keys),
                                ptr(img), torch.cuda.current_stream(dev).cuda_stream),
          "visulize_3d_in_2d_fast")
    return img.cpu().numpy().astype(np.float64)
