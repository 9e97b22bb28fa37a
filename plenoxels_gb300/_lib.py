"""ctypes binding of the C ABI in ``include/plenoxels_gb300.h``.

The library is the in-tree ``libplenoxels_gb300.so`` built by ``plenoxels_gb300.build``.
There is no fallback: if the library is missing or fails to load, every operator raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (POINTER, Structure, c_char_p, c_double, c_float, c_int32, c_int64,
                    c_uint32, c_uint64, c_void_p)

import torch

# PLENOXELS_GB300_LIB names an alternative build (plenoxels_gb300.build with lib_path)
LIB_PATH = os.environ.get("PLENOXELS_GB300_LIB") or os.path.join(
    os.path.dirname(os.path.abspath(__file__)), "libplenoxels_gb300.so")

PGB_OK, PGB_ERR_ARG, PGB_ERR_ALIGN, PGB_ERR_LAUNCH, PGB_ERR_UNSUPPORTED = 0, -1, -2, -3, -4
PGB_F32, PGB_BF16, PGB_F64 = 0, 1, 2
PGB_NEAREST, PGB_TRILINEAR = 0, 1
PGB_INDEX_F32, PGB_INDEX_F64, PGB_INDEX_I64 = 0, 1, 2
PGB_NOALLOC_MAX_RAYS = 32768


class PgbGrid(Structure):
    _fields_ = [
        ("cells", c_void_p),
        ("dtype", c_int32),
        ("dims", c_int32 * 3),
        ("origin", c_double * 3),
        ("points_distance", c_double),
        ("clip", c_int32),
        ("mode", c_int32),
        ("alpha_floor", c_float),
    ]


class PgbCameras(Structure):
    _fields_ = [
        ("transforms", c_void_p),
        ("images", c_void_p),
        ("num_cameras", c_int32),
        ("height", c_int32),
        ("width", c_int32),
        ("camera_angle_x", c_float),
        ("near", c_float),
        ("seed", c_uint64),
    ]


class PgbRays(Structure):
    _fields_ = [
        ("origins", c_void_p),
        ("dirs", c_void_p),
        ("cameras", POINTER(PgbCameras)),
        ("num_rays", c_int64),
        ("num_samples", c_int32),
        ("delta_step", c_double),
        ("stratified", c_int32),
        ("seed", c_uint64),
        ("term_threshold", c_float),
        ("use_background", c_int32),
        ("background", c_float * 3),
        ("log_transmittance", c_int32),
        ("chunk_samples", c_int32),
        ("first_ray", c_int64),
        ("grad_marks", c_void_p),
    ]


class PgbScene(Structure):
    _fields_ = [
        ("cells", c_void_p),
        ("bricks", c_void_p),
        ("occupancy", c_void_p),
        ("grad_cells", c_void_p),
        ("dims", c_int32 * 3),
        ("brick_log2", c_int32),
        ("brick_dims", c_int32 * 3),
        ("origin", c_float * 3),
        ("points_distance", c_float),
        ("num_samples", c_int32),
        ("delta_step", c_float),
    ]


class PgbLossTerms(Structure):
    _fields_ = [("mse_weight", c_double), ("beta_weight", c_double), ("beta_eps", c_float)]


_P = c_void_p
_SIGNATURES = {
    "pgb_render_fwd": (c_int32, [POINTER(PgbGrid), POINTER(PgbRays), _P, _P]),
    "pgb_render_bwd": (c_int32, [POINTER(PgbGrid), POINTER(PgbRays), _P, _P, _P]),
    "pgb_render_train": (c_int32, [POINTER(PgbGrid), POINTER(PgbRays), _P, c_double, _P, _P, _P, _P, _P]),
    "pgb_train_workspace_bytes": (c_int64, []),
    "pgb_render_train_terms": (c_int32, [POINTER(PgbGrid), POINTER(PgbRays), _P, POINTER(PgbLossTerms), _P, _P, _P, _P, _P]),
    "pgb_render_train_noalloc": (c_int32, [POINTER(PgbGrid), POINTER(PgbRays), _P, c_double, _P, _P, _P, _P]),
    "pgb_render_sample_indices": (c_int32, [POINTER(PgbGrid), POINTER(PgbRays), _P, _P, _P]),
    "pgb_render_sample_coords": (c_int32, [POINTER(PgbGrid), POINTER(PgbRays), _P, _P]),
    "pgb_build_bricks": (c_int32, [_P, POINTER(c_int32), c_int32, _P, _P]),
    "pgb_pack_mask": (c_int32, [_P, c_int64, _P, _P]),
    "pgb_batch_zero_grads": (c_int32, [_P, c_int32, c_int64, _P]),
    "pgb_batch_workspace_bytes": (c_int64, [c_int64]),
    "pgb_batch_train": (c_int32, [_P, c_int32, c_int32, c_int32, c_int32, _P, _P, _P, _P, c_int64, c_float,
                                  c_int32, c_uint64, c_double, _P, _P, _P, c_int32, c_int32, c_int32, _P]),
    "pgb_tv_workspace_bytes": (c_int64, []),
    "pgb_tv_sumsq": (c_int32, [_P, POINTER(c_int32), _P, _P, _P]),
    "pgb_tv_grad": (c_int32, [_P, POINTER(c_int32), _P, c_float, _P, _P]),
    "pgb_adam_step": (c_int32, [_P, _P, _P, _P, _P, c_int64, c_double, c_double, c_double, c_double,
                                c_int64, c_int32, _P]),
    "pgb_adam_tv_step": (c_int32, [_P, _P, _P, _P, _P, _P, POINTER(c_int32), _P, c_float, c_double, c_double,
                                   c_double, c_double, c_int64, c_int32, _P]),
    "pgb_avg_pool3d_shape": (c_int32, [POINTER(c_int32), c_int32, c_int32, POINTER(c_int32), POINTER(c_int64)]),
    "pgb_avg_pool3d_fwd": (c_int32, [_P, POINTER(c_int32), c_int32, c_int32, _P, _P, _P]),
    "pgb_avg_pool3d_bwd": (c_int32, [_P, POINTER(c_int32), c_int32, c_int32, _P, _P, _P]),
    "pgb_generate_rays": (c_int32, [_P, c_int32, c_int64, c_float, _P, c_int32, c_int32, _P, c_int32, _P, _P, _P, _P]),
    "pgb_sample_points": (c_int32, [_P, c_int32, c_int64, _P, c_int32, c_float, _P, _P]),
    "pgb_coords_min": (c_int32, [_P, c_int64, _P, _P]),
    "pgb_normalize_samples": (c_int32, [_P, c_int64, _P, c_float, _P, _P]),
    "pgb_nearest_gather": (c_int32, [POINTER(PgbGrid), _P, c_int64, _P, _P, _P, _P]),
    "pgb_nearest_scatter": (c_int32, [POINTER(PgbGrid), _P, c_int64, _P, _P, _P]),
    "pgb_grid_coords": (c_int32, [POINTER(c_int32), c_float, _P, _P, _P]),
    "pgb_gather_cells": (c_int32, [POINTER(PgbGrid), _P, c_int64, _P, _P, _P]),
    "pgb_scatter_cells": (c_int32, [POINTER(PgbGrid), _P, c_int64, _P, _P, _P, _P]),
    "pgb_corner_indices": (c_int32, [_P, c_int32, c_int64, _P, _P]),
    "pgb_in_bounds": (c_int32, [_P, c_int32, c_int64, POINTER(c_int32), _P, _P]),
    "pgb_wrap_indices": (c_int32, [_P, c_int64, POINTER(c_int32), _P]),
    "pgb_trilinear_gather": (c_int32, [POINTER(PgbGrid), _P, _P, c_int64, _P, _P, _P]),
    "pgb_trilinear_scatter": (c_int32, [POINTER(PgbGrid), _P, _P, c_int64, _P, _P, _P, _P]),
    "pgb_composite_fwd": (c_int32, [_P, c_int32, c_int64, c_int32, _P, _P]),
    "pgb_composite_bwd": (c_int32, [_P, c_int32, c_int64, c_int32, _P, _P, _P]),
    "pgb_fill_zero": (c_int32, [_P, c_int64, _P]),
    "pgb_clear_marked": (c_int32, [_P, c_int32, c_int64, _P, _P]),
    "pgb_mark_words": (c_int64, [c_int64]),
    "pgb_rgba_to_image": (c_int32, [_P, c_int32, _P, _P]),
    "pgb_splat_size": (c_int32, [POINTER(c_float), c_int32, POINTER(c_int32)]),
    "pgb_splat_preview": (c_int32, [_P, POINTER(c_int32), c_float, POINTER(c_float), c_float, c_int32, c_float,
                                    _P, _P, _P]),
    "pgb_remove_noise": (c_int32, [_P, POINTER(c_int32), c_int32, c_double, c_float, c_int32, _P, _P]),
    "pgb_hash_uniform": (c_float, [c_uint64, c_uint64, c_uint32]),
    "pgb_launch_count": (c_int64, []),
    "pgb_version": (c_char_p, []),
    "pgb_status_string": (c_char_p, [c_int32]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Loads the library once; raises RuntimeError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"plenoxels_gb300: {LIB_PATH} is missing; build it with "
                "`python -m plenoxels_gb300.build` (there is no CPU or torch fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def symbols() -> list[str]:
    return list(_SIGNATURES)


class PlenoxelsError(RuntimeError):
    """A C ABI entry point returned an error status."""


def check(status: int, what: str) -> None:
    if status != PGB_OK:
        msg = load().pgb_status_string(status).decode()
        if status == PGB_ERR_UNSUPPORTED:
            raise NotImplementedError(f"{what}: {msg} (status {status})")
        raise PlenoxelsError(f"{what}: {msg} (status {status})")


def stream_of(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def require_cuda(*tensors: torch.Tensor) -> None:
    for t in tensors:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"expected a torch.Tensor, got {type(t).__name__}")
        if not t.is_cuda:
            raise ValueError("plenoxels_gb300 operators take CUDA tensors (there is no CPU path)")
    devs = {t.device for t in tensors}
    if len(devs) > 1:
        raise ValueError(f"tensors are on different devices: {sorted(map(str, devs))}")


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


STORAGE_CODES = {torch.float32: PGB_F32, torch.bfloat16: PGB_BF16, torch.float64: PGB_F64}


def real_dtype(storage: torch.dtype) -> torch.dtype:
    """Arithmetic (and gradient) dtype of a storage dtype."""
    return torch.float64 if storage == torch.float64 else torch.float32


def make_grid(cells: torch.Tensor, origin, points_distance: float, mode: int, clip: bool,
              alpha_floor: float = 0.0) -> PgbGrid:
    if cells.dim() != 4 or cells.shape[-1] != 4:
        raise ValueError(f"grid must be [X,Y,Z,4], got {tuple(cells.shape)}")
    if cells.dtype not in STORAGE_CODES:
        raise TypeError(f"grid dtype {cells.dtype} not supported (float32, bfloat16, float64)")
    if not cells.is_contiguous():
        raise ValueError("grid must be contiguous channels-last [X,Y,Z,4]")
    g = PgbGrid()
    g.cells = cells.data_ptr()
    g.dtype = STORAGE_CODES[cells.dtype]
    g.dims[0], g.dims[1], g.dims[2] = (int(s) for s in cells.shape[:3])
    for a in range(3):
        g.origin[a] = float(origin[a])
    g.points_distance = float(points_distance)
    g.clip = 1 if clip else 0
    g.mode = mode
    g.alpha_floor = float(alpha_floor)
    return g


def dims3(shape) -> ctypes.Array:
    d = (c_int32 * 3)()
    d[0], d[1], d[2] = (int(s) for s in shape[:3])
    return d
