"""plenoxels_gb300 — GB300-native (sm_103a) differentiable voxel-grid render path.

A drop-in for the render path of DanJbk/Plenoxels: the functions of its
src/ray_sampling.py and src/grid_functions.py that the training step calls keep their
names, arguments and return values, and run as hand-written CUDA kernels reached
through the C ABI of ``libplenoxels_gb300.so`` (include/plenoxels_gb300.h). The fused
entry points (``render_rays``, ``FusedTrainStep``) run the whole path in one launch;
``FusedAdam`` and ``Trainer`` carry the rest of the reference's training step
(scripts/train.py), and ``batch.BatchedTrainStep`` trains many sparse scenes per launch.
"""
from . import _lib
from .grid_functions import (average_pool3d_grid, collect_cell_information_via_indices,
                             convolve_grid_to_remove_noise, find_out_of_bound, fix_out_of_bounds,
                             generate_grid, get_grid_points_indices, get_nearest_voxels, grid_origin,
                             trilinear_interpolation)
from .ray_sampling import (compute_alpha_weighted_pixels, generate_rays_batched,
                           normalize_samples_for_indecies, sample_camera_rays_batched)
from .render import FusedTrainStep, render_rays, render_sample_indices
from .optim import FusedAdam
from .train import Trainer
from .inference import load_checkpoint, save_checkpoint, visulize_3d_in_2d
from .visualization import visulize_3d_in_2d_fast

__all__ = [
    "generate_grid", "grid_origin", "get_nearest_voxels", "find_out_of_bound", "fix_out_of_bounds",
    "get_grid_points_indices", "collect_cell_information_via_indices", "trilinear_interpolation",
    "average_pool3d_grid", "convolve_grid_to_remove_noise",
    "normalize_samples_for_indecies", "generate_rays_batched", "sample_camera_rays_batched",
    "compute_alpha_weighted_pixels", "render_rays", "render_sample_indices", "FusedTrainStep",
    "FusedAdam", "Trainer", "save_checkpoint", "load_checkpoint", "visulize_3d_in_2d",
    "visulize_3d_in_2d_fast", "load_library", "launch_count",
]


def load_library():
    """Loads libplenoxels_gb300.so (raises if it has not been built)."""
    return _lib.load()


def launch_count() -> int:
    """Kernels launched by the library in this process."""
    return int(_lib.load().pgb_launch_count())
