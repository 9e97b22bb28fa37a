"""pgb_render_train_noalloc against pgb_render_train, through the C ABI.

Some callers of this library cannot allocate device memory: their device memory belongs
to another allocator (a framework's caching allocator, or a fixed pool reserved up
front that hands out no extra buffers), or they run a loop that must not allocate once
it has started (a real-time render or training loop with a fixed memory budget). The
no-allocation entry point serves them: it takes the same inputs and outputs as the
regular fused training step but keeps the loss-reduction scratch in a fixed array inside
the library instead of a caller-provided workspace. Its results must equal the regular
entry point's, call after call, because every call reuses that one array.

This file is named so that pytest collects it after every other test file.
"""
import ctypes

import numpy as np
import pytest
import torch

import scenes
from oracle import torch_port as tp
from plenoxels_gb300 import _lib

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _problem(mode, rays=700, side=32, S=96, dtype=torch.float32, alpha_floor=0.0, cameras=False,
             logsum=False):
    grid = torch.from_numpy(scenes.make_grid(side, 4, 41, amp=(0.3, 3), negative_frac=0.02))
    T = torch.from_numpy(scenes.make_cameras(3, 42))
    imgs = torch.from_numpy(scenes.make_images(3, 16, 16, 43))
    o, d, target = tp.camera_batch(T, 0.691, imgs, rays, 44, 2.0)
    pd = scenes.points_distance(side)
    tensors = dict(grid=grid.to(DEV).to(dtype), o=o.to(DEV), d=d.to(DEV), target=target.to(DEV),
                   T=T.to(DEV), imgs=imgs.to(DEV))
    g = _lib.make_grid(tensors["grid"], tp.grid_min(grid.shape, pd).tolist(), pd,
                       _lib.PGB_NEAREST if mode == "nearest" else _lib.PGB_TRILINEAR, True,
                       alpha_floor=alpha_floor)
    r = _lib.PgbRays()
    if cameras:
        cams = _lib.PgbCameras()
        cams.transforms, cams.images = tensors["T"].data_ptr(), tensors["imgs"].data_ptr()
        cams.num_cameras, cams.height, cams.width = 3, 16, 16
        cams.camera_angle_x, cams.near, cams.seed = 0.691, 2.0, 77
        tensors["cams"] = cams  # keeps the descriptor alive
        r.cameras = ctypes.pointer(cams)
    else:
        r.origins, r.dirs = tensors["o"].data_ptr(), tensors["d"].data_ptr()
    r.num_rays, r.num_samples, r.delta_step = rays, S, 4.0 / S
    r.stratified, r.seed = 1, 12345
    r.log_transmittance = 1 if logsum else 0
    return g, r, tensors


def _outputs(t, rays):
    grad = torch.zeros(t["grid"].shape, dtype=torch.float32, device=DEV)
    rgba = torch.full((rays, 4), float("nan"), device=DEV)
    loss = torch.full((), float("nan"), device=DEV)
    return grad, rgba, loss


CASES = {
    "trilinear": dict(mode="trilinear"),
    "nearest": dict(mode="nearest"),
    "alpha_floor": dict(mode="trilinear", alpha_floor=0.3),
    "bf16_cells": dict(mode="trilinear", dtype=torch.bfloat16),
    "camera_rays": dict(mode="trilinear", cameras=True),
    "logsum": dict(mode="nearest", logsum=True),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_no_alloc_train_matches_workspace_train(case):
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    g, r, t = _problem(**CASES[case])
    rays = r.num_rays
    target = t["target"].data_ptr()
    # the regular entry point with a caller workspace
    ws = torch.zeros(lib.pgb_train_workspace_bytes(), dtype=torch.uint8, device=DEV)
    grad_ref, rgba_ref, loss_ref = _outputs(t, rays)
    assert lib.pgb_render_train(ctypes.byref(g), ctypes.byref(r), target, 1.0,
                                rgba_ref.data_ptr(), grad_ref.data_ptr(), loss_ref.data_ptr(),
                                ws.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    scale = float(grad_ref.abs().max())
    assert np.isfinite(float(loss_ref)) and scale > 0
    # two no-allocation calls in a row share the library's scratch array
    for _ in range(2):
        grad, rgba, loss = _outputs(t, rays)
        assert lib.pgb_render_train_noalloc(ctypes.byref(g), ctypes.byref(r), target, 1.0,
                                            rgba.data_ptr(), grad.data_ptr(), loss.data_ptr(),
                                            stream) == 0
        torch.cuda.synchronize()
        np.testing.assert_allclose(float(loss), float(loss_ref), rtol=1e-5)
        np.testing.assert_allclose(rgba.cpu().numpy(), rgba_ref.cpu().numpy(), rtol=1e-5, atol=1e-6)
        assert float((grad - grad_ref).abs().max()) <= 1e-4 * scale


def test_no_alloc_rejects_more_rays_than_its_scratch_holds():
    lib = _lib.load()
    g, r, t = _problem("trilinear", rays=8)
    grad, rgba, loss = _outputs(t, 8)
    r.num_rays = _lib.PGB_NOALLOC_MAX_RAYS + 1
    before = lib.pgb_launch_count()
    st = lib.pgb_render_train_noalloc(ctypes.byref(g), ctypes.byref(r), t["target"].data_ptr(), 1.0,
                                      None, grad.data_ptr(), loss.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    assert st == _lib.PGB_ERR_UNSUPPORTED
    assert lib.pgb_launch_count() == before
