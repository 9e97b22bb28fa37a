"""Fused kernels against the oracle (oracle/torch_port.py, pinned to the reference by
tests/golden) on seeded synthetic scenes: bit-exact voxel indices, forward within 1e-5
relative, gradients within 1e-4 of the largest entry; plus the fp64 adjoint against
central finite differences, BF16 storage against the fp32 path, and edge sizes."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
from plenoxels_gb300 import _lib
import scenes
from oracle import torch_port as tp

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _grad_close(got, ref, rel=1e-4):
    got = got.detach().cpu().double().numpy() if torch.is_tensor(got) else got
    ref = ref.detach().cpu().double().numpy() if torch.is_tensor(ref) else ref
    scale = np.abs(ref).max()
    err = np.abs(got - ref).max()
    assert err <= rel * scale + 1e-12, f"max grad error {err:.3e} vs scale {scale:.3e}"


def _scene(side, n_cams, rays, seed, near=2.0, far=6.0, S=64, amp=(5, 20), neg=0.0):
    grid = torch.from_numpy(scenes.make_grid(side, 4, seed, amp=amp, negative_frac=neg))
    T = torch.from_numpy(scenes.make_cameras(n_cams, seed + 1))
    imgs = torch.from_numpy(scenes.make_images(n_cams, 32, 32, seed + 2))
    o, d, target = tp.camera_batch(T, 0.691, imgs, rays, seed + 3, near)
    delta = (far - near) / S
    return grid, T, imgs, o, d, target, delta


CASES = [
    # side, cams, rays, S, mode, stratified, amp, neg
    (32, 3, 300, 64, "trilinear", False, (5, 20), 0.0),
    (32, 3, 300, 64, "nearest", False, (0.2, 2), 0.05),
    (48, 4, 200, 256, "trilinear", True, (0.2, 3), 0.02),
    (48, 4, 200, 256, "nearest", True, (5, 20), 0.0),
    (24, 2, 100, 600, "trilinear", False, (0.1, 1), 0.0),   # reference default S, 3 chunks
    (24, 2, 64, 512, "trilinear", True, (0.1, 1), 0.0),     # 16 slots per lane
    (16, 2, 50, 17, "nearest", False, (0.5, 2), 0.1),       # ragged S
    (16, 1, 33, 1, "trilinear", False, (0.5, 2), 0.1),      # single sample
]


@pytest.mark.parametrize("side,cams,rays,S,mode,strat,amp,neg", CASES)
def test_fused_matches_oracle(side, cams, rays, S, mode, strat, amp, neg):
    grid, T, imgs, o, d, target, delta = _scene(side, cams, rays, side + S, S=S, amp=amp, neg=neg)
    pd = scenes.points_distance(side)
    gmin = tp.grid_min(grid.shape, pd)
    jitter = tp.jitter_for(9, rays, S) if strat else None
    # oracle (CPU)
    g_ref = grid.clone().requires_grad_(True)
    px_ref = tp.render(g_ref, o, d, S, delta, gmin, pd, mode, True, jitter)
    idx_ref, inb_ref = tp.sample_indices(o, d, S, delta, gmin, pd, grid.shape, mode, jitter)
    loss_ref = torch.nn.functional.mse_loss(px_ref, target)
    loss_ref.backward()
    # CUDA
    g = grid.to(DEV).requires_grad_(True)
    od, dd = o.to(DEV), d.to(DEV)
    idx, inb = pg.render_sample_indices(g, od, dd, delta, S, pd, mode=mode, stratified=strat, seed=9)
    np.testing.assert_array_equal(idx.cpu().numpy().reshape(-1), idx_ref.numpy().reshape(-1))
    np.testing.assert_array_equal(inb.cpu().numpy().reshape(-1), inb_ref.numpy())
    px = pg.render_rays(g, od, dd, delta, S, pd, mode=mode, stratified=strat, seed=9)
    np.testing.assert_allclose(px.detach().cpu().numpy(), px_ref.detach().numpy(), rtol=1e-5, atol=2e-6)
    loss = torch.nn.functional.mse_loss(px, target.to(DEV))
    loss.backward()
    _grad_close(g.grad, g_ref.grad)
    # fused training step: same loss and gradient in one launch
    step = pg.FusedTrainStep(g.detach(), pd, S, delta, mode=mode, stratified=strat, seed=9)
    l2 = step.step_rays(od, dd, target.to(DEV))
    np.testing.assert_allclose(float(l2), float(loss_ref), rtol=1e-5)
    _grad_close(step.grad, g_ref.grad)


@pytest.mark.parametrize("mode", ["nearest", "trilinear"])
def test_camera_rays_generated_in_kernel(mode):
    side, S, rays = 40, 128, 1000
    grid = torch.from_numpy(scenes.make_grid(side, 4, 3, amp=(0.3, 3)))
    T = torch.from_numpy(scenes.make_cameras(7, 4))
    imgs = torch.from_numpy(scenes.make_images(7, 24, 24, 5))
    pd, near, far = scenes.points_distance(side), 2.0, 6.0
    delta = (far - near) / S
    o, d, target = tp.camera_batch(T, 0.691, imgs, rays, 77, near)
    gmin = tp.grid_min(grid.shape, pd)
    g_ref = grid.clone().requires_grad_(True)
    px_ref = tp.render(g_ref, o, d, S, delta, gmin, pd, mode, True, tp.jitter_for(5, rays, S))
    loss_ref = torch.nn.functional.mse_loss(px_ref, target)
    loss_ref.backward()
    g = grid.to(DEV)
    step = pg.FusedTrainStep(g, pd, S, delta, mode=mode, stratified=True, seed=5)
    rgba = torch.empty(rays, 4, device=DEV)
    loss = step.step_cameras(T.to(DEV), imgs.to(DEV), 0.691, rays, 77, near=near, rgba_out=rgba)
    np.testing.assert_allclose(rgba.cpu().numpy(), px_ref.detach().numpy(), rtol=1e-5, atol=2e-6)
    np.testing.assert_allclose(float(loss), float(loss_ref), rtol=1e-5)
    _grad_close(step.grad, g_ref.grad)


def test_fp64_adjoint_matches_central_differences():
    """32^3 fp64 grid, 1024 rays, 64 samples, trilinear: the fp64 adjoint against
    central differences (eps 1e-4) of the fp64 oracle on 200 random entries, and against
    the oracle's autograd gradient over all cells."""
    side, S, rays = 32, 64, 1024
    grid = torch.from_numpy(scenes.make_grid(side, 3, 21, amp=(0.2, 0.9))).double()
    T = torch.from_numpy(scenes.make_cameras(4, 22))
    imgs = torch.from_numpy(scenes.make_images(4, 16, 16, 23))
    o, d, target = tp.camera_batch(T, 0.691, imgs, rays, 24, 2.0)
    o, d, target = o.double(), d.double(), target.double()
    pd, delta = scenes.points_distance(side), 4.0 / S
    gmin = tp.grid_min(grid.shape, pd, torch.float64)
    g = grid.to(DEV).requires_grad_(True)
    px = pg.render_rays(g, o.to(DEV), d.to(DEV), delta, S, pd, grid_min=gmin.tolist())
    loss = torch.nn.functional.mse_loss(px, target.to(DEV))
    loss.backward()
    grad = g.grad.cpu().numpy()
    g_ref = grid.clone().requires_grad_(True)
    tp.train_loss(g_ref, o, d, target, S, delta, gmin, pd).backward()
    _grad_close(grad, g_ref.grad, rel=1e-10)
    # central differences on entries with a non-zero gradient whose value stays inside
    # the clip range [0, 1] under +-eps (the loss has a kink at the clip boundary)
    eps = 1e-4
    rng = np.random.default_rng(0)
    gv = grid.numpy()
    cand = np.argwhere((np.abs(grad) > 1e-8 * np.abs(grad).max()) & (gv > 2 * eps) & (gv < 1 - 2 * eps))
    pick = cand[rng.choice(len(cand), size=min(200, len(cand)), replace=False)]
    worst = 0.0
    with torch.no_grad():
        for i, j, k, c in pick:
            gp = grid.clone(); gp[i, j, k, c] += eps
            gm = grid.clone(); gm[i, j, k, c] -= eps
            lp = tp.train_loss(gp, o, d, target, S, delta, gmin, pd)
            lm = tp.train_loss(gm, o, d, target, S, delta, gmin, pd)
            fd = float(lp - lm) / (2 * eps)
            worst = max(worst, abs(fd - grad[i, j, k, c]) / max(abs(fd), 1e-3 * np.abs(grad).max()))
    assert worst < 1e-4, f"max relative error vs central differences {worst:.2e}"


def test_bf16_storage_matches_fp32_on_rounded_grid():
    side, S, rays = 48, 256, 500
    grid = torch.from_numpy(scenes.make_grid(side, 6, 31, amp=(0.3, 3)))
    g16 = grid.to(torch.bfloat16)
    g32 = g16.float()  # the values the bf16 kernel sees
    T = torch.from_numpy(scenes.make_cameras(3, 32))
    imgs = torch.from_numpy(scenes.make_images(3, 16, 16, 33))
    o, d, target = tp.camera_batch(T, 0.691, imgs, rays, 34, 2.0)
    pd, delta = scenes.points_distance(side), 4.0 / S
    a = pg.FusedTrainStep(g16.to(DEV), pd, S, delta)
    b = pg.FusedTrainStep(g32.to(DEV), pd, S, delta)
    ra, rb = torch.empty(rays, 4, device=DEV), torch.empty(rays, 4, device=DEV)
    la = a.step_rays(o.to(DEV), d.to(DEV), target.to(DEV), rgba_out=ra)
    lb = b.step_rays(o.to(DEV), d.to(DEV), target.to(DEV), rgba_out=rb)
    assert a.grad.dtype == torch.float32
    np.testing.assert_allclose(ra.cpu().numpy(), rb.cpu().numpy(), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(float(la), float(lb), rtol=1e-6)
    _grad_close(a.grad, b.grad, rel=1e-6)


def test_empty_batches_and_zero_samples():
    grid = torch.rand(8, 8, 8, 4, device=DEV, requires_grad=True)
    o = torch.zeros(0, 3, device=DEV)
    px = pg.render_rays(grid, o, o, 0.1, 16, 0.25)
    assert px.shape == (0, 4)
    o1 = torch.tensor([[0.0, 0.0, -3.0]], device=DEV)
    d1 = torch.tensor([[0.0, 0.0, 1.0]], device=DEV)
    px = pg.render_rays(grid, o1, d1, 0.1, 0, 0.25)
    assert px.shape == (1, 4) and float(px.abs().sum()) == 0.0
    px.sum().backward()
    assert float(grid.grad.abs().sum()) == 0.0


def test_non_contiguous_grid_view_gets_gradient():
    """A permuted view (the pooled grid of scripts/train.py:118) is made contiguous by the
    wrapper and autograd carries the gradient back through the permute."""
    base = torch.rand(4, 16, 16, 16, device=DEV, requires_grad=True)
    view = base.permute(1, 2, 3, 0)
    assert not view.is_contiguous()
    o = torch.tensor([[0.05, -0.02, -3.0]], device=DEV)
    d = torch.tensor([[0.0, 0.0, 1.0]], device=DEV)
    px = pg.render_rays(view, o, d, 0.05, 120, 3.0 / 16)
    px.sum().backward()
    ref_grid = view.detach().cpu().requires_grad_(True)
    ref = tp.render(ref_grid, o.cpu(), d.cpu(), 120, 0.05, tp.grid_min(ref_grid.shape, 3.0 / 16),
                    3.0 / 16)
    ref.sum().backward()
    np.testing.assert_allclose(px.detach().cpu().numpy(), ref.detach().numpy(), rtol=1e-5, atol=1e-6)
    _grad_close(base.grad.permute(1, 2, 3, 0), ref_grid.grad)


def test_determinism_of_forward_and_loss():
    grid, T, imgs, o, d, target, delta = _scene(32, 3, 500, 5, S=128)
    pd = scenes.points_distance(32)
    g = grid.to(DEV)
    step = pg.FusedTrainStep(g, pd, 128, delta)
    r1, r2 = torch.empty(500, 4, device=DEV), torch.empty(500, 4, device=DEV)
    l1 = float(step.step_rays(o.to(DEV), d.to(DEV), target.to(DEV), rgba_out=r1))
    g1 = step.grad.clone()
    l2 = float(step.step_rays(o.to(DEV), d.to(DEV), target.to(DEV), rgba_out=r2))
    assert l1 == l2
    assert torch.equal(r1, r2)
    _grad_close(step.grad, g1, rel=1e-6)  # atomics: order may differ, values agree


def test_overlapped_gradient_zeroing_gives_the_same_steps():
    """overlap_zero=True zeroes the next step's gradient buffer on a side stream; every
    step must still see a fully zeroed buffer and produce the serial result."""
    grid = torch.from_numpy(scenes.make_grid(32, 4, 51, amp=(0.3, 3))).to(DEV)
    T = torch.from_numpy(scenes.make_cameras(5, 52)).to(DEV)
    imgs = torch.from_numpy(scenes.make_images(5, 16, 16, 53)).to(DEV)
    pd, S = scenes.points_distance(32), 128
    a = pg.FusedTrainStep(grid, pd, S, 4.0 / S, stratified=True, seed=3, overlap_zero=True)
    b = pg.FusedTrainStep(grid, pd, S, 4.0 / S, stratified=True, seed=3)
    seen = set()
    for i in range(5):
        la = a.step_cameras(T, imgs, 0.691, 900, 100 + i, near=2.0)
        lb = b.step_cameras(T, imgs, 0.691, 900, 100 + i, near=2.0)
        seen.add(a.grad.data_ptr())
        torch.cuda.synchronize()
        assert float(la) == float(lb)
        _grad_close(a.grad, b.grad, rel=1e-6)
    assert len(seen) == 2, "the two gradient buffers alternate"


def test_random_access_probes_stay_inside_their_table():
    """The memory probes behind the roofline report: every atomic lands in the table
    (its sum is exactly 4 per update) and the read probe completes."""
    from plenoxels_gb300 import probes
    lib = probes.load()
    stream = torch.cuda.current_stream().cuda_stream
    table = torch.zeros(1000 * 4, device=DEV)  # 1000 slots of 16 B
    n = 123457
    _lib.check(lib.pgb_probe_random_atomics(table.data_ptr(), table.numel() * 4, n, 5, stream), "atomics")
    assert float(table.double().sum()) == 4.0 * n
    hit = table.view(-1, 4)[:, 0] > 0
    assert int(hit.sum()) > 900  # the slots are spread over the whole table
    sink = torch.zeros(1, device=DEV)
    _lib.check(lib.pgb_probe_random_reads(table.data_ptr(), table.numel() * 4, n, 6, sink.data_ptr(), stream), "reads")
    torch.cuda.synchronize()
    assert float(sink) == 0.0


def _parity(grid, o, d, target, S, delta, pd, gmin, mode, strat=False, seed=9):
    """Indices bit-exact, forward within 1e-5, gradients within 1e-4 of the largest entry,
    through both the autograd path and the fused training step."""
    jitter = tp.jitter_for(seed, o.shape[0], S) if strat else None
    g_ref = grid.clone().requires_grad_(True)
    px_ref = tp.render(g_ref, o, d, S, delta, gmin, pd, mode, True, jitter)
    idx_ref, inb_ref = tp.sample_indices(o, d, S, delta, gmin, pd, grid.shape, mode, jitter)
    loss_ref = torch.nn.functional.mse_loss(px_ref, target)
    loss_ref.backward()
    gmin = tuple(float(x) for x in gmin)
    g = grid.to(DEV).requires_grad_(True)
    od, dd = o.to(DEV), d.to(DEV)
    idx, inb = pg.render_sample_indices(g, od, dd, delta, S, pd, grid_min=gmin, mode=mode,
                                        stratified=strat, seed=seed)
    np.testing.assert_array_equal(idx.cpu().numpy().reshape(-1), idx_ref.numpy().reshape(-1))
    np.testing.assert_array_equal(inb.cpu().numpy().reshape(-1), inb_ref.numpy())
    px = pg.render_rays(g, od, dd, delta, S, pd, grid_min=gmin, mode=mode, stratified=strat, seed=seed)
    np.testing.assert_allclose(px.detach().cpu().numpy(), px_ref.detach().numpy(), rtol=1e-5, atol=2e-6)
    torch.nn.functional.mse_loss(px, target.to(DEV)).backward()
    _grad_close(g.grad, g_ref.grad)
    step = pg.FusedTrainStep(g.detach(), pd, S, delta, mode=mode, grid_min=gmin, stratified=strat, seed=seed)
    loss = step.step_rays(od, dd, target.to(DEV))
    np.testing.assert_allclose(float(loss), float(loss_ref), rtol=1e-5)
    _grad_close(step.grad, g_ref.grad)
    return px_ref, g_ref.grad


@pytest.mark.parametrize("mode", ["nearest", "trilinear"])
def test_non_cubic_grid_matches_oracle(mode):
    """X != Y != Z (the kernels index with all three extents; the reference's own grids
    are cubic but nothing in the path assumes it)."""
    g = torch.Generator().manual_seed(31)
    grid = torch.rand(20, 28, 12, 4, generator=g) * 1.2 - 0.1   # some channels outside [0,1]
    grid[..., 3] *= 0.1  # translucent enough that most samples carry gradient
    pd = 0.11
    gmin = tp.grid_min(grid.shape, pd)
    T = torch.from_numpy(scenes.make_cameras(3, 32))
    imgs = torch.from_numpy(scenes.make_images(3, 16, 16, 33))
    o, d, target = tp.camera_batch(T, 0.691, imgs, 240, 34, 2.0)
    _parity(grid, o, d, target, 96, 4.0 / 96, pd, gmin, mode)


def test_maximum_samples_per_ray_matches_oracle():
    """8192 samples per ray (32 chunks of 256, the largest the kernels take), stratified."""
    grid = torch.from_numpy(scenes.make_grid(16, 3, 41, amp=(0.05, 0.3)))
    pd = scenes.points_distance(16)
    gmin = tp.grid_min(grid.shape, pd)
    T = torch.from_numpy(scenes.make_cameras(2, 42))
    imgs = torch.from_numpy(scenes.make_images(2, 16, 16, 43))
    o, d, target = tp.camera_batch(T, 0.691, imgs, 12, 44, 2.0)
    S = 8192
    _parity(grid, o, d, target, S, 4.0 / S, pd, gmin, "trilinear", strat=True)
    with pytest.raises(NotImplementedError):
        pg.render_rays(grid.to(DEV), o.to(DEV), d.to(DEV), 4.0 / S, S + 1, pd)


@pytest.mark.parametrize("side", [1, 2])
def test_tiny_grids_match_oracle(side):
    """One- and two-cell grids: every trilinear ceil corner wraps to index 0."""
    g = torch.Generator().manual_seed(50 + side)
    grid = torch.rand(side, side, side, 4, generator=g)
    grid[..., 3] *= 0.1
    pd = 1.5 / side
    gmin = tp.grid_min(grid.shape, pd)
    o = torch.tensor([[-2.0, 0.1, 0.05], [0.2, -2.0, 0.3], [0.01, 0.02, -2.0]]).repeat(8, 1)
    o = o + 0.05 * torch.rand(o.shape, generator=g)
    d = torch.nn.functional.normalize(-o + 0.1 * torch.rand(o.shape, generator=g), dim=1)
    target = torch.rand(o.shape[0], 4, generator=g)
    for mode in ("nearest", "trilinear"):
        _parity(grid, o, d, target, 64, 4.0 / 64, pd, gmin, mode)


def test_rays_that_miss_the_grid():
    """Every sample outside the box: RGBA 0, loss = mean(target^2), no gradient."""
    grid = torch.rand(16, 16, 16, 4, device=DEV)
    o = torch.tensor([[5.0, 5.0, 5.0], [-5.0, 0.0, 0.0]], device=DEV)
    d = torch.tensor([[0.0, 0.0, 1.0], [-1.0, 0.0, 0.0]], device=DEV)
    target = torch.rand(2, 4, device=DEV)
    step = pg.FusedTrainStep(grid, 0.2, 128, 0.05)
    loss = step.step_rays(o, d, target)
    assert abs(float(loss) - float((target ** 2).mean())) <= 1e-7
    assert float(step.grad.abs().sum()) == 0.0
    px = pg.render_rays(grid, o, d, 0.05, 128, 0.2)
    assert float(px.abs().sum()) == 0.0


@pytest.mark.parametrize("mode", ["nearest", "trilinear"])
def test_rays_clipped_to_the_grid_match_oracle(mode):
    """Chunks whose samples all lie outside the grid are skipped: axis-parallel rays
    (zero direction components) inside and outside the box's slabs, rays starting inside
    the grid, rays pointing away from it, grazing rays along a face, and long rays that
    cross the box in a few of many chunks must give the oracle's results."""
    g = torch.Generator().manual_seed(61)
    side = 24
    grid = torch.rand(side, side, side, 4, generator=g)
    grid[..., 3] *= 0.15
    pd = scenes.points_distance(side)
    gmin = tp.grid_min(grid.shape, pd)
    lo = float(gmin[0])
    hi = lo + side * pd
    rays = [
        ([-3.0, 0.1, 0.2], [1.0, 0.0, 0.0]),      # x-parallel through the box
        ([-3.0, 2.0, 0.2], [1.0, 0.0, 0.0]),      # x-parallel, outside the y slab
        ([0.1, 0.2, 0.3], [0.0, 1.0, 0.0]),       # starts inside
        ([0.1, -0.2, 0.3], [0.3, 0.4, 0.866]),    # starts inside, oblique
        ([3.0, 3.0, 3.0], [0.577, 0.577, 0.577]), # points away
        ([-3.0, lo, 0.0], [1.0, 0.0, 0.0]),       # along the lower y face
        ([-3.0, hi, 0.0], [1.0, 0.0, 0.0]),       # along the upper y face (outside)
        ([-3.0, 0.0, hi - 0.5 * pd], [1.0, 0.0, 0.0]),  # inside the last z cell
        ([0.0, 0.0, -9.0], [0.0, 0.0, 1.0]),      # long way to the box
    ]
    o = torch.tensor([r[0] for r in rays], dtype=torch.float32)
    d = torch.nn.functional.normalize(torch.tensor([r[1] for r in rays], dtype=torch.float32), dim=1)
    target = torch.rand(o.shape[0], 4, generator=g)
    _parity(grid, o, d, target, 1200, 12.0 / 1200, pd, gmin, mode, strat=True)
    _parity(grid, o, d, target, 96, 0.06, pd, gmin, mode)


@pytest.mark.parametrize("mode", ["nearest", "trilinear"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_early_stop_behind_opaque_cells_is_exact(mode, dtype):
    """Rays stop after the chunk where their transmittance reaches 0. The first opaque
    sample's own alpha gradient reads the samples behind it when the clamp passes it (a
    stored alpha of exactly 1.0), so every chunk size must give the oracle's loss and
    gradient, on a grid where opaque cells hold exactly 1.0 or values above 1."""
    side, S, R = 32, 256, 600
    g = scenes.make_grid(side, 5, 201, amp=(0.8, 6.0))
    rng = np.random.default_rng(202)
    a = g[..., 3]
    opaque = a >= 1.0
    a[opaque & (rng.random(a.shape) < 0.5)] = 1.0  # clamp gradient open at exactly 1
    a[(a > 0.9) & (a < 1.0)] = 1.0
    grid = torch.from_numpy(g).to(dtype).float()  # the values the kernels see
    assert int((grid[..., 3] == 1.0).sum()) > 100 and int((grid[..., 3] > 1.0).sum()) > 100
    T = torch.from_numpy(scenes.make_cameras(4, 203))
    imgs = torch.from_numpy(scenes.make_images(4, 16, 16, 204))
    o, d, tgt = tp.camera_batch(T, 0.691, imgs, R, 205, 2.0)
    pd, delta = scenes.points_distance(side), 4.0 / S
    ref = grid.clone().requires_grad_(True)
    loss = tp.train_loss(ref, o, d, tgt, S, delta, tp.grid_min(grid.shape, pd), pd, mode)
    loss.backward()
    for chunk in (32, 64, 128, 256):
        step = pg.FusedTrainStep(grid.to(dtype).to(DEV), pd, S, delta, mode=mode,
                                 chunk_samples=chunk)
        rgba = torch.empty(R, 4, device=DEV)
        got = step.step_rays(o.to(DEV), d.to(DEV), tgt.to(DEV), rgba_out=rgba)
        torch.cuda.synchronize()
        np.testing.assert_allclose(float(got), float(loss), rtol=1e-5, err_msg=f"chunk {chunk}")
        _grad_close(step.grad, ref.grad)


@pytest.mark.parametrize("mode", ["trilinear", "nearest"])
@pytest.mark.parametrize("overlap", [False, True])
def test_marked_zeroing_gives_the_dense_steps(mode, overlap):
    """zeroing="marked" re-zeroes only the 4-cell units the buffer's last step wrote; over
    steps on different rays (each touching other cells) every step must see an all-zero
    buffer, so its gradient equals the dense-fill step's, zeros included; an accumulating
    step (zero_grad=False) and the next zeroing clear its units too."""
    grid = torch.from_numpy(scenes.make_grid(32, 4, 91, amp=(0.3, 3))).to(DEV)
    T = torch.from_numpy(scenes.make_cameras(5, 92)).to(DEV)
    imgs = torch.from_numpy(scenes.make_images(5, 16, 16, 93)).to(DEV)
    pd, S = scenes.points_distance(32), 128
    a = pg.FusedTrainStep(grid, pd, S, 4.0 / S, mode=mode, stratified=True, seed=3,
                          overlap_zero=overlap, zeroing="marked")
    b = pg.FusedTrainStep(grid, pd, S, 4.0 / S, mode=mode, stratified=True, seed=3)
    for i in range(6):
        acc = i == 3
        la = a.step_cameras(T, imgs, 0.691, 700, 300 + i, near=2.0, zero_grad=not acc)
        lb = b.step_cameras(T, imgs, 0.691, 700, 300 + i, near=2.0, zero_grad=not acc)
        torch.cuda.synchronize()
        np.testing.assert_allclose(float(la), float(lb), rtol=1e-6)
        # a cell left over from an earlier step would differ by that step's gradient
        _grad_close(a.grad, b.grad, rel=1e-6)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("num_cells", [1000, 128 * 40 + 3, 256 * 1024 + 130])
def test_clear_marked_zeroes_exactly_the_marked_units(dtype, num_cells):
    """pgb_clear_marked zeroes the cells of every marked unit (bit u%32 of word u/32, a
    unit being the cells the library's mark layout groups, pgb_mark_words words), leaves
    every other cell as it was, stops at num_cells (a ragged last unit and word) and
    leaves the bitmap all zero; words with every bit set, none, and random sparse bits."""
    lib = _lib.load()
    rng = np.random.default_rng(num_cells)
    words = lib.pgb_mark_words(num_cells)
    per_unit = next(p for p in (1, 2, 4, 8) if ((num_cells + p - 1) // p + 31) // 32 == words)
    units = (num_cells + per_unit - 1) // per_unit
    bits = rng.random(words * 32) < 0.05
    bits[: 32 * min(3, words)] = True  # full words at the start
    bits[32 * 5: 32 * 7] = False       # empty words
    bits[units - 1] = True             # the ragged last unit
    bits[units:] = False               # no unit past the cells
    words_np = np.packbits(bits.reshape(words, 32)[:, ::-1], axis=1, bitorder="big")
    marks_np = words_np.view(">u4").astype(np.uint32).reshape(words)
    grad = torch.arange(1, num_cells * 4 + 1, dtype=dtype, device=DEV).reshape(num_cells, 4)
    marks = torch.from_numpy(marks_np.view(np.int32)).to(DEV)
    before = grad.clone()
    cell_bytes = 4 * grad.element_size()
    st = lib.pgb_clear_marked(grad.data_ptr(), cell_bytes, num_cells, marks.data_ptr(),
                              torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    cell_marked = torch.from_numpy(np.repeat(bits[:units], per_unit)[:num_cells]).to(DEV)
    expect = torch.where(cell_marked[:, None], torch.zeros_like(before), before)
    assert torch.equal(grad, expect)
    assert int(marks.abs().sum()) == 0


@pytest.mark.parametrize("mode", ["trilinear", "nearest"])
def test_loss_written_into_pinned_host_memory(mode):
    """loss_out in pinned host memory: the kernel writes the step's losses there directly,
    the same values as into the step's own device buffer (same inputs, same kernel), and
    the gradient is the same; other tensors are rejected."""
    grid, T, imgs, o, d, target, delta = _scene(24, 3, 200, 61, S=96)
    pd = scenes.points_distance(24)
    g = grid.to(DEV)
    od, dd, td = o.to(DEV), d.to(DEV), target.to(DEV)
    a = pg.FusedTrainStep(g, pd, 96, delta, mode=mode, stratified=True, seed=4, beta=1e-3)
    b = pg.FusedTrainStep(g, pd, 96, delta, mode=mode, stratified=True, seed=4, beta=1e-3)
    host = torch.full((2,), -1.0, dtype=torch.float32).pin_memory()
    la = a.step_rays(od, dd, td)
    lb = b.step_rays(od, dd, td, loss_out=host)
    torch.cuda.synchronize()
    assert lb.data_ptr() == host.data_ptr()
    assert float(host[0]) == float(la) and float(host[1]) == float(a.losses[1])
    _grad_close(b.grad, a.grad, rel=1e-6)  # float atomics: run-dependent summation order
    with pytest.raises(ValueError):
        b.step_rays(od, dd, td, loss_out=torch.zeros(2))  # not pinned
    with pytest.raises(ValueError):
        b.step_rays(od, dd, td, loss_out=torch.zeros(2, dtype=torch.float64).pin_memory())
    with pytest.raises(ValueError):
        b.step_rays(od, dd, td, loss_out=torch.zeros(1).pin_memory())
