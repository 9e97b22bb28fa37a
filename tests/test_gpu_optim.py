"""The optimiser side of the training step against torch.optim.Adam and the oracle's
restatement of the reference's TV and beta losses (scripts/train.py:44-65, :89,
:163-184), and a few full training steps against the reference's loop.

Tolerances: Adam parameters within 1e-6 relative (same formula, fp32); TV sum of squares
within 1e-6 relative (fp64 reduction of fp32 partials); gradients within 1e-5 of their
largest entry; loss trajectories within 1e-4 relative."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes
from oracle import torch_port as tp
from plenoxels_gb300.optim import FusedAdam
from plenoxels_gb300.train import Trainer

pytestmark = pytest.mark.gpu
DEV = "cuda"


def test_adam_matches_torch_adam_and_clears_the_gradient():
    torch.manual_seed(0)
    p0 = torch.randn(12, 10, 8, 4, device=DEV)
    ref = p0.clone().requires_grad_(True)
    topt = torch.optim.Adam([ref], lr=0.0075)
    mine = p0.clone()
    opt = FusedAdam(mine, lr=0.0075)
    acc = torch.zeros_like(p0)
    for i in range(6):
        g = torch.randn_like(p0) * (10.0 ** (i - 3))
        ref.grad = g.clone()
        topt.step()
        gm = g.clone()
        opt.step(gm)
        acc += g.abs()
        assert float(gm.abs().max()) == 0.0
        np.testing.assert_allclose(mine.cpu().numpy(), ref.detach().cpu().numpy(), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(opt.abs_grad.cpu().numpy(), acc.cpu().numpy(), rtol=1e-6)


@pytest.mark.parametrize("shape", [(16, 16, 16, 4), (7, 5, 9, 4), (1, 3, 2, 4)])
def test_tv_loss_and_gradient_match_the_reference_formula(shape):
    torch.manual_seed(1)
    grid = torch.rand(shape, device=DEV)
    g = grid.clone().requires_grad_(True)
    w = 1e-2
    (w * tp.tv_loss(g)).backward()
    opt = FusedAdam(grid.clone(), lr=0.1)
    opt.grid.copy_(grid)
    grad = torch.zeros_like(grid)
    val = opt.add_tv(grad, w)
    torch.cuda.synchronize()
    ref_val = float(w * tp.tv_loss(grid))
    np.testing.assert_allclose(float(val), ref_val, rtol=1e-6)
    scale = float(g.grad.abs().max())
    assert float((grad - g.grad).abs().max()) <= 1e-5 * scale


@pytest.mark.parametrize("mode", ["nearest", "trilinear"])
def test_beta_loss_fused_in_the_train_kernel(mode):
    side, S, R = 24, 96, 300
    grid = torch.from_numpy(scenes.make_grid(side, 3, 61, amp=(0.2, 1.5), negative_frac=0.05))
    T = torch.from_numpy(scenes.make_cameras(3, 62))
    imgs = torch.from_numpy(scenes.make_images(3, 8, 8, 63))
    o, d, tgt = tp.camera_batch(T, 0.691, imgs, R, 64, 2.0)
    pd, delta, beta = scenes.points_distance(side), 4.0 / S, 5e-3
    g = grid.clone().requires_grad_(True)
    gmin = tp.grid_min(g.shape, pd)
    px, vals = tp.render_samples(g, o, d, S, delta, gmin, pd, mode)
    mse = torch.nn.functional.mse_loss(px, tgt)
    bl = beta * tp.beta_loss(vals[..., -1])
    (mse + bl).backward()
    step = pg.FusedTrainStep(grid.to(DEV), pd, S, delta, mode=mode, beta=beta)
    step.step_rays(o.to(DEV), d.to(DEV), tgt.to(DEV))
    torch.cuda.synchronize()
    np.testing.assert_allclose(float(step.losses[0]), float(mse), rtol=1e-5)
    np.testing.assert_allclose(float(step.losses[1]), float(bl), rtol=1e-5)
    scale = float(g.grad.abs().max())
    assert float((step.grad.cpu() - g.grad).abs().max()) <= 1e-4 * scale


def test_training_steps_follow_the_reference_loop():
    """Five steps of scripts/train.py:142-184 (nearest lookup, MSE + TV + beta, Adam).

    At every step the trainer's own gradient (render + beta + TV, as its Adam pass
    receives it) is checked against the oracle's autograd gradient of the reference's loss
    at the same pre-step grid, and the same gradient is fed to torch.optim.Adam, so that
    differences cannot compound: after every step the grid, both moments and the |grad|
    accumulator (:184) must agree with the reference optimiser to 1e-6 relative."""
    side, S, R = 24, 64, 400
    grid0 = torch.from_numpy(scenes.make_grid(side, 3, 71, amp=(0.2, 1.5)))
    T = torch.from_numpy(scenes.make_cameras(4, 72))
    imgs = torch.from_numpy(scenes.make_images(4, 8, 8, 73))
    pd, delta, lr, tv, beta = scenes.points_distance(side), 4.0 / S, 0.0075, 1e-5, 5e-3
    gmin = tp.grid_min(grid0.shape, pd)
    ref = torch.nn.Parameter(grid0.clone())
    topt = torch.optim.Adam([ref], lr=lr, foreach=False)
    trainer = Trainer(grid0.to(DEV), pd, S, delta, lr, tv=tv, beta=beta, mode="nearest",
                      fuse_tv=False)
    captured = []
    adam_step = trainer.opt.step

    def spy(grad=None, zero_grad=True):
        captured.append(grad.detach().clone())
        return adam_step(grad, zero_grad)

    trainer.opt.step = spy
    acc = torch.zeros_like(grid0)
    for i in range(5):
        o, d, tgt = tp.camera_batch(T, 0.691, imgs, R, 80 + i, 2.0)
        # the reference's loss and gradient at the trainer's pre-step grid
        g = trainer.grid.detach().cpu().clone().requires_grad_(True)
        px, vals = tp.render_samples(g, o, d, S, delta, gmin, pd, "nearest")
        mse = torch.nn.functional.mse_loss(px, tgt)
        tvl = tv * tp.tv_loss(g)
        bl = beta * tp.beta_loss(vals[..., -1])
        (mse + tvl + bl).backward()
        losses = trainer.step_rays(o.to(DEV), d.to(DEV), tgt.to(DEV)).cpu()
        np.testing.assert_allclose(losses.numpy(), [float(mse), float(tvl), float(bl)], rtol=1e-5)
        G = captured[-1].cpu()
        scale = float(g.grad.abs().max())
        assert float((G - g.grad).abs().max()) <= 1e-4 * scale, f"step {i}: gradient"
        # the reference optimiser on the trainer's own gradient
        ref.grad = G.clone()
        topt.step()
        acc += G.abs()
        st = topt.state[ref]
        for name, got, want in (("grid", trainer.grid, ref.detach()),
                                ("exp_avg", trainer.opt.exp_avg, st["exp_avg"]),
                                ("exp_avg_sq", trainer.opt.exp_avg_sq, st["exp_avg_sq"]),
                                ("abs_grad", trainer.opt.abs_grad, acc)):
            np.testing.assert_allclose(got.cpu().numpy(), want.numpy(), rtol=1e-6,
                                       atol=1e-6 * float(want.abs().max()),
                                       err_msg=f"step {i}: {name}")


def test_fused_tv_adam_pass_equals_the_separate_passes():
    """On the same gradient, the TV gradient evaluated inside the Adam pass (two grid
    buffers) gives bit-identical grids, moments, accumulators and TV values to the TV
    gradient pass followed by Adam; over whole training steps (whose gradients are summed
    by atomics in a run-dependent order) the two trainers agree to rounding."""
    from plenoxels_gb300.optim import FusedAdam
    g = torch.Generator(device=DEV).manual_seed(95)
    grid0 = torch.rand(20, 28, 12, 4, generator=g, device=DEV)
    opts = {fuse: FusedAdam(grid0.clone(), 0.0075) for fuse in (True, False)}
    spare = torch.empty_like(grid0)
    for i in range(3):
        grad = 1e-2 * torch.randn(grid0.shape, generator=g, device=DEV)
        ga, gb = grad.clone(), grad.clone()
        old = opts[True].grid
        tv_a = opts[True].step_tv(ga, 1e-3, spare)
        spare = old
        tv_b = opts[False].add_tv(gb, 1e-3)
        opts[False].step(gb)
        assert torch.equal(tv_a, tv_b)
        assert float(ga.abs().sum()) == 0.0 and float(gb.abs().sum()) == 0.0
    a, b = opts[True], opts[False]
    for x, y in ((a.grid, b.grid), (a.exp_avg, b.exp_avg), (a.exp_avg_sq, b.exp_avg_sq),
                 (a.abs_grad, b.abs_grad)):
        assert torch.equal(x, y)
    assert not torch.equal(a.grid, grid0)
    # whole steps through Trainer
    side, S, R = 20, 48, 300
    gridt = torch.from_numpy(scenes.make_grid(side, 3, 91, amp=(0.2, 1.5))).to(DEV)
    T = torch.from_numpy(scenes.make_cameras(3, 92))
    imgs = torch.from_numpy(scenes.make_images(3, 8, 8, 93))
    pd, delta = scenes.points_distance(side), 4.0 / S
    runs = {}
    for fuse in (True, False):
        tr = Trainer(gridt.clone(), pd, S, delta, 0.0075, tv=1e-3, beta=5e-3, mode="trilinear",
                     fuse_tv=fuse)
        losses = []
        for i in range(4):
            o, d, tgt = tp.camera_batch(T, 0.691, imgs, R, 120 + i, 2.0)
            losses.append(tr.step_rays(o.to(DEV), d.to(DEV), tgt.to(DEV)).cpu().clone())
        runs[fuse] = (tr.grid.cpu(), torch.stack(losses))
    np.testing.assert_allclose(runs[True][1].numpy(), runs[False][1].numpy(), rtol=1e-5)
    # Adam turns rounding-level gradient differences on cells with ~0 gradient into
    # step-size differences (as in the reference-loop test above)
    diff = (runs[True][0] - runs[False][0]).abs()
    assert float(diff.max()) <= 5 * 0.0075
    assert float((diff > 1e-5).float().mean()) < 0.01
