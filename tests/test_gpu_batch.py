"""Batched form (many scenes, one persistent launch) against the oracle, scene by scene.

Semantics checked: unoccupied cells are zero and are not parameters, so the gradient is
compared on occupied cells only; empty-space skipping must be exact (same results with
and without the brick mask); early termination at T < 1e-4 may only drop contributions
smaller than the threshold; a captured CUDA graph replays on new rays with the eager
results; every autotuner tile gives the same step."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes
from oracle import torch_port as tp
from plenoxels_gb300.batch import BatchedTrainStep, Scene

pytestmark = pytest.mark.gpu
DEV = "cuda"

SPECS = [  # side, rays, samples
    (16, 120, 64), (24, 300, 96), (32, 200, 128), (20, 80, 200), (32, 260, 72)]


def _make(dtype, seed=0, frac=0.10):
    out = []
    for i, (side, rays, S) in enumerate(SPECS):
        g = torch.from_numpy(scenes.make_grid(side, 3, 100 + i + seed, amp=(0.5, 4)))
        dens = g[..., 3]
        thr = torch.quantile(dens.flatten(), 1 - frac)
        occ = dens > thr
        g[~occ] = 0.0
        cells = g.to(dtype)
        T = torch.from_numpy(scenes.make_cameras(3, 200 + i + seed))
        imgs = torch.from_numpy(scenes.make_images(3, 8, 8, 300 + i + seed))
        o, d, tgt = tp.camera_batch(T, 0.691, imgs, rays, 400 + i + seed, 2.0)
        out.append(dict(cells=cells, occ=occ, o=o, d=d, tgt=tgt, S=S, side=side,
                        pd=scenes.points_distance(side), delta=4.0 / S))
    return out


def _batch(problem, **kw):
    sc = [Scene(p["cells"].to(DEV), p["occ"].to(DEV), p["pd"], p["S"], p["delta"]) for p in problem]
    R = sum(p["o"].shape[0] for p in problem)
    step = BatchedTrainStep(sc, R, **kw)
    o = torch.cat([p["o"] for p in problem]).to(DEV)
    d = torch.cat([p["d"] for p in problem]).to(DEV)
    t = torch.cat([p["tgt"] for p in problem]).to(DEV)
    rs = torch.cat([torch.full((p["o"].shape[0],), i, dtype=torch.int32) for i, p in enumerate(problem)]).to(DEV)
    step.set_rays(o, d, t, rs)
    step.rgba = torch.empty(R, 4, device=DEV)
    return step, R


def _oracle(problem, R_total):
    rgba, grads, loss = [], [], 0.0
    for p in problem:
        g = p["cells"].float().clone().requires_grad_(True)
        gmin = tp.grid_min(g.shape, p["pd"])
        px = tp.render(g, p["o"], p["d"], p["S"], p["delta"], gmin, p["pd"])
        sq = ((px - p["tgt"]) ** 2).sum()
        (sq / (4 * R_total)).backward()
        rgba.append(px.detach())
        grads.append(g.grad * p["occ"].unsqueeze(-1))
        loss += float(sq) / (4 * R_total)
    return torch.cat(rgba), grads, loss


def _grad_err(step, grads):
    worst = 0.0
    for sc, ref in zip(step.scenes, grads):
        got = sc.grad.cpu()
        # nothing outside the occupancy, the masked oracle inside it
        assert float((got * (~sc.occupancy.cpu()).unsqueeze(-1)).abs().max()) == 0.0
        worst = max(worst, float((got - ref).abs().max()) / max(float(ref.abs().max()), 1e-30))
    return worst


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_batched_step_matches_oracle_without_termination(dtype):
    problem = _make(dtype)
    step, R = _batch(problem, term_threshold=0.0)
    for sc in step.scenes:  # stale values outside the occupancy must stay untouched (zero)
        sc.grad.fill_(0.0)
    step.step()  # a first step leaves gradient at occupied cells; the next must clear them
    loss = float(step.step())
    torch.cuda.synchronize()
    rgba_ref, grads, loss_ref = _oracle(problem, R)
    np.testing.assert_allclose(step.rgba.cpu().numpy(), rgba_ref.numpy(), rtol=1e-5, atol=2e-6)
    np.testing.assert_allclose(loss, loss_ref, rtol=1e-5)
    assert _grad_err(step, grads) < 1e-4


def test_skipping_is_exact_and_termination_is_bounded():
    problem = _make(torch.float32, seed=7)
    a, R = _batch(problem, term_threshold=0.0)
    a.step()
    ga = [sc.grad.clone() for sc in a.scenes]
    ra = a.rgba.clone()
    # same batch without the brick masks: no skipping
    b, _ = _batch(problem, term_threshold=0.0)
    for sc in b.scenes:
        sc.bricks.zero_()
        sc.bricks.fill_(-1)  # every brick marked occupied
    b.step()
    torch.cuda.synchronize()
    np.testing.assert_allclose(ra.cpu().numpy(), b.rgba.cpu().numpy(), rtol=1e-6, atol=1e-7)
    for x, y, sc in zip(ga, [s.grad for s in b.scenes], a.scenes):
        m = sc.occupancy.unsqueeze(-1)
        assert float(((x - y) * m).abs().max()) <= 1e-6 * float((y * m).abs().max()) + 1e-12
    # every brick size skips exactly (down to single cells)
    for L in (0, 1, 2, 4):
        e, _ = _batch(problem, term_threshold=0.0)
        e._set_bricks(L)
        e.step()
        torch.cuda.synchronize()
        np.testing.assert_allclose(ra.cpu().numpy(), e.rgba.cpu().numpy(), rtol=1e-6, atol=1e-7)
        for x, sc in zip(ga, e.scenes):
            m = sc.occupancy.unsqueeze(-1)
            assert float(((x - sc.grad) * m).abs().max()) <= 1e-6 * float((x * m).abs().max()) + 1e-12
    # early termination: only contributions behind T < 1e-4 may change
    c, _ = _batch(problem, term_threshold=1e-4)
    c.step()
    torch.cuda.synchronize()
    assert float((c.rgba - ra).abs().max()) <= 1e-4


def test_graph_replay_on_new_rays_and_autotune():
    problem = _make(torch.bfloat16, seed=3)
    step, R = _batch(problem, term_threshold=1e-4)
    times = step.autotune(reps=2, brick_sizes=(1, 2, 3))
    assert step.tiles in times and len(times) >= 3 and step.brick_log2 in (1, 2, 3)
    eager = float(step.step())
    torch.cuda.synchronize()
    g_eager = [sc.grad.clone() for sc in step.scenes]
    step.capture()
    assert float(step.step()) == eager
    torch.cuda.synchronize()
    for x, sc in zip(g_eager, step.scenes):
        assert float((x - sc.grad).abs().max()) <= 1e-6 * float(x.abs().max()) + 1e-12
    # new rays through the same graph
    other = _make(torch.bfloat16, seed=3)
    perm = torch.randperm(R)
    o = torch.cat([p["o"] for p in other])[perm].to(DEV)
    d = torch.cat([p["d"] for p in other])[perm].to(DEV)
    t = torch.cat([p["tgt"] for p in other])[perm].to(DEV)
    rs = torch.cat([torch.full((p["o"].shape[0],), i, dtype=torch.int32)
                    for i, p in enumerate(other)])[perm].to(DEV)
    step.set_rays(o, d, t, rs)
    replay = float(step.step())
    torch.cuda.synchronize()
    np.testing.assert_allclose(replay, eager, rtol=1e-5)  # same rays, new order


def test_invalid_scene_index_contributes_nothing():
    problem = _make(torch.float32, seed=5)
    step, R = _batch(problem, term_threshold=0.0)
    step.ray_scene[:10] = 99  # not a scene of the batch
    step.step()
    torch.cuda.synchronize()
    assert float(step.rgba[:10].abs().sum()) == 0.0


@pytest.mark.parametrize("tiles", [(1, 256), (4, 128), (1, 256, 1), (2, 256, 1)])
def test_every_tile_gives_the_oracle_step(tiles):
    """A 32-sample chunk per ray (K = 1) and a 128-sample one (K = 4) on the same batch,
    and the tiles whose scatter merges a warp's updates of the same cell."""
    problem = _make(torch.float32, seed=11)
    step, R = _batch(problem, term_threshold=0.0, tiles=tiles)
    loss = float(step.step())
    torch.cuda.synchronize()
    rgba_ref, grads, loss_ref = _oracle(problem, R)
    np.testing.assert_allclose(step.rgba.cpu().numpy(), rgba_ref.numpy(), rtol=1e-5, atol=2e-6)
    np.testing.assert_allclose(loss, loss_ref, rtol=1e-5)
    assert _grad_err(step, grads) < 1e-4


def test_long_rays_take_a_tile_that_covers_them():
    """2500 samples per ray need 32 * 32 * K >= 2500: the default tile is K = 4, a K = 2 tile
    is refused on the host, and the autotuner only tries tiles that fit."""
    side, rays, S = 12, 40, 2500
    g = torch.from_numpy(scenes.make_grid(side, 2, 77, amp=(0.05, 0.3)))
    occ = g[..., 3] > torch.quantile(g[..., 3].flatten(), 0.7)
    g[~occ] = 0.0
    T = torch.from_numpy(scenes.make_cameras(2, 78))
    imgs = torch.from_numpy(scenes.make_images(2, 8, 8, 79))
    o, d, tgt = tp.camera_batch(T, 0.691, imgs, rays, 80, 2.0)
    problem = [dict(cells=g, occ=occ, o=o, d=d, tgt=tgt, S=S, side=side,
                    pd=scenes.points_distance(side), delta=4.0 / S)]
    with pytest.raises(ValueError):
        _batch(problem, term_threshold=0.0, tiles=(2, 256))
    step, R = _batch(problem, term_threshold=0.0)
    assert step.tiles[0] == 4
    times = step.autotune(reps=1)
    assert all(32 * 32 * k >= S for k, *_ in times)
    loss = float(step.step())
    torch.cuda.synchronize()
    rgba_ref, grads, loss_ref = _oracle(problem, R)
    np.testing.assert_allclose(step.rgba.cpu().numpy(), rgba_ref.numpy(), rtol=1e-5, atol=2e-6)
    np.testing.assert_allclose(loss, loss_ref, rtol=1e-5)
    assert _grad_err(step, grads) < 1e-4


def test_loss_over_many_rays_is_the_mean_squared_error_of_their_rgba():
    """5760 rays: the ordered loss sum spans several blocks of its kernel; the step's loss
    equals the mean over rays and channels of (rgba - target)^2 from its own outputs."""
    problem = _make(torch.float32, seed=7)
    for p in problem:
        p["o"], p["d"], p["tgt"] = p["o"].repeat(6, 1), p["d"].repeat(6, 1), p["tgt"].repeat(6, 1)
    step, R = _batch(problem, term_threshold=0.0)
    assert R > 4 * 1024
    loss = float(step.step())
    torch.cuda.synchronize()
    tgt = torch.cat([p["tgt"] for p in problem]).to(DEV).double()
    ref = float(((step.rgba.double() - tgt) ** 2).mean())
    np.testing.assert_allclose(loss, ref, rtol=1e-6)
