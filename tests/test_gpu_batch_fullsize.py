"""The batched configuration at its full size: 64 scenes with sides drawn from
{32, 64, 128, 256}, 5 % occupied cells, BF16 cells, rays per scene log-uniform in
[1k, 64k] (about 0.9 M rays), 512 samples per ray, one persistent launch. Early
termination is off here so the step is comparable sample for sample: the RGBA of every
ray of three scenes (the smallest side, a middle one, the largest) and those scenes'
occupancy-masked gradients are checked against the oracle."""
import math

import numpy as np
import pytest
import torch

import scenes
from oracle import torch_port as tp
from plenoxels_gb300 import generate_rays_batched
from plenoxels_gb300.batch import BatchedTrainStep, Scene

pytestmark = pytest.mark.gpu
DEV = "cuda"
S = 512


def _scene(rng, g, i):
    side = int(rng.choice([32, 64, 128, 256]))
    pd = 3.0 / side
    ax = (torch.arange(side, device=DEV, dtype=torch.float32) - math.ceil(side / 2) + 1) * pd
    dens = torch.zeros(side, side, side, device=DEV)
    for _ in range(8):
        c = torch.rand(3, generator=g, device=DEV) * 2 - 1
        a = 5 + 15 * torch.rand((), generator=g, device=DEV)
        d2 = ((ax - c[0]) ** 2)[:, None, None] + ((ax - c[1]) ** 2)[None, :, None] + \
            ((ax - c[2]) ** 2)[None, None, :]
        dens += a * torch.exp(-d2 / (2 * 0.3 ** 2))
    sub = dens.flatten()[torch.randint(0, dens.numel(), (1 << 20,), generator=g, device=DEV)]
    occ = dens > torch.quantile(sub, 0.95)
    cells = torch.cat([torch.rand(side, side, side, 3, generator=g, device=DEV), dens.unsqueeze(-1)], -1)
    cells[~occ] = 0.0
    n = int(round(math.exp(rng.uniform(math.log(1000), math.log(64000)))))
    per_cam = -(-n // 4)
    T = torch.from_numpy(scenes.make_cameras(4, 7000 + i)).to(DEV)
    imgs = torch.rand(4, 32, 32, 4, generator=g, device=DEV)
    dd, px = generate_rays_batched(imgs, per_cam, T, 0.691, device=DEV)
    oo = torch.repeat_interleave(T[:, :3, 3], per_cam, 0) + 2.0 * dd
    return dict(cells=cells.to(torch.bfloat16).contiguous(), occ=occ, pd=pd, side=side,
                o=oo[:n].contiguous(), d=dd[:n].contiguous(), tgt=px[:n].contiguous())


def test_full_size_batch_matches_oracle_on_three_scenes():
    rng = np.random.default_rng(21)
    g = torch.Generator(device=DEV).manual_seed(21)
    probs = [_scene(rng, g, i) for i in range(64)]
    scs = [Scene(p["cells"], p["occ"], p["pd"], S, 4.0 / S) for p in probs]
    R = sum(p["o"].shape[0] for p in probs)
    assert 200_000 < R < 3_000_000
    step = BatchedTrainStep(scs, R, term_threshold=0.0)
    owners = torch.cat([torch.full((p["o"].shape[0],), i, dtype=torch.int32, device=DEV)
                        for i, p in enumerate(probs)])
    step.set_rays(torch.cat([p["o"] for p in probs]), torch.cat([p["d"] for p in probs]),
                  torch.cat([p["tgt"] for p in probs]), owners)
    step.rgba = torch.empty(R, 4, device=DEV)
    step.autotune(reps=1, brick_sizes=(0, 2))
    step.step()
    torch.cuda.synchronize()
    starts = np.cumsum([0] + [p["o"].shape[0] for p in probs])
    sides = [p["side"] for p in probs]
    # the smallest side, a middle one and the largest, each the one with the fewest rays
    picks = []
    for want in sorted(set(sides))[::max(1, len(set(sides)) // 3)][:2] + [max(sides)]:
        cand = [i for i in range(64) if sides[i] == want and i not in picks]
        picks.append(min(cand, key=lambda i: probs[i]["o"].shape[0]))
    for i in picks:
        p = probs[i]
        cells = p["cells"].float().cpu().clone().requires_grad_(True)
        gmin = tp.grid_min(cells.shape, p["pd"])
        px = tp.render(cells, p["o"].cpu(), p["d"].cpu(), S, 4.0 / S, gmin, p["pd"])
        (((px - p["tgt"].cpu()) ** 2).sum() / (4 * R)).backward()
        got = step.rgba[starts[i]:starts[i + 1]].cpu()
        np.testing.assert_allclose(got.numpy(), px.detach().numpy(), rtol=1e-5, atol=2e-6)
        ref = cells.grad * p["occ"].cpu().unsqueeze(-1)
        err = float((scs[i].grad.cpu() - ref).abs().max())
        assert err <= 1e-4 * float(ref.abs().max()) + 1e-12, (i, p["side"], err)
