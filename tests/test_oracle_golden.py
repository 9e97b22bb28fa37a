"""Pins the oracle (oracle/torch_port.py) to outputs of the reference itself: every
fixture in tests/golden was produced by running the reference's own functions
(tests/golden/make_golden.py). CPU only."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import torch_port as tp

PATH_CASES = ["ref_nearest", "ref_trilinear", "ref_trilinear_saturated", "ref_even_spread",
              "ref_edge_nearest", "ref_edge_trilinear"]


def _oracle_step(d):
    grid = torch.from_numpy(d["grid"]).requires_grad_(True)
    T = torch.from_numpy(d["transforms"])
    imgs = torch.from_numpy(d["imgs"])
    C, R, S = T.shape[0], int(d["rays_per_cam"]), int(d["num_samples"])
    if int(d["even_spread"]):
        uv = tp.even_uv(C, int(round(R ** 0.5)))
    else:
        uv = torch.from_numpy(d["uv"])
    dirs, target = tp.camera_rays(T, float(d["camera_angle_x"]), imgs, uv)
    origins = torch.repeat_interleave(T[:, :3, 3], R, 0)
    pts = tp.sample_positions(origins, dirs, S, float(d["delta"]))
    gmin = tp.grid_min(grid.shape, float(d["points_distance"]))
    n = tp.normalize(pts, gmin, float(d["points_distance"]))
    if str(d["mode"]) == "nearest":
        vals, mask, idx = tp.nearest_lookup(n, grid.clip(0, 1))
    else:
        vals, mask, idx = tp.trilinear_lookup(n, grid.clip(0, 1))
    vals = vals * mask.unsqueeze(-1)
    px = tp.composite(vals.reshape(C, R, S, 4)).reshape(C * R, 4)
    loss = torch.nn.functional.mse_loss(px, target)
    loss.backward()
    return dict(dirs=dirs, pixels=target, samples=pts, grid_min=gmin, normalized=n, index=idx,
                mask=mask, vals=vals, rgba=px, loss=loss, grad=grid.grad)


@pytest.mark.parametrize("case", PATH_CASES)
def test_oracle_matches_reference_bit_exact(case):
    d = load_golden(case)
    o = _oracle_step(d)
    for key in ["dirs", "pixels", "samples", "grid_min", "normalized", "index", "mask", "vals"]:
        got = o[key].detach().numpy()
        np.testing.assert_array_equal(got, d[key], err_msg=f"{case}:{key}")
    # same ATen ops in the same order on the same CPU: forward and gradient agree to the
    # last bit or, for reductions whose CPU vector width may differ, to 1e-6 relative
    np.testing.assert_allclose(o["rgba"].detach().numpy(), d["rgba"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(float(o["loss"]), float(d["loss"]), rtol=1e-6)
    g, gr = o["grad"].numpy(), d["grad"]
    assert np.abs(g - gr).max() <= 1e-6 * np.abs(gr).max() + 1e-12


def test_oracle_composite_matches_reference():
    d = load_golden("ref_composite")
    x = torch.from_numpy(d["samples"]).requires_grad_(True)
    out = tp.composite(x)
    out.backward(torch.from_numpy(d["dout"]))
    np.testing.assert_allclose(out.detach().numpy(), d["out"], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(x.grad.numpy(), d["dsamples"], rtol=1e-5, atol=1e-6)


def test_fixtures_cover_edge_cases():
    """The fixtures exercise what the reference's semantics hinge on."""
    e = load_golden("ref_edge_nearest")
    n = e["normalized"]
    assert ((n - np.floor(n)) == 0.5).sum() > 0, "rounding ties at .5"
    assert (~e["mask"]).sum() > 0, "samples outside the box"
    t = load_golden("ref_edge_trilinear")
    n = t["normalized"]
    side = int(t["side"])
    assert ((n > side - 1) & (n < side)).sum() > 0, "upper-face wrap"
    assert (n == np.floor(n)).sum() > 0, "integer coordinates (ceil == floor)"
    assert ((n > -1) & (n < 0)).sum() > 0, "negative fractions (masked)"
    s = load_golden("ref_trilinear_saturated")
    assert (s["grid"][..., 3] > 1).sum() > 0, "alpha saturation after the clip"
    assert ((s["grid"] < 0) | (s["grid"] > 1)).sum() > 0


def test_oracle_collect_cells_matches_reference():
    """src/grid_functions.py:154-170: the wrapped 8-corner gather, its mask on the float
    coordinates and the autograd scatter of its values."""
    d = load_golden("ref_collect_cells")
    grid = torch.from_numpy(d["grid"]).requires_grad_(True)
    vals, mask = tp.collect_cells(torch.from_numpy(d["normalized"]), grid)
    vals.backward(torch.from_numpy(d["dvals"]))
    np.testing.assert_array_equal(vals.detach().numpy(), d["vals"])
    np.testing.assert_array_equal(mask.numpy(), d["mask"])
    np.testing.assert_allclose(grid.grad.numpy(), d["grad"], rtol=1e-6, atol=1e-6)
    n = d["normalized"]
    dims = np.array(d["grid"].shape[:3])
    assert (~d["mask"]).sum() > 0 and d["mask"].sum() > 0
    assert ((n > dims - 1) & (n < dims)).any(), "upper-face wrap"
    assert (n == np.floor(n)).all(axis=1).any(), "integer coordinates"


def test_oracle_remove_noise_matches_reference():
    d = load_golden("ref_remove_noise")
    for i in range(3):
        k, r, t = d[f"params_{i}"]
        got = tp.remove_noise(torch.from_numpy(d["grid"].copy()), int(k), float(r), float(t),
                              repeats=6)
        np.testing.assert_array_equal(got.numpy(), d[f"out_{i}"])
    assert not np.array_equal(d["out_0"], d["grid"]), "the clean-up must clear something"


def _splat_ref(d, c):
    T = torch.from_numpy(d["transforms"][c])
    return tp.splat_preview(torch.from_numpy(d["grid"]), float(d["points_distance"]), T,
                            float(d["camera_angle_x"]), int(d["size_y"]))


def nearest_wins_image(info, colors_of, shape):
    """The preview painted by the rule the GPU kernel implements: at each pixel the point
    nearest to the camera; also returns the pixels where the two nearest points' distances
    tie (where the reference's unstable far-to-near sort may let either win)."""
    img = np.ones(shape)
    best = {}
    ties = set()
    xx, yy, dist = info["xx"].numpy(), info["yy"].numpy(), info["dist"].numpy()
    for i in range(len(xx)):
        p = (int(xx[i]), int(yy[i]))
        if p not in best or dist[i] < dist[best[p]]:
            if p in best and dist[i] == dist[best[p]]:
                ties.add(p)
            best[p] = i
        elif dist[i] == dist[best[p]]:
            ties.add(p)
    for p, i in best.items():
        img[p] = colors_of(i)
    return img, ties


def test_oracle_splat_matches_reference_and_the_nearest_wins_rule():
    """The oracle's preview equals the reference's image bit for bit, and so do the
    per-point projections it returns; painting each pixel with its nearest point (the rule
    the GPU kernel follows) reproduces the reference's far-to-near painter everywhere but at
    exact distance ties."""
    d = load_golden("ref_splat")
    for c in range(d["transforms"].shape[0]):
        img, info = _splat_ref(d, c)
        np.testing.assert_array_equal(img, d[f"img_{c}"])
        grid = torch.from_numpy(d["grid"])
        cells = grid[grid[..., 3] > 0.1]
        ok = ((info["xn"] < 1) & (info["xn"] >= 0) & (info["yn"] < 1) & (info["yn"] >= 0))
        assert bool(ok.all())
        drawn = cells[:, :3].double().numpy()
        # points inside the view, in the order splat_preview keeps them
        inside = np.nonzero(_fov_mask(d, c))[0]
        painted, ties = nearest_wins_image(info, lambda i: drawn[inside[i]], img.shape)
        differ = np.argwhere(np.any(painted != img, axis=-1))
        assert all(tuple(p) in ties for p in differ), "a pixel differs without a distance tie"
        assert (~np.all(img == 1.0, axis=-1)).sum() > 100


def _fov_mask(d, c):
    """Which of the drawn cells (alpha > 0.1, row-major) project inside the view (the
    reference's unfitxy filter, src/visualization.py:198-208), from the oracle's ops."""
    grid = torch.from_numpy(d["grid"])
    T = torch.from_numpy(d["transforms"][c])
    pts = np.argwhere(grid[..., 3] > 0.1)
    half = (torch.tensor(grid.shape[:3]) / 2).unsqueeze(1).ceil()
    pts = ((pts - half) + 1) * float(d["points_distance"])
    ctp = pts.T - T[:3, 3]
    yz, xz = T[:3, 0], T[:3, 1]
    aspect = yz.norm(dim=0) / xz.norm(dim=0)
    nm = ctp.norm(dim=1) * yz.norm()
    ax, ay = torch.matmul(ctp, yz) / nm, torch.matmul(ctp, xz) / nm
    fov = float(d["camera_angle_x"])
    xn = 0.5 + ay / -fov
    yn = 0.5 + ax / (fov / aspect)
    return ((xn < 1.0) & (xn >= 0.0) & (yn < 1.0) & (yn >= 0.0)).numpy()
