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
