"""Point-splat preview (src/visualization.py:157-232) and stray-voxel clean-up
(src/grid_functions.py:260-280) against the oracle's restatement of the reference.

The clean-up must agree exactly (random opacities put no neighbour sum on the threshold).
The splat's pixel positions may differ where a projected coordinate lies within the
reference's BLAS dot-product rounding of a pixel boundary, so the image must agree on
all but a small fraction of pixels, and every differing pixel must be explained by a
point whose projection sits at such a boundary or by a distance tie."""
import numpy as np
import pytest
import torch

import plenoxels_gb300 as pg
import scenes
from conftest import load_golden
from oracle import torch_port as tp
from plenoxels_gb300.visualization import visulize_3d_in_2d_fast

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel_size,radius,threshold", [(3, 1.0, 2.0), (5, 1.5, 3.0), (3, 2.0, 4.5)])
def test_remove_noise_matches_reference(kernel_size, radius, threshold):
    torch.manual_seed(0)
    g = torch.rand(20, 18, 22, 4)
    g[..., 3] = torch.where(torch.rand(20, 18, 22) < 0.4, torch.rand(20, 18, 22), torch.zeros(20, 18, 22))
    ref = tp.remove_noise(g.clone(), kernel_size, radius, threshold, repeats=6)
    got = pg.grid_functions.convolve_grid_to_remove_noise(g.clone().cuda(), kernel_size, radius,
                                                          threshold, repeats=6).cpu()
    assert torch.equal(got, ref)


def test_splat_preview_matches_reference():
    side = 48
    grid = torch.from_numpy(scenes.make_grid(side, 4, 11, amp=(0.05, 0.6)))
    T = torch.from_numpy(scenes.make_cameras(1, 12))[0]
    ref, _ = tp.splat_preview(grid, scenes.points_distance(side), T, 0.691, 64)
    got = visulize_3d_in_2d_fast(grid, scenes.points_distance(side), T, 0.691, 64)
    assert got.shape == ref.shape and got.dtype == np.float64
    differ = np.any(got != ref, axis=-1)
    assert (~np.all(ref == 1.0, axis=-1)).sum() > 100, "the scene must cover part of the image"
    assert differ.mean() < 0.01, f"{differ.sum()} of {differ.size} pixels differ"


def test_remove_noise_matches_reference_fixture():
    """Bit for bit against convolve_grid_to_remove_noise run by the reference itself."""
    d = load_golden("ref_remove_noise")
    for i in range(3):
        k, r, t = d[f"params_{i}"]
        got = pg.grid_functions.convolve_grid_to_remove_noise(
            torch.from_numpy(d["grid"].copy()).cuda(), int(k), float(r), float(t), repeats=6)
        np.testing.assert_array_equal(got.cpu().numpy(), d[f"out_{i}"])


def _sensitive_pixels(info, xs, ys, tol_px=1e-3, tol_rel=1e-6):
    """Pixels whose colour may legitimately differ from the reference's: those a point can
    reach when its unrounded pixel coordinate lies within tol_px of a rounding boundary
    (x.5) or its normalised coordinate within tol_px / size of the view's edge (the
    reference's BLAS dot products round differently from op-by-op arithmetic), and those
    where the two nearest points' distances agree to tol_rel (the far-to-near sort of the
    reference and the nearest-wins rule may pick either)."""
    out = set()
    fx, fy = info["fx"].numpy(), info["fy"].numpy()
    xn, yn = info["xn"].numpy(), info["yn"].numpy()
    dist = info["dist"].numpy().astype(np.float64)

    def cands(f, n, size):
        c = {int(np.clip(np.round(f), 0, size - 1))}
        if abs(f - np.floor(f) - 0.5) < tol_px:
            c |= {int(np.clip(np.floor(f), 0, size - 1)), int(np.clip(np.floor(f) + 1, 0, size - 1))}
        return c, min(abs(n), abs(1 - n)) < tol_px / size

    by_pixel = {}
    for i in range(len(fx)):
        cx, ex = cands(fx[i], xn[i], xs)
        cy, ey = cands(fy[i], yn[i], ys)
        if len(cx) > 1 or len(cy) > 1 or ex or ey:
            out |= {(a, b) for a in cx for b in cy}
        p = (int(info["xx"][i]), int(info["yy"][i]))
        by_pixel.setdefault(p, []).append(dist[i])
    for p, ds in by_pixel.items():
        if len(ds) > 1:
            a, b = sorted(ds)[:2]
            if b - a <= tol_rel * b:
                out.add(p)
    return out


def test_splat_preview_matches_reference_fixture():
    """visulize_3d_in_2d_fast against the reference's own images: every pixel agrees
    except where _sensitive_pixels says the reference's rounding or an exact distance tie
    decides it, and those are under 1 % of the image."""
    d = load_golden("ref_splat")
    for c in range(d["transforms"].shape[0]):
        T = torch.from_numpy(d["transforms"][c])
        ref = d[f"img_{c}"]
        got = visulize_3d_in_2d_fast(torch.from_numpy(d["grid"]), float(d["points_distance"]), T,
                                     float(d["camera_angle_x"]), int(d["size_y"]))
        assert got.shape == ref.shape
        _, info = tp.splat_preview(torch.from_numpy(d["grid"]), float(d["points_distance"]), T,
                                   float(d["camera_angle_x"]), int(d["size_y"]))
        allowed = _sensitive_pixels(info, ref.shape[0], ref.shape[1])
        differ = [tuple(p) for p in np.argwhere(np.any(got != ref, axis=-1))]
        assert all(p in allowed for p in differ), \
            f"pixels differ without a rounding boundary or tie: {[p for p in differ if p not in allowed][:5]}"
        assert len(differ) < 0.01 * ref.shape[0] * ref.shape[1]
