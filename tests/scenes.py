"""Seeded synthetic scenes (numpy RNG) standing in for the NeRF-synthetic data the
reference trains on: a dense [s,s,s,4] grid in the box [-1.5, 1.5]^3 with RGB =
sigmoid(N(0,1)) and opacity = ReLU(sum of Gaussian blobs), and look-at pinhole cameras
at radius 4 on the upper hemisphere (NeRF convention: columns x, y, back, position)."""
from __future__ import annotations

import math

import numpy as np

BOX = 1.5


def points_distance(side: int) -> float:
    return 2 * BOX / side


def cell_coords(side: int) -> np.ndarray:
    pd = np.float32(points_distance(side))
    i = np.arange(side, dtype=np.float32) - np.float32(math.ceil(side / 2)) + np.float32(1)
    x = (i * pd).astype(np.float32)
    return np.stack(np.meshgrid(x, x, x, indexing="ij"), -1)


def make_grid(side: int, n_blobs: int, seed: int, amp=(5.0, 20.0), width: float = 0.3,
              negative_frac: float = 0.0) -> np.ndarray:
    """[side]^3 x 4 float32. negative_frac sets that fraction of cells' channels to
    values outside [0,1] (to exercise the clamp)."""
    rng = np.random.default_rng(seed)
    rgb = 1.0 / (1.0 + np.exp(-rng.standard_normal((side, side, side, 3))))
    centres = rng.uniform(-1, 1, (n_blobs, 3))
    amps = rng.uniform(amp[0], amp[1], n_blobs)
    xyz = cell_coords(side).astype(np.float64)
    dens = np.zeros((side, side, side))
    for c, a in zip(centres, amps):
        dens += a * np.exp(-np.sum((xyz - c) ** 2, -1) / (2 * width ** 2))
    grid = np.concatenate([rgb, np.maximum(dens, 0)[..., None]], -1).astype(np.float32)
    if negative_frac > 0:
        m = rng.random(grid.shape) < negative_frac
        grid[m] = rng.uniform(-0.5, 1.5, m.sum()).astype(np.float32)
    return grid


def look_at(pos: np.ndarray) -> np.ndarray:
    back = pos / np.linalg.norm(pos)
    up = np.array([0.0, 0.0, 1.0])
    if abs(back[2]) > 0.999:
        up = np.array([0.0, 1.0, 0.0])
    x = np.cross(up, back)
    x /= np.linalg.norm(x)
    y = np.cross(back, x)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = x, y, back, pos
    return m.astype(np.float32)


def make_cameras(n: int, seed: int, radius: float = 4.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        p = rng.standard_normal(3)
        p[2] = abs(p[2]) + 0.1
        out.append(look_at(radius * p / np.linalg.norm(p)))
    return np.stack(out)


def make_images(n: int, h: int, w: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.random((n, h, w, 4)).astype(np.float32)


def make_grid_fast(side: int, n_blobs: int, seed: int, rgb: str = "sigmoid",
                   amp=(5.0, 20.0), width: float = 0.3):
    """A scene of make_grid's kind for large sides, built with torch on the CPU in
    seconds: [side]^3 x 4 float32 with opacity = ReLU(sum of Gaussian blobs of the given
    width), each blob evaluated as the product of three 1-D exponentials, centres
    U[-1,1]^3 and amplitudes U[amp] from numpy's generator; RGB = sigmoid(N(0,1))
    ("sigmoid") or U[0,1] ("uniform") from a seeded torch generator. Same distribution as
    make_grid, different draws."""
    import torch
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-1, 1, (n_blobs, 3))
    amps = rng.uniform(amp[0], amp[1], n_blobs)
    x = torch.from_numpy(cell_coords_1d(side)).double()
    dens = torch.zeros(side, side, side, dtype=torch.float32)
    for c, a in zip(centres, amps):
        e = [torch.exp(-(x - float(c[k])) ** 2 / (2 * width ** 2)).float() for k in range(3)]
        dens.add_(float(a) * e[0][:, None, None] * e[1][None, :, None] * e[2][None, None, :])
    g = torch.Generator().manual_seed(int(seed))
    out = torch.empty(side, side, side, 4, dtype=torch.float32)
    if rgb == "sigmoid":
        out[..., :3] = torch.sigmoid(torch.randn(side, side, side, 3, generator=g))
    elif rgb == "uniform":
        out[..., :3] = torch.rand(side, side, side, 3, generator=g)
    else:
        raise ValueError(rgb)
    out[..., 3] = dens.clamp_(min=0)
    return out


def cell_coords_1d(side: int) -> np.ndarray:
    """World coordinate of each cell index along one axis (generate_grid's layout)."""
    pd = np.float32(points_distance(side))
    i = np.arange(side, dtype=np.float32) - np.float32(math.ceil(side / 2)) + np.float32(1)
    return (i * pd).astype(np.float32)
