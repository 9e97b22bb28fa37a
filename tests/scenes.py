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
