"""ORACLE — test infrastructure, not part of the product.

Host restatement of the library's counter-based uniform (splitmix64 finaliser of Steele,
Lea and Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014):

    mix(z):  z += 0x9e3779b97f4a7c15
             z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9
             z = (z ^ (z >> 27)) * 0x94d049bb133111eb
             z ^ (z >> 31)
    uniform(seed, a, b) = (mix(mix(mix(seed) ^ a) ^ b) >> 40) * 2^-24

All arithmetic is modulo 2^64 (numpy uint64 wraps). The values are exact multiples of
2^-24 in [0, 1), so float32 and float64 see the same numbers.
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0x9E3779B97F4A7C15)
_M2 = np.uint64(0xBF58476D1CE4E5B9)
_M3 = np.uint64(0x94D049BB133111EB)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + _M1
        z = (z ^ (z >> np.uint64(30))) * _M2
        z = (z ^ (z >> np.uint64(27))) * _M3
    return z ^ (z >> np.uint64(31))


def hash_stream(seed: int, a):
    return mix64(mix64(np.uint64(seed & 0xFFFFFFFFFFFFFFFF)) ^ np.asarray(a, dtype=np.uint64))


def hash_to_unit(h, b):
    v = mix64(np.asarray(h, dtype=np.uint64) ^ np.asarray(b, dtype=np.uint64)) >> np.uint64(40)
    return (v.astype(np.float64) * 2.0 ** -24).astype(np.float32)


def uniform(seed: int, a, b):
    return hash_to_unit(hash_stream(seed, a), b)


def stratified_jitter(seed: int, num_rays: int, num_samples: int) -> np.ndarray:
    """[R,S] float32 jitter j(r, s) = uniform(seed, r, s)."""
    h = hash_stream(seed, np.arange(num_rays, dtype=np.uint64))
    s = np.arange(num_samples, dtype=np.uint64)
    return hash_to_unit(h[:, None], s[None, :])


def camera_uniforms(seed: int, num_rays: int):
    """(u, v) pixel uniforms of the in-kernel camera rays: uniform(seed, r, 0 / 1)."""
    h = hash_stream(seed, np.arange(num_rays, dtype=np.uint64))
    return hash_to_unit(h, 0), hash_to_unit(h, 1)
