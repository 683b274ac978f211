"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The reference measures on no public dataset; these generators stand in for its scenes.
All randomness comes from numpy's PCG64 generator (bit-identical on x86-64 and aarch64
for the uniform draws used here); arithmetic is float64, rounded once to float32.
"""
from __future__ import annotations

import numpy as np


def jittered_lattice(n_side: int = 1024, jitter: float = 0.1, seed: int = 0, extent: float = 1.0):
    """Square lattice x = ((i + 1/2) dx, (j + 1/2) dx) + U(-jitter dx, jitter dx)^2, dx = extent/n_side.

    Search + density variant A: n_side = 1024 gives N = 2^20 in [0, 1]^2."""
    dx = extent / n_side
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(n_side, dtype=np.float64), np.arange(n_side, dtype=np.float64), indexing="ij")
    base = np.stack([(i.ravel() + 0.5) * dx, (j.ravel() + 0.5) * dx], 1)
    u = rng.random((base.shape[0], 2))
    return (base + (2.0 * u - 1.0) * jitter * dx).astype(np.float32)


def gaussian_uniform_mix(n: int = 1 << 20, sigma: float = 0.1, center=(0.5, 0.5), seed: int = 0):
    """Half the particles from an isotropic Gaussian blob (rejection-resampled into
    [0,1]^2), half uniform in [0,1]^2 (search + density variant B)."""
    rng = np.random.default_rng(seed)
    ng = n // 2
    out = np.empty((n, 2), np.float64)
    filled = 0
    while filled < ng:
        # Box-Muller from uniform draws (deterministic float64 arithmetic)
        m = (ng - filled) * 2 + 64
        u1 = 1.0 - rng.random(m)
        u2 = rng.random(m)
        r = np.sqrt(-2.0 * np.log(u1))
        z = np.stack([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)], 1) * sigma + np.asarray(center)
        ok = z[np.all((z >= 0.0) & (z <= 1.0), axis=1)]
        take = min(len(ok), ng - filled)
        out[filled:filled + take] = ok[:take]
        filled += take
    out[ng:] = rng.random((n - ng, 2))
    return out.astype(np.float32)


def search_density_case(variant: str = "A", n_side: int = 1024):
    """(positions, support, area, min_coord, max_coord, hash_len) of the search + density
    configuration: h = 3 dx, A = dx^2, domain [0,1]^2, hash table 2^22 entries at N = 2^20."""
    n = n_side * n_side
    dx = 1.0 / n_side
    if variant == "A":
        pos = jittered_lattice(n_side, 0.1, 0)
    elif variant == "B":
        pos = gaussian_uniform_mix(n, 0.1, (0.5, 0.5), 0)
    else:
        raise ValueError(variant)
    h = np.full(n, np.float32(3.0 * dx), np.float32)
    area = np.full(n, np.float32(dx * dx), np.float32)
    hash_len = 1 << 22 if n == 1 << 20 else -1
    return pos, h, area, np.array([0.0, 0.0], np.float32), np.array([1.0, 1.0], np.float32), hash_len
