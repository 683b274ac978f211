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


def tank_walls(width: float, height: float, dx: float, layers: int = 3):
    """Ghost-particle walls of a rectangular tank [0, width] x [0, height].

    Layer k lies at distance (k + 1/2) dx outside the tank walls (the offsets
    (2k+1) * packing/2 of src/modules/solidBoundary.py:142-146), sampled every dx along the
    offset rectangle.  Each wall particle's ghost is its mirror image inside the tank (the
    `mirrored` samples of src/ghostParticles.py:132-135), reflected through the corner at
    corners.  Returns (wall_positions, ghost_positions), float32 [Nb, 2]."""
    pts = []
    for k in range(layers):
        d = (k + 0.5) * dx
        x0, x1, y0, y1 = -d, width + d, -d, height + d
        nxs = int(round((x1 - x0) / dx)) + 1
        nys = int(round((y1 - y0) / dx)) + 1
        xs = x0 + np.arange(nxs) * dx
        ys = y0 + np.arange(nys) * dx
        pts.append(np.stack([xs, np.full(nxs, y0)], 1))
        pts.append(np.stack([xs, np.full(nxs, y1)], 1))
        pts.append(np.stack([np.full(nys - 2, x0), ys[1:-1]], 1))
        pts.append(np.stack([np.full(nys - 2, x1), ys[1:-1]], 1))
    w = np.concatenate(pts)
    g = w.copy()
    g[:, 0] = np.where(w[:, 0] < 0, -w[:, 0], np.where(w[:, 0] > width, 2 * width - w[:, 0], w[:, 0]))
    g[:, 1] = np.where(w[:, 1] < 0, -w[:, 1], np.where(w[:, 1] > height, 2 * height - w[:, 1], w[:, 1]))
    return w.astype(np.float32), g.astype(np.float32)


def dam_break(nx: int = 64, ny: int = 128, dx: float = 0.01, tank=(4.0, 2.0), layers: int = 3):
    """Dam-break scene: an nx x ny lattice fluid block (spacing dx) at the lower-left corner
    of the tank, at rest, relative density 1, with ghost-particle walls.  Support h = 3 dx and
    particle area A = dx^2 (particle radius dx / sqrt(pi)).  The search domain is the tank
    widened by 2 h on every side (virtualMin/Max with buffer 2, src/simulationBase.py:968-969)."""
    i, j = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64), indexing="ij")
    pos = np.stack([(i.ravel() + 0.5) * dx, (j.ravel() + 0.5) * dx], 1).astype(np.float32)
    n = len(pos)
    h = np.float32(3 * dx)
    wall, ghost = tank_walls(tank[0], tank[1], dx, layers)
    return {
        "pos": pos, "vel": np.zeros((n, 2), np.float32), "rho": np.ones(n, np.float32),
        "area": np.full(n, np.float32(dx * dx), np.float32), "support": np.full(n, h, np.float32),
        "wall_pos": wall, "ghost_pos": ghost, "wall_area": np.full(len(wall), np.float32(dx * dx), np.float32),
        "h": float(h), "dx": float(dx), "tank": (float(tank[0]), float(tank[1])),
        "vmin": np.array([-2 * h, -2 * h], np.float32),
        "vmax": np.array([tank[0] + 2 * h, tank[1] + 2 * h], np.float32),
        "column_height": float(ny * dx),
    }


def oscillating_drop(n_target: int = 16384, radius: float = 0.5, amplitude: float = 1.0):
    """Oscillating drop: lattice particles inside a circle of `radius` centred at the origin,
    initial velocity v = A (x, -y) (the velocity idea of the reference notebook), no walls.
    The spacing dx is chosen so that about n_target particles fall inside the circle."""
    dx = float(np.sqrt(np.pi * radius * radius / n_target))
    m = int(np.ceil(radius / dx)) + 1
    k = np.arange(-m, m + 1, dtype=np.float64)
    gx, gy = np.meshgrid(k * dx, k * dx, indexing="ij")
    p = np.stack([gx.ravel(), gy.ravel()], 1)
    p = p[np.linalg.norm(p, axis=1) <= radius - 0.5 * dx]
    pos = p.astype(np.float32)
    n = len(pos)
    vel = (amplitude * np.stack([pos[:, 0], -pos[:, 1]], 1)).astype(np.float32)
    h = np.float32(3 * dx)
    ext = radius * 3
    return {
        "pos": pos, "vel": vel, "rho": np.ones(n, np.float32), "area": np.full(n, np.float32(dx * dx), np.float32),
        "support": np.full(n, h, np.float32), "wall_pos": np.zeros((0, 2), np.float32),
        "ghost_pos": np.zeros((0, 2), np.float32), "wall_area": np.zeros(0, np.float32), "h": float(h), "dx": dx,
        "vmin": np.array([-ext, -ext], np.float32), "vmax": np.array([ext, ext], np.float32),
    }


def dam_break_scene(n_target: int, aspect: float, tank=(4.0, 2.0)):
    """Dam break with about n_target fluid particles in a block of width/height `aspect`
    whose area is a quarter of the tank's (dx = sqrt(area / n)), with 3-layer walls."""
    W, H = tank
    area = 0.25 * W * H
    dx = float(np.sqrt(area / n_target))
    nx = max(2, int(round(np.sqrt(n_target * aspect))))
    ny = max(2, int(round(n_target / nx)))
    while ny * dx > H - dx:
        ny -= 1
    return dam_break(nx, ny, dx, tank)


def serving_trace(n_requests: int = 1024, rate: float = 50.0, n_min: int = 2048, n_max: int = 131072,
                  steps: int = 1000, seed: int = 0):
    """The serving workload: Poisson arrivals (mean `rate` per second), sizes log-uniform in
    [n_min, n_max], half dam breaks with block width/height ~ U[0.5, 2], half oscillating
    drops (radius 0.5, v = A (x, -y), A ~ U[0.5, 2]).  Everything derives from one master
    seed through numpy SeedSequence.  Returns a list of dicts with the arrival time and the
    scene parameters; `make_request_scene` builds the arrays when a request is admitted."""
    ss = np.random.SeedSequence(seed)
    rng = np.random.default_rng(ss)
    gaps = rng.exponential(1.0 / rate, n_requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    sizes = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_requests)).astype(np.int64)
    kinds = rng.integers(0, 2, n_requests)
    shape = rng.uniform(0.5, 2.0, n_requests)
    out = []
    for k in range(n_requests):
        out.append({"rid": k, "arrival": float(arrivals[k]), "n": int(sizes[k]),
                    "kind": "dam_break" if kinds[k] == 0 else "drop", "shape": float(shape[k]), "steps": steps})
    return out


# Time step of the serving requests, dt = SERVING_CFL h / c0.  With semi-implicit Euler the
# restated reference step stays bounded over 1000 steps at 0.1 for both scene kinds (dam
# breaks and drops; relative density within 0.5 %), while at 0.25 drops diverge after a few
# hundred steps and tall dam breaks after about 500; the MOG density diffusion diverges on the
# drops' free surface even at small steps, so requests use the renormalized deltaSPH scheme.
SERVING_CFL = 0.1


def make_request_scene(req):
    """(scene arrays, deltaSPH parameters) of one serving request."""
    if req["kind"] == "dam_break":
        sc = dam_break_scene(req["n"], req["shape"])
        c0 = float(10.0 * np.sqrt(2 * 9.81 * sc["column_height"]))
        params = {"c0": c0, "gravity": (0.0, -9.81), "point_source": False}
    else:
        sc = oscillating_drop(req["n"], 0.5, req["shape"])
        c0 = 10.0
        params = {"c0": c0, "gravity": (0.0, 0.0), "point_source": True}
    params.update(dt=SERVING_CFL * sc["h"] / c0, diffusion="deltaSPH")
    return sc, params
