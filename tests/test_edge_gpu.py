"""Edge cases of the search path on the GPU: no particles, coincident particles, particles
exactly on cell boundaries and at the domain's corners, against the oracle (pair sets bit
for bit, densities within 1e-5 of the maximum)."""
import numpy as np
import pytest
import torch

import nsearch as ns

pytestmark = pytest.mark.gpu


def run(pos, h, vmin=None, vmax=None):
    from pytorchsph_gb300.search import GridSearch
    dev = torch.device("cuda")
    n = len(pos)
    area = np.full(n, 1e-4, np.float32)
    res = GridSearch(dev).run(torch.from_numpy(pos).to(dev), torch.from_numpy(h).to(dev),
                              torch.from_numpy(area).to(dev), kernel_support=float(h[0]) if n else 1.0,
                              min_coord=vmin, max_coord=vmax)
    return res, area


def keys(rows, cols):
    return np.sort(rows.astype(np.int64) * (1 << 32) + cols.astype(np.int64))


def test_no_particles(cuda):
    pos = np.zeros((0, 2), np.float32)
    h = np.zeros(0, np.float32)
    res, _ = run(pos, h, np.zeros(2, np.float32), np.ones(2, np.float32))
    assert res.num_pairs == 0
    pairs, _, _ = res.to_coo(distances=False)
    assert pairs.shape == (2, 0)


@pytest.mark.parametrize("layout", ["coincident", "cell_boundaries", "corners"])
def test_degenerate_layouts_match_oracle(cuda, layout):
    h = np.float32(0.1)
    if layout == "coincident":
        # clusters of particles at one position (distance 0 between different particles)
        base = np.array([[0.5, 0.5], [0.55, 0.5], [0.2, 0.8]], np.float32)
        pos = np.repeat(base, [5, 3, 1], axis=0)
    elif layout == "cell_boundaries":
        # particles exactly on multiples of the support (cell faces of a grid of cells h)
        k = np.arange(0, 11, dtype=np.float32) * h
        gx, gy = np.meshgrid(k, k, indexing="ij")
        pos = np.stack([gx.ravel(), gy.ravel()], 1).astype(np.float32)
    else:
        pos = np.array([[0, 0], [1, 0], [0, 1], [1, 1], [0.5, 0.5], [np.float32(0.1), 0], [0, np.float32(0.1)]],
                       np.float32)
    n = len(pos)
    hs = np.full(n, h, np.float32)
    vmin, vmax = np.zeros(2, np.float32), np.ones(2, np.float32)
    res, area = run(pos, hs, vmin, vmax)
    _, off, cols = ns.search(pos, hs, vmin, vmax)
    pairs, _, _ = res.to_coo(distances=False)
    p = pairs.cpu().numpy()
    rows = np.repeat(np.arange(n), np.diff(off))
    assert np.array_equal(keys(p[0], p[1]), keys(rows, cols))
    rho = res.density().cpu().numpy()
    ref = ns.density(off, cols, pos, area, float(h), use_double=True)
    assert np.abs(rho - ref).max() <= 1e-5 * np.abs(ref).max()


def test_no_particles_density(cuda):
    pos = np.zeros((0, 2), np.float32)
    res, _ = run(pos, np.zeros(0, np.float32), np.zeros(2, np.float32), np.ones(2, np.float32))
    assert res.density().numel() == 0
