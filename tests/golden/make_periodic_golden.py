"""Golden vectors of the reference's periodic boundaries at the search level.

The reference's periodic boundary condition (src/modules/periodicBC.py) appends ghost copies
of the particles within buffer * support of the domain's edges (createGhostParticlesKernel,
:23-103: index lists and position offsets in a fixed category order) and searches the
extended arrays.  Its time integration cannot run with them (the integrator adds arrays of
the real and the extended length, src/simulationBase.py:505-569), so the path is pinned here
at the search level: for seeded particle sets in a periodic box this records the reference's
ghost indices and offsets and the pair list of its own search (constructNeighborhoods,
src/modules/neighborSearch.py:91-115) over the real + ghost particles.
Needs the reference checkout; writes tests/golden/periodic_golden.npz.
Usage:  python tests/golden/make_periodic_golden.py
"""
from __future__ import annotations

import importlib
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import ref_harness  # noqa: E402

CASES = {
    # name: (n, support, periodicX, periodicY, seed)
    "x": (1500, 0.06, True, False, 11),
    "xy": (1500, 0.06, True, True, 12),
    "xy_dense": (4000, 0.03, True, True, 13),
}
BUFFER = 2


def main():
    torch.set_num_threads(4)
    R = ref_harness.load()
    pbc = importlib.import_module("src.modules.periodicBC")
    out, meta = {}, {}
    dmin, dmax = np.array([0.0, 0.0]), np.array([1.0, 1.0])
    for name, (n, h, px, py, seed) in CASES.items():
        rng = np.random.default_rng(seed)
        pos = rng.random((n, 2)).astype(np.float32)
        P = torch.from_numpy(pos)
        filters, offsets = pbc.createGhostParticlesKernel(P, dmin, dmax, BUFFER, h, px, py)
        gi = torch.cat(filters)
        go = torch.vstack(offsets)
        ext = torch.cat((P, P[gi] + go))
        hs = torch.full((ext.shape[0],), np.float32(h), dtype=torch.float32)
        vmin = torch.tensor(dmin - BUFFER * h, dtype=torch.float32)
        vmax = torch.tensor(dmax + BUFFER * h, dtype=torch.float32)
        rows, cols, *_ = R.neighborSearch.constructNeighborhoods(ext, hs, -1, 1.0, vmin, vmax)
        out[f"{name}/pos"] = pos
        out[f"{name}/ghost_indices"] = gi.numpy().astype(np.int64)
        out[f"{name}/ghost_offsets"] = go.numpy().astype(np.float32)
        out[f"{name}/ghost_counts"] = np.array([len(f) for f in filters], np.int64)
        out[f"{name}/rows"] = rows.numpy().astype(np.int32)
        out[f"{name}/cols"] = cols.numpy().astype(np.int32)
        meta[name] = {"n": n, "support": float(np.float32(h)), "periodicX": px, "periodicY": py, "buffer": BUFFER,
                      "domain_min": dmin.tolist(), "domain_max": dmax.tolist()}
        print(name, n, "ghosts", len(gi), "pairs", len(rows), flush=True)
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, "periodic_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()
