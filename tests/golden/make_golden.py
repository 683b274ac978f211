"""Generate the golden neighbor-search / density fixtures from the reference itself.

Runs only where the reference checkout exists (it imports the reference's own Python
modules through oracle/ref_harness.py and its compiled CPU neighbor search through
oracle/build_ref.py).  Output: tests/golden/nsearch_golden.npz.

Each case stores its inputs and what the reference returns for them:
  * sortPositions / constructHashMap outputs (src/modules/neighborSearch.py:30-88);
  * the pair list of neighborSearchModule.search on CPU (src/modules/neighborSearch.py:203-229,
    buildNeighborList in cppSrc/neighSearch.cpp:172-259), canonicalised to (i, j) order;
  * computeDensity (src/modules/density.py:26-30) on those pairs, in float32 and float64;
  * for query / asymmetric cases, buildNeighborListUnsortedPerParticle /
    buildNeighborListAsymmetric pairs.
Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import ref_harness  # noqa: E402

from pytorchsph_gb300 import workloads  # noqa: E402


def canon(rows, cols):
    key = rows.astype(np.int64) * (1 << 32) + cols.astype(np.int64)
    key = np.sort(key)
    return (key >> 32).astype(np.int32), (key & 0xFFFFFFFF).astype(np.int32)


def to_csr(rows, cols, n):
    rows, cols = canon(rows, cols)
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, rows.astype(np.int64) + 1, 1)
    return np.cumsum(off).astype(np.int32), cols


def ref_search(R, pos, h, support, vmin, vmax, keep_state=None):
    mod = R.neighborSearch.neighborSearchModule()
    cfg = {"particle": {"support": support}, "compute": {"maxNeighbors": 256, "precision": torch.float32,
                                                          "device": "cpu"},
           "neighborSearch": {"gradientThreshold": 1e-7, "supportScale": 1.0, "sortNeighborhoods": True},
           "domain": {"virtualMin": vmin, "virtualMax": vmax}}
    mod.initialize(cfg, {})
    state = {"fluidPosition": torch.from_numpy(pos), "fluidSupport": torch.from_numpy(h)}
    if vmin is not None:
        nb, dist, radial = mod.search(state, None)
    else:  # no domain: the module-level function with minCoord = maxCoord = None, then the
        # distance lines of neighborSearchModule.search (src/modules/neighborSearch.py:216-223)
        P = torch.from_numpy(pos)
        row, col, *_ = R.neighborSearch.constructNeighborhoods(P, torch.from_numpy(h), -1)
        nb = torch.stack([row, col], 0)
        dist = P[nb[0]] - P[nb[1]]
        radial = torch.linalg.norm(dist, axis=1)
        radial /= support
    mod._state = state
    return mod, nb.numpy(), dist, radial


def sort_info(R, pos, h, vmin, vmax, hash_len):
    P, H = torch.from_numpy(pos), torch.from_numpy(h)
    sp, ss, sli, si, cc, qmin, hmax = R.neighborSearch.sortPositions(
        P, H, 1.0, torch.tensor(vmin, dtype=torch.float32) if vmin is not None else None,
        torch.tensor(vmax, dtype=torch.float32) if vmax is not None else None)
    L = hash_len
    table, ci, cum, span = R.neighborSearch.constructHashMap(sp, ss, sli, si, L, cc)
    return dict(cells_x=np.int32(cc), qmin=qmin.numpy().astype(np.float32), hmax=np.float32(hmax),
                sorted_lin=sli.numpy().astype(np.int32), table=table.numpy(), cell_indices=ci.numpy(),
                cum_cell=cum.numpy(), cell_span=span.numpy(), sort=si.numpy().astype(np.int32),
                sorted_pos=sp.numpy(), sorted_h=ss.numpy())


def add_case(R, out, name, pos, h, area, support, vmin, vmax, hash_len=-1):
    from nsearch import next_prime
    n = pos.shape[0]
    L = next_prime(n) if hash_len == -1 else hash_len
    mod, nb, dist, radial = ref_search(R, pos, h, support, vmin, vmax)
    off, cols = to_csr(nb[0], nb[1], n)
    A = torch.from_numpy(area)
    rho32 = R.density.computeDensity(radial, A, torch.from_numpy(nb), support).numpy()
    rho64 = R.density.computeDensity(radial.double(), A.double(), torch.from_numpy(nb), float(support)).numpy()
    si = sort_info(R, pos, h, vmin, vmax, L)
    out[f"{name}/pos"] = pos
    out[f"{name}/h"] = h
    out[f"{name}/area"] = area
    out[f"{name}/support"] = np.float32(support)
    out[f"{name}/vmin"] = np.asarray(vmin if vmin is not None else [np.nan, np.nan], np.float32)
    out[f"{name}/vmax"] = np.asarray(vmax if vmax is not None else [np.nan, np.nan], np.float32)
    out[f"{name}/hash_len"] = np.int64(L)
    out[f"{name}/offsets"] = off
    out[f"{name}/cols"] = cols
    out[f"{name}/rho32"] = rho32.astype(np.float32)
    out[f"{name}/rho64"] = rho64
    for k, v in si.items():
        out[f"{name}/si_{k}"] = v
    return mod


def main():
    R = ref_harness.load()
    torch.set_num_threads(4)
    out = {}
    cases = []

    # 1. jittered lattice (variant A shape), 48 x 48
    ns = 48
    dx = 1.0 / ns
    pos = workloads.jittered_lattice(ns, 0.1, 0)
    h = np.full(len(pos), np.float32(3 * dx), np.float32)
    area = np.full(len(pos), np.float32(dx * dx), np.float32)
    mod = add_case(R, out, "lattice", pos, h, area, np.float32(3 * dx), [0.0, 0.0], [1.0, 1.0])
    cases.append("lattice")

    # query: wall-like points around the lattice (buildNeighborListUnsortedPerParticle via searchExisting)
    rng = np.random.default_rng(1)
    q = np.concatenate([rng.uniform(-0.05, 1.05, (300, 2)), rng.uniform(0.0, 1.0, (200, 2))]).astype(np.float32)
    qh = np.full(len(q), np.float32(3 * dx), np.float32)
    qnb, qdist, qrad = mod.searchExisting(torch.from_numpy(q), torch.from_numpy(qh), mod._state, None)
    qr, qc = canon(qnb[0].numpy(), qnb[1].numpy())
    out["lattice/query_pos"] = q
    out["lattice/query_h"] = qh
    out["lattice/query_rows"] = qr
    out["lattice/query_cols"] = qc

    # 2. Gaussian blob + uniform (variant B shape), 2304 particles, same h as the lattice
    pos = workloads.gaussian_uniform_mix(2304, 0.1, (0.5, 0.5), 0)
    add_case(R, out, "mix", pos, h.copy(), area.copy(), np.float32(3 * dx), [0.0, 0.0], [1.0, 1.0])
    cases.append("mix")

    # 3. near-ties: partners placed within ~3e-7 relative of distance h
    n2 = 1500
    hh = np.float32(3.0 / 1024)
    c = rng.uniform(0.1, 0.9, (n2, 2))
    ang = rng.uniform(0, 2 * np.pi, n2)
    d = hh * (1 + rng.uniform(-3e-7, 3e-7, n2))
    pos = np.concatenate([c, c + np.stack([np.cos(ang) * d, np.sin(ang) * d], 1)]).astype(np.float32)
    hs = np.full(len(pos), hh, np.float32)
    add_case(R, out, "ties", pos, hs, np.full(len(pos), hh * hh / 9, np.float32), hh, [0.0, 0.0], [1.0, 1.0])
    cases.append("ties")

    # 4. edges: cell-boundary coordinates, duplicates, ragged per-particle supports, no domain given
    hh = np.float32(0.05)
    k = np.arange(0, 12, dtype=np.float32)
    gx, gy = np.meshgrid(k * hh, k * hh, indexing="ij")
    pos = np.stack([gx.ravel(), gy.ravel()], 1).astype(np.float32)
    pos = np.concatenate([pos, pos[:30], pos[::7] + np.float32(0.5) * hh]).astype(np.float32)
    hs = (hh * rng.uniform(0.5, 1.0, len(pos))).astype(np.float32)
    hs[::5] = hh
    add_case(R, out, "edges", pos, hs, np.full(len(pos), hh * hh / 9, np.float32), hh, None, None)
    cases.append("edges")

    # 5. single particle
    add_case(R, out, "single", np.array([[0.25, 0.75]], np.float32), np.array([0.1], np.float32),
             np.array([0.01], np.float32), np.float32(0.1), [0.0, 0.0], [1.0, 1.0])
    cases.append("single")

    # asymmetric: two point sets binned with the same cellsX and table length
    from nsearch import next_prime
    pa = workloads.jittered_lattice(32, 0.1, 3)
    pb = workloads.gaussian_uniform_mix(1000, 0.15, (0.5, 0.5), 4)
    ha = np.full(len(pa), np.float32(3 / 32), np.float32)
    hb = np.full(len(pb), np.float32(3 / 32), np.float32)
    L = next_prime(len(pa))
    sa = sort_info(R, pa, ha, [0.0, 0.0], [1.0, 1.0], L)
    sb = sort_info(R, pb, hb, [0.0, 0.0], [1.0, 1.0], L)
    assert sa["cells_x"] == sb["cells_x"]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
    ar, ac = R.ext.buildNeighborListAsymmetric(
        t(sa["sorted_pos"]), t(sa["sorted_h"]), t(sa["table"]), t(sa["cell_indices"]), t(sa["cum_cell"]),
        t(sa["cell_span"]), t(sa["sort"]), t(sb["sorted_pos"]), t(sb["sorted_h"]), t(sb["table"]),
        t(sb["cell_indices"]), t(sb["cum_cell"]), t(sb["cell_span"]), t(sb["sort"]), int(sa["cells_x"]), L)
    ar, ac = canon(ar.numpy(), ac.numpy())
    out["asym/pos_a"], out["asym/h_a"], out["asym/pos_b"], out["asym/h_b"] = pa, ha, pb, hb
    out["asym/hash_len"] = np.int64(L)
    out["asym/rows"], out["asym/cols"] = ar, ac
    out["cases"] = np.array(cases)

    path = os.path.join(HERE, "nsearch_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes;", {c: int(out[f"{c}/offsets"][-1]) for c in cases})


if __name__ == "__main__":
    main()
