"""Periodic boundaries on the GPU (pytorchsph_gb300.periodic) against the reference's own
createGhostParticlesKernel and search (tests/golden/periodic_golden.npz): ghost indices,
offsets and category counts bit for bit; the search over real + ghost particles gives the
reference's pair set bit for bit; the copy-free periodic search gives the same pairs of the
real particles, each ghost column replaced by (its particle, its image shift)."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "periodic_golden.npz")
CASES = ["x", "xy", "xy_dense"]


@pytest.fixture(scope="module")
def gold():
    g = np.load(GOLDEN)
    return g, json.loads(str(g["meta"]))


def key(r, c, code=None):
    k = np.asarray(r, np.int64) * (1 << 33) + np.asarray(c, np.int64) * 16
    if code is not None:
        k = k + np.asarray(code, np.int64)
    return np.sort(k)


@pytest.mark.parametrize("case", CASES)
def test_ghosts_match_reference(cuda, gold, case):
    from pytorchsph_gb300.periodic import createGhostParticlesKernel
    g, meta = gold
    m = meta[case]
    pos = torch.from_numpy(g[f"{case}/pos"]).to(cuda)
    filters, offsets = createGhostParticlesKernel(pos, m["domain_min"], m["domain_max"], m["buffer"], m["support"],
                                                  m["periodicX"], m["periodicY"])
    assert [len(f) for f in filters] == [int(c) for c in g[f"{case}/ghost_counts"]]
    assert np.array_equal(torch.cat(filters).cpu().numpy(), g[f"{case}/ghost_indices"])
    assert np.array_equal(torch.vstack(offsets).cpu().numpy(), g[f"{case}/ghost_offsets"])


@pytest.mark.parametrize("case", CASES)
def test_module_and_extended_search_match_reference(cuda, gold, case):
    """periodicBCModule.enforcePeriodicBC appends the copies; the search over the extended
    arrays gives the reference's pairs."""
    from pytorchsph_gb300.periodic import periodicBCModule
    from pytorchsph_gb300.search import GridSearch
    g, meta = gold
    m = meta[case]
    pos = torch.from_numpy(g[f"{case}/pos"]).to(cuda)
    n = pos.shape[0]
    h = m["support"]
    st = {"fluidPosition": pos.clone(), "UID": torch.arange(n, device=cuda), "numParticles": n,
          "fluidSupport": torch.full((n,), h, device=cuda)}
    cfg = {"particle": {"support": h}, "periodicBC": {"periodicX": m["periodicX"], "periodicY": m["periodicY"],
                                                      "buffer": m["buffer"]},
           "domain": {"min": m["domain_min"], "max": m["domain_max"],
                      "virtualMin": [v - m["buffer"] * h for v in m["domain_min"]],
                      "virtualMax": [v + m["buffer"] * h for v in m["domain_max"]]},
           "compute": {"precision": torch.float32}}
    mod = periodicBCModule()
    mod.initialize(cfg, st)
    mod.enforcePeriodicBC(st, None)
    gi = g[f"{case}/ghost_indices"]
    assert st["numParticles"] == n + len(gi) and st["realParticles"] == n
    ext = np.concatenate([g[f"{case}/pos"], g[f"{case}/pos"][gi] + g[f"{case}/ghost_offsets"]])
    assert np.array_equal(st["fluidPosition"].cpu().numpy(), ext)
    assert np.array_equal(st["UID"].cpu().numpy(), np.concatenate([np.arange(n), gi]))
    res = GridSearch(cuda).run(st["fluidPosition"], st["fluidSupport"], density=False,
                               min_coord=np.array(cfg["domain"]["virtualMin"], np.float32),
                               max_coord=np.array(cfg["domain"]["virtualMax"], np.float32))
    pairs, _, _ = res.to_coo(distances=False)
    p = pairs.cpu().numpy()
    assert np.array_equal(key(p[0], p[1]), key(g[f"{case}/rows"], g[f"{case}/cols"]))
    # the copies go away again
    mod.resetState(st)
    assert st["numParticles"] == n and torch.equal(st["fluidPosition"], pos)


@pytest.mark.parametrize("case", CASES)
def test_copy_free_periodic_search_matches_reference(cuda, gold, case):
    from pytorchsph_gb300.periodic import periodic_neighbors
    g, meta = gold
    m = meta[case]
    pos = torch.from_numpy(g[f"{case}/pos"]).to(cuda)
    n = pos.shape[0]
    rows, cols, codes = periodic_neighbors(pos, torch.full((n,), m["support"], device=cuda), m["domain_min"],
                                           m["domain_max"], m["periodicX"], m["periodicY"])
    r, c, k = rows.cpu().numpy(), cols.cpu().numpy(), codes.cpu().numpy()
    assert np.all(np.diff(r * (1 << 32) + c) > 0)            # (i, j) order, no duplicates
    # the reference's pairs of real rows, ghost columns mapped to (particle, image shift)
    gr, gc = g[f"{case}/rows"].astype(np.int64), g[f"{case}/cols"].astype(np.int64)
    sel = gr < n
    gr, gc = gr[sel], gc[sel]
    gi, go = g[f"{case}/ghost_indices"], g[f"{case}/ghost_offsets"]
    L = np.array(m["domain_max"]) - np.array(m["domain_min"])
    shift = np.zeros((len(gc), 2), np.int64)
    ghost = gc >= n
    shift[ghost] = np.rint(go[gc[ghost] - n] / L).astype(np.int64)
    real = np.where(ghost, gi[np.clip(gc - n, 0, len(gi) - 1)], gc)
    ref_code = (shift[:, 0] + 1) | ((shift[:, 1] + 1) << 2)
    assert np.array_equal(key(r, c, k), key(gr, real, ref_code))
