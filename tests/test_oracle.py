"""The oracle (oracle/nsearch_oracle.c) against the golden vectors produced by the
reference itself (tests/golden/make_golden.py), and — where the reference checkout is
present — against the compiled reference directly."""
import os

import numpy as np
import pytest

import nsearch as ns


def _csr_to_pairs(off, cols):
    rows = np.repeat(np.arange(len(off) - 1), np.diff(off))
    return rows.astype(np.int64) * (1 << 32) + cols.astype(np.int64)


def _dom(g, c):
    v = g[f"{c}/vmin"]
    return None if np.isnan(v).any() else v, None if np.isnan(v).any() else g[f"{c}/vmax"]


@pytest.mark.parametrize("case", ["lattice", "mix", "ties", "edges", "single"])
def test_oracle_pairs_match_reference(golden, case):
    g = golden
    vmin, vmax = _dom(g, case)
    si, off, cols = ns.search(g[f"{case}/pos"], g[f"{case}/h"], vmin, vmax, int(g[f"{case}/hash_len"]))
    got = _csr_to_pairs(off, cols)
    ref = _csr_to_pairs(g[f"{case}/offsets"], g[f"{case}/cols"])
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("case", ["lattice", "mix", "edges"])
def test_oracle_sort_and_hash_map_match_reference(golden, case):
    g = golden
    vmin, vmax = _dom(g, case)
    si = ns.SortInfo(g[f"{case}/pos"], g[f"{case}/h"], vmin, vmax, int(g[f"{case}/hash_len"]))
    assert si.cells_x == int(g[f"{case}/si_cells_x"])
    assert np.array_equal(si.qmin, g[f"{case}/si_qmin"])
    assert np.float32(si.hmax) == g[f"{case}/si_hmax"]
    assert np.array_equal(si.sorted_lin, g[f"{case}/si_sorted_lin"])
    assert np.array_equal(si.table, g[f"{case}/si_table"])
    # cells inside one hash bucket may come in any order (the reference's argsort is not stable)
    def cells(ci, cc, cs):
        return sorted(zip(ci.tolist(), cc.tolist(), cs.tolist()))
    assert cells(si.cell_indices, si.cum_cell, si.cell_span) == cells(
        g[f"{case}/si_cell_indices"], g[f"{case}/si_cum_cell"], g[f"{case}/si_cell_span"])


def test_oracle_query_matches_reference(golden):
    g = golden
    si = ns.SortInfo(g["lattice/pos"], g["lattice/h"], g["lattice/vmin"], g["lattice/vmax"],
                     int(g["lattice/hash_len"]))
    r, c = ns.nl_query(si, g["lattice/query_pos"], g["lattice/query_h"])
    got = np.sort(r.astype(np.int64) * (1 << 32) + c)
    ref = g["lattice/query_rows"].astype(np.int64) * (1 << 32) + g["lattice/query_cols"]
    assert np.array_equal(got, ref)


def test_oracle_asym_matches_reference(golden):
    g = golden
    L = int(g["asym/hash_len"])
    a = ns.SortInfo(g["asym/pos_a"], g["asym/h_a"], np.zeros(2, np.float32), np.ones(2, np.float32), L)
    b = ns.SortInfo(g["asym/pos_b"], g["asym/h_b"], np.zeros(2, np.float32), np.ones(2, np.float32), L)
    r, c = ns.nl_asym(a, b)
    got = np.sort(r.astype(np.int64) * (1 << 32) + c)
    ref = g["asym/rows"].astype(np.int64) * (1 << 32) + g["asym/cols"]
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("case", ["lattice", "mix", "ties", "edges"])
def test_oracle_density_matches_reference(golden, case):
    g = golden
    off, cols = g[f"{case}/offsets"], g[f"{case}/cols"]
    sup = float(g[f"{case}/support"])
    r32 = ns.density(off, cols, g[f"{case}/pos"], g[f"{case}/area"], sup)
    r64 = ns.density(off, cols, g[f"{case}/pos"], g[f"{case}/area"], sup, use_double=True)
    ref32, ref64 = g[f"{case}/rho32"], g[f"{case}/rho64"]
    scale = np.abs(ref64).max()
    assert np.abs(r32 - ref32).max() <= 2e-6 * scale
    # float64 oracle vs the reference's float64 run (same float32 radial distances in both)
    assert np.abs(r64 - ref64).max() <= 1e-6 * scale


def test_predicate_spellings_differ_on_ties(golden):
    """The near-tie case separates the predicate spellings: only fmaf(dx,dx,dy*dy) reproduces
    the reference's pair set, the other spellings differ."""
    g = golden
    ref = _csr_to_pairs(g["ties/offsets"], g["ties/cols"])
    for pred in (ns.PRED_FMA_YY, ns.PRED_UNFUSED, ns.PRED_DOUBLE_SQRT):
        si, off, cols = ns.search(g["ties/pos"], g["ties/h"], g["ties/vmin"], g["ties/vmax"], pred=pred)
        assert not np.array_equal(_csr_to_pairs(off, cols), ref)


from build_ref import REF_ROOT as REF  # noqa: E402  (where the reference checkout lies, if anywhere)


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "cppSrc", "neighSearch.cpp")),
                    reason="reference checkout not present")
@pytest.mark.parametrize("seed", [0, 1])
def test_oracle_against_compiled_reference(seed):
    import torch
    import build_ref
    ext = build_ref.build()
    from pytorchsph_gb300 import workloads
    pos = workloads.gaussian_uniform_mix(20000, 0.05, (0.5, 0.5), seed)
    h = np.full(len(pos), np.float32(3 / 200), np.float32)
    si = ns.SortInfo(pos, h, np.zeros(2, np.float32), np.ones(2, np.float32))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
    rr, rc = ext.buildNeighborList(t(si.sorted_pos), t(si.sorted_h), t(si.table), t(si.cell_indices),
                                   t(si.cum_cell), t(si.cell_span), t(si.sort), si.cells_x, si.hash_len, 1)
    r, c = ns.nl_cells(si)
    ref = np.sort(rr.numpy().astype(np.int64) * (1 << 32) + rc.numpy())
    got = np.sort(r.astype(np.int64) * (1 << 32) + c)
    assert np.array_equal(got, ref)


def test_square_root_free_predicate_is_exact():
    """The GPU tests v <= F(h) instead of sqrtf(v) < h (csrc/sph_common.cuh, sq_threshold).
    Restated here with numpy float32/float64 and checked against IEEE sqrtf on random and
    adversarial (v within a few ulps of h^2) inputs."""
    rng = np.random.default_rng(0)
    h = np.concatenate([rng.uniform(1e-4, 10, 200000), np.float32(3 / 1024) * np.ones(1000),
                        2.0 ** rng.integers(-20, 20, 1000)]).astype(np.float32)
    p = np.nextafter(h, np.float32(0))
    m = (p.astype(np.float64) + h.astype(np.float64)) * 0.5
    m2 = m * m
    F = m2.astype(np.float32)
    F = np.where(F.astype(np.float64) >= m2, np.nextafter(F, np.float32(0)), F)
    base = (h.astype(np.float64) ** 2).astype(np.float32)
    for k in range(-6, 7):
        v = base.view(np.int32) + np.int32(k)
        v = v.view(np.float32)
        ref = np.sqrt(v) < h
        assert np.array_equal(v <= F, ref), k
    v = rng.uniform(0, 100, h.shape).astype(np.float32)
    assert np.array_equal(v <= F, np.sqrt(v) < h)
