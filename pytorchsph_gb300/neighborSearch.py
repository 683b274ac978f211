"""Drop-in for the reference's `neighborSearch` extension module.

The reference builds `neighborSearch` with
`torch.utils.cpp_extension.load(name="neighborSearch", sources=[...])`
(src/modules/neighborSearch.py:28) and binds four functions
(cppSrc/neighSearch.cpp:413-418).  This module exposes the same four names with the
same argument order and meaning, implemented by the GB300 kernels of
libsph_gb300.so; a maintainer swaps the `load(...)` call for
`from pytorchsph_gb300 import neighborSearch`.

Differences a caller can observe:
* every tensor must be a contiguous CUDA tensor (the reference's CUDA entry point
  checks the same, cppSrc/neighSearch.cpp:117-119; its CPU entry points accepted CPU
  tensors — there is no CPU path here and CPU inputs raise RuntimeError);
* the outputs are int32 CUDA tensors; pair order is deterministic (per query, or per
  occupied cell, in the reference's visiting order) where the reference CPU order
  depended on thread timing.  Pair sets are identical.
"""
from __future__ import annotations

import torch

from . import _native as N

__all__ = ["buildNeighborListCUDA", "buildNeighborList", "buildNeighborListAsymmetric",
           "buildNeighborListUnsortedPerParticle"]


def _check_input(t, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")


def _check_dtype(t, name, dtype):
    if t.dtype != dtype:
        raise RuntimeError(f"{name} must have dtype {dtype}, got {t.dtype}")


def _two_pass(count_fn, fill_fn, m, device):
    st = N.stream_ptr()
    counts = torch.empty(max(m, 1), dtype=torch.int32, device=device)
    if m == 0:
        e = torch.empty(0, dtype=torch.int32, device=device)
        return [e, e.clone()]
    count_fn(counts, st)
    offsets = torch.empty(m + 1, dtype=torch.int64, device=device)
    lib = N.load()
    sb = lib.sph_scan_scratch_bytes(m)
    scratch = torch.empty((sb + 7) // 8, dtype=torch.int64, device=device)
    N.call("sph_exclusive_scan_i32_to_i64", N.ptr(counts), N.ptr(offsets), m, N.ptr(scratch), scratch.numel() * 8, st)
    P = int(offsets[m].item())  # the reference reads the total back too (cppSrc/neighSearch_cuda.cu:267)
    rows = torch.empty(P, dtype=torch.int32, device=device)
    cols = torch.empty(P, dtype=torch.int32, device=device)
    if P > 0:
        fill_fn(offsets, rows, cols, st)
    return [rows, cols]


def _qmin_device(qMin, device):
    q = qMin.to(device=device, dtype=torch.float32).contiguous()
    if q.numel() != 2:
        raise RuntimeError("qMin must hold 2 values")
    return q


def buildNeighborListCUDA(queryParticles_, support_, sortedParticles, sortedSupport, hashTable_, cellIndices_,
                          cumCell_, cellSpan_, sort_, qMin_, hMax: float, cellsX: int, hashMapLength: int,
                          searchRadius: int):
    """cppSrc/neighSearch.cpp:143-170: pairs (query idx, sort[j]) with |x_q - x_j| < h_q."""
    for t, nm in [(queryParticles_, "queryParticles_"), (support_, "support_"), (sortedParticles, "sortedParticles"),
                  (sortedSupport, "sortedSupport"), (hashTable_, "hashTable_"), (cellIndices_, "cellIndices_"),
                  (cumCell_, "cumCell_"), (cellSpan_, "cellSpan_"), (sort_, "sort_"), (qMin_, "qMin_")]:
        _check_input(t, nm)
    for t, nm in [(queryParticles_, "queryParticles_"), (support_, "support_"), (sortedParticles, "sortedParticles"),
                  (qMin_, "qMin_")]:
        _check_dtype(t, nm, torch.float32)
    for t, nm in [(hashTable_, "hashTable_"), (cellIndices_, "cellIndices_"), (cumCell_, "cumCell_"),
                  (cellSpan_, "cellSpan_"), (sort_, "sort_")]:
        _check_dtype(t, nm, torch.int32)
    return _query(queryParticles_, support_, sortedParticles, hashTable_, cellIndices_, cumCell_, cellSpan_, sort_,
                  qMin_, hMax, cellsX, hashMapLength, searchRadius)


def _query(qpos, qh, spos, table, ci, cc, cs, sort, qmin, hmax, cells_x, L, r):
    m = qpos.shape[0]
    dev = qpos.device
    qmin = _qmin_device(qmin, dev)

    def count(counts, st):
        N.call("sph_nl_hashed_query_count", N.ptr(qpos), N.ptr(qh), m, N.ptr(spos), N.ptr(table), N.ptr(ci),
               N.ptr(cc), N.ptr(cs), N.ptr(qmin), float(hmax), int(cells_x), int(L), int(r), N.ptr(counts), st)

    def fill(offsets, rows, cols, st):
        N.call("sph_nl_hashed_query_fill", N.ptr(qpos), N.ptr(qh), m, N.ptr(spos), N.ptr(table), N.ptr(ci),
               N.ptr(cc), N.ptr(cs), N.ptr(sort), N.ptr(qmin), float(hmax), int(cells_x), int(L), int(r),
               N.ptr(offsets), N.ptr(rows), N.ptr(cols), st)

    return _two_pass(count, fill, m, dev)


def buildNeighborList(queryParticles_, support_, hashTable_, cellIndices_, cumCell_, cellSpan_, sort_,
                      cellsX: int, hashMapLength: int, searchRadius: int):
    """cppSrc/neighSearch.cpp:172-259: every occupied cell against its neighbor cells,
    pairs (sort[i], sort[j]) with |x_i - x_j| < h_i."""
    for t, nm in [(queryParticles_, "queryParticles_"), (support_, "support_"), (hashTable_, "hashTable_"),
                  (cellIndices_, "cellIndices_"), (cumCell_, "cumCell_"), (cellSpan_, "cellSpan_"), (sort_, "sort_")]:
        _check_input(t, nm)
    C = cellIndices_.shape[0]
    dev = queryParticles_.device

    def count(counts, st):
        N.call("sph_nl_hashed_cells_count", N.ptr(queryParticles_), N.ptr(support_), N.ptr(hashTable_),
               N.ptr(cellIndices_), N.ptr(cumCell_), N.ptr(cellSpan_), C, int(cellsX), int(hashMapLength),
               int(searchRadius), N.ptr(counts), st)

    def fill(offsets, rows, cols, st):
        N.call("sph_nl_hashed_cells_fill", N.ptr(queryParticles_), N.ptr(support_), N.ptr(hashTable_),
               N.ptr(cellIndices_), N.ptr(cumCell_), N.ptr(cellSpan_), N.ptr(sort_), C, int(cellsX),
               int(hashMapLength), int(searchRadius), N.ptr(offsets), N.ptr(rows), N.ptr(cols), st)

    return _two_pass(count, fill, C, dev)


def buildNeighborListUnsortedPerParticle(inputParticles_, inputSupport_, queryParticles_, support_, hashTable_,
                                         cellIndices_, cumCell_, cellSpan_, sort_, cellsX: int, hashMapLength: int,
                                         qMin_, hMax: float, searchRadius: int):
    """cppSrc/neighSearch.cpp:261-331: input points (any order) against the sorted set,
    pairs (input idx, sort[j]) with |x_b - x_j| < h_b."""
    for t, nm in [(inputParticles_, "inputParticles_"), (inputSupport_, "inputSupport_"),
                  (queryParticles_, "queryParticles_"), (support_, "support_"), (hashTable_, "hashTable_"),
                  (cellIndices_, "cellIndices_"), (cumCell_, "cumCell_"), (cellSpan_, "cellSpan_"), (sort_, "sort_")]:
        _check_input(t, nm)
    return _query(inputParticles_, inputSupport_, queryParticles_, hashTable_, cellIndices_, cumCell_, cellSpan_,
                  sort_, qMin_, hMax, cellsX, hashMapLength, searchRadius)


def buildNeighborListAsymmetric(queryParticlesA_, supportA_, hashTableA_, cellIndicesA_, cumCellA_, cellSpanA_, sortA_,
                                queryParticlesB_, supportB_, hashTableB_, cellIndicesB_, cumCellB_, cellSpanB_, sortB_,
                                cellsX: int, hashMapLength: int):
    """cppSrc/neighSearch.cpp:333-410: cells of A against the table of B (radius 1),
    pairs (sortA[i], sortB[j]) with |x_i - x_j| < h_i."""
    for t, nm in [(queryParticlesA_, "queryParticlesA_"), (supportA_, "supportA_"), (hashTableA_, "hashTableA_"),
                  (cellIndicesA_, "cellIndicesA_"), (cumCellA_, "cumCellA_"), (cellSpanA_, "cellSpanA_"),
                  (sortA_, "sortA_"), (queryParticlesB_, "queryParticlesB_"), (supportB_, "supportB_"),
                  (hashTableB_, "hashTableB_"), (cellIndicesB_, "cellIndicesB_"), (cumCellB_, "cumCellB_"),
                  (cellSpanB_, "cellSpanB_"), (sortB_, "sortB_")]:
        _check_input(t, nm)
    C = cellIndicesA_.shape[0]
    dev = queryParticlesA_.device

    def count(counts, st):
        N.call("sph_nl_hashed_asym_count", N.ptr(queryParticlesA_), N.ptr(supportA_), N.ptr(hashTableA_),
               N.ptr(cellIndicesA_), N.ptr(cumCellA_), N.ptr(cellSpanA_), C, N.ptr(queryParticlesB_),
               N.ptr(hashTableB_), N.ptr(cellIndicesB_), N.ptr(cumCellB_), N.ptr(cellSpanB_), int(cellsX),
               int(hashMapLength), N.ptr(counts), st)

    def fill(offsets, rows, cols, st):
        N.call("sph_nl_hashed_asym_fill", N.ptr(queryParticlesA_), N.ptr(supportA_), N.ptr(hashTableA_),
               N.ptr(cellIndicesA_), N.ptr(cumCellA_), N.ptr(cellSpanA_), N.ptr(sortA_), C, N.ptr(queryParticlesB_),
               N.ptr(hashTableB_), N.ptr(cellIndicesB_), N.ptr(cumCellB_), N.ptr(cellSpanB_), N.ptr(sortB_),
               int(cellsX), int(hashMapLength), N.ptr(offsets), N.ptr(rows), N.ptr(cols), st)

    return _two_pass(count, fill, C, dev)
