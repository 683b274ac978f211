"""The module-level search functions of the reference's src/modules/neighborSearch.py on the GPU.

`sortPositions` (:30-55), `constructHashMap` (:58-88), `constructNeighborhoods` (:91-115),
`constructNeighborhoodsPreSorted` (:118-136), `constructNeighborhoodsCUDA` (:139-159),
`constructNeighborhoodsPreSortedCUDA` (:161-171) and `nextprime`, with the reference's
argument order and return tuples, running on libsph_gb300.so (sph_grid_build,
sph_cell_keys, sph_counting_sort, sph_gather_sorted, sph_hash_map_build) and on the
extension drop-in (`pytorchsph_gb300.neighborSearch`).

What a caller can observe against the reference:
* inputs must be float32 CUDA tensors; there is no CPU path;
* particles of one cell keep their input order (a stable sort), and cells of one hash bucket
  come in increasing cell order; the reference's `torch.argsort` is not stable, so its order
  inside a cell or a bucket is unspecified.  Sorted keys, the grid, the hash table and every
  pair set are the same;
* `supportScale` must be 1.0, the value every caller in the reference passes.
"""
from __future__ import annotations

import torch

from . import _native as N
from . import neighborSearch as _ext
from .search import MAX_CELLS, _f2, grid_from_bytes, next_prime

__all__ = ["sortPositions", "constructHashMap", "constructNeighborhoods", "constructNeighborhoodsPreSorted",
           "constructNeighborhoodsCUDA", "constructNeighborhoodsPreSortedCUDA", "nextprime"]


def nextprime(n: int) -> int:
    """Smallest prime greater than n (sympy.nextprime, used at neighborSearch.py:95)."""
    return next_prime(int(n))


def _float32_cuda(t, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32:
        raise RuntimeError(f"{name} must be a float32 CUDA tensor")
    return t.contiguous()


def _host2(v):
    if v is None:
        return None
    if isinstance(v, torch.Tensor):
        v = v.detach().to("cpu", torch.float32)
    return [float(v[0]), float(v[1])]


def sortPositions(queryParticles, querySupport, supportScale: float = 1.0, qMin=None, qMax=None):
    """src/modules/neighborSearch.py:30-55: (sortedPositions, sortedSupport,
    sortedLinearIndices int32, sortingIndices int64, cellCount int, qMin float32 [2] (device),
    hMax float).  Reads the grid back to the host once (the reference's int() / float())."""
    if float(supportScale) != 1.0:
        raise RuntimeError("sortPositions: only supportScale = 1.0 is supported")
    pos = _float32_cuda(queryParticles, "queryParticles")
    sup = _float32_cuda(querySupport, "querySupport")
    if pos.dim() != 2 or pos.shape[1] != 2 or sup.shape[0] != pos.shape[0]:
        raise RuntimeError("sortPositions: positions [N, 2] and supports [N] expected")
    n = pos.shape[0]
    if n == 0:
        raise RuntimeError("sortPositions: no particles")
    lib = N.load()
    dev = pos.device
    st = N.stream_ptr()
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    grid = torch.empty(8, dtype=torch.int32, device=dev)
    gs = torch.empty((lib.sph_grid_scratch_bytes(n) + 7) // 8, dtype=torch.int64, device=dev)
    N.call("sph_grid_build", N.ptr(pos), N.ptr(sup), n, _f2(_host2(qMin)), _f2(_host2(qMax)), MAX_CELLS,
           N.ptr(grid), N.ptr(status), N.ptr(gs), gs.numel() * 8, st)
    info = grid_from_bytes(grid)
    if int(status.item()) != 0:
        raise RuntimeError("sortPositions: non-finite input or a grid of more than 2^28 cells")
    cap = max(info["num_cells"], 1)
    keys = torch.empty(n, dtype=torch.int32, device=dev)
    order = torch.empty(n, dtype=torch.int32, device=dev)
    skeys = torch.empty(n, dtype=torch.int32, device=dev)
    cell_count = torch.zeros(cap + 1, dtype=torch.int32, device=dev)
    cell_start = torch.empty(cap + 2, dtype=torch.int32, device=dev)
    N.call("sph_cell_keys", N.ptr(pos), n, N.ptr(grid), cap, N.ptr(keys), None, N.ptr(cell_count), N.ptr(status), st)
    cs = torch.empty((lib.sph_counting_sort_scratch_bytes(n, cap) + 7) // 8, dtype=torch.int64, device=dev)
    N.call("sph_counting_sort", N.ptr(keys), n, cap, N.ptr(cell_count), N.ptr(cell_start), N.ptr(order),
           N.ptr(skeys), N.ptr(status), N.ptr(cs), cs.numel() * 8, st)
    xy = torch.empty((n, 2), dtype=torch.float32, device=dev)
    sh = torch.empty(n, dtype=torch.float32, device=dev)
    N.call("sph_gather_sorted", N.ptr(order), n, N.ptr(pos), N.ptr(sup), None, N.ptr(xy), N.ptr(sh), None, st)
    flags = int(status.item())
    if flags & (N.SPH_FLAG_OUT_OF_GRID | N.SPH_FLAG_NONFINITE):
        raise RuntimeError("sortPositions: particles outside the grid given by qMin / qMax")
    qmin = torch.tensor(info["qmin"], dtype=torch.float32, device=dev)
    return xy, sh, skeys, order.long(), int(info["cells_x"]), qmin, float(info["hmax"])


def constructHashMap(sortedPositions, sortedSupport, sortedIndices, sort, hashMapLength: int, cellCount: int):
    """src/modules/neighborSearch.py:58-88: (hashTable int32 [L, 2], cellIndices, cumCell (the
    particle count of each cell), cellSpan (its first sorted index)), all int32 [C] in hash
    order.  The map is built on the device without a host wait; slicing the C occupied
    cells reads C back once (the reference's output shapes need it as well)."""
    keys = sortedIndices
    if not isinstance(keys, torch.Tensor) or not keys.is_cuda:
        raise RuntimeError("sortedIndices must be a CUDA tensor")
    keys = keys.to(torch.int32).contiguous()
    n = keys.shape[0]
    L = int(hashMapLength)
    if n == 0 or L <= 0 or int(cellCount) <= 0:
        raise RuntimeError("constructHashMap: empty input or bad hashMapLength / cellCount")
    dev = keys.device
    lib = N.load()
    table = torch.empty((L, 2), dtype=torch.int32, device=dev)
    ci = torch.empty(n, dtype=torch.int32, device=dev)
    cum = torch.empty(n, dtype=torch.int32, device=dev)
    span = torch.empty(n, dtype=torch.int32, device=dev)
    C = torch.empty(1, dtype=torch.int32, device=dev)
    sc = torch.empty((lib.sph_hash_map_scratch_bytes(n, L) + 7) // 8, dtype=torch.int64, device=dev)
    N.call("sph_hash_map_build", N.ptr(keys), n, int(cellCount), L, N.ptr(table), N.ptr(ci), N.ptr(cum), N.ptr(span),
           N.ptr(C), N.ptr(sc), sc.numel() * 8, N.stream_ptr())
    c = int(C.item())
    return table, ci[:c], cum[:c], span[:c]


def constructNeighborhoods(queryPositions, querySupports, hashMapLength: int = -1, supportScale: float = 1.0,
                           minCoord=None, maxCoord=None, searchRadius: int = 1):
    """src/modules/neighborSearch.py:91-115 (the extension's buildNeighborList on the hash map)."""
    sp, ss, sli, si, cellCount, qMin, hMax = sortPositions(queryPositions, querySupports, 1.0, minCoord, maxCoord)
    if hashMapLength == -1:
        hashMapLength = nextprime(queryPositions.shape[0])
    table, cli, cellOffsets, cellCounters = constructHashMap(sp, ss, sli, si, hashMapLength, cellCount)
    si = si.to(torch.int32)
    rows, cols = _ext.buildNeighborList(sp, ss, table, cli, cellOffsets, cellCounters, si, cellCount, hashMapLength,
                                        searchRadius)
    return (rows.to(torch.int64), cols.to(torch.int64), None, None, (qMin, hMax, si, sp, ss), (table, hashMapLength),
            (cli, cellOffsets, cellCounters, cellCount))


def constructNeighborhoodsPreSorted(queryPositions, querySupports, particleState, hashMap, cellMap,
                                    searchRadius: int = 1):
    """src/modules/neighborSearch.py:118-136: query points against an existing map."""
    qMin, hMax, si, sp, ss = particleState
    table, L = hashMap
    cli, cellOffsets, cellCounters, cellCount = cellMap
    rows, cols = _ext.buildNeighborListUnsortedPerParticle(
        _float32_cuda(queryPositions, "queryPositions"), _float32_cuda(querySupports, "querySupports"), sp, ss, table,
        cli, cellOffsets, cellCounters, si, cellCount, L, qMin.to(torch.float32), float(hMax), searchRadius)
    return rows.to(torch.int64), cols.to(torch.int64)


def constructNeighborhoodsCUDA(queryPositions, querySupports, hashMapLength: int = -1, supportScale: float = 1.0,
                               minCoord=None, maxCoord=None, searchRadius: int = 1):
    """src/modules/neighborSearch.py:139-159: per-query search, pairs finalised in (i, j) order."""
    sp, ss, sli, si, cellCount, qMin, hMax = sortPositions(queryPositions, querySupports, 1.0, minCoord, maxCoord)
    if hashMapLength == -1:
        hashMapLength = nextprime(queryPositions.shape[0])
    table, cli, cellOffsets, cellCounters = constructHashMap(sp, ss, sli, si, hashMapLength, cellCount)
    si = si.to(torch.int32)
    i, j = _ext.buildNeighborListCUDA(_float32_cuda(queryPositions, "queryPositions"),
                                      _float32_cuda(querySupports, "querySupports"), sp, ss, table, cli, cellOffsets,
                                      cellCounters, si, qMin, hMax, cellCount, hashMapLength, searchRadius)
    # the finalize of neighborSearch.py:153-157: stable sort by j, then by i
    j, jj = torch.sort(j, dim=0, stable=True)
    i = i[jj]
    i, ii = torch.sort(i, dim=0, stable=True)
    j = j[ii]
    return (i.to(torch.int64), j.to(torch.int64), None, None, (qMin, hMax, si, sp, ss), (table, hashMapLength),
            (cli, cellOffsets, cellCounters, cellCount))


def constructNeighborhoodsPreSortedCUDA(queryPositions, querySupports, particleState, hashMap, cellMap,
                                        searchRadius: int = 1):
    """src/modules/neighborSearch.py:161-171."""
    qMin, hMax, si, sp, ss = particleState
    table, L = hashMap
    cli, cellOffsets, cellCounters, cellCount = cellMap
    rows, cols = _ext.buildNeighborListCUDA(
        _float32_cuda(queryPositions, "queryPositions"), _float32_cuda(querySupports, "querySupports"), sp, ss, table,
        cli, cellOffsets, cellCounters, si, qMin.to(torch.float32), float(hMax), cellCount, L, searchRadius)
    return rows.to(torch.int64), cols.to(torch.int64)
