"""Native GB300 neighbor search: cell keys -> sort by cell key -> sorted SoA -> cell table
-> two-pass CSR (count with fused density, scan, fill).

This replaces the reference's search path (src/modules/neighborSearch.py:30-171 and
cppSrc/neighSearch*.{cpp,cu}).  Pairs are kept as CSR over the particles in cell-sorted
order (`offsets[n+1]`, `cols[P]` = sorted neighbor indices); the reference's COO form
(`fluidNeighbors` [2, P] in original indices, ordered by (i, j)) is produced on request
by `CSRNeighbors.to_coo()`.

With `cell_capacity` and `pair_capacity` given, `GridSearch.run(..., sync=False)` issues
no host synchronisation and can be captured in a CUDA graph; overflow is reported
through the device status word (`CSRNeighbors.check()`).
"""
from __future__ import annotations

import ctypes
import math

import torch

from . import _native as N

MAX_CELLS = 1 << 28  # dense cell table limit (1 GiB of int32 starts)


class Workspace:
    """Grow-only device buffers, reused across calls (one torch allocation per name)."""

    def __init__(self, device):
        self.device = torch.device(device)
        self._bufs = {}

    def get(self, name, numel, dtype=torch.int32):
        numel = max(int(numel), 1)
        b = self._bufs.get(name)
        if b is None or b.numel() < numel or b.dtype != dtype:
            b = torch.empty(numel, dtype=dtype, device=self.device)
            self._bufs[name] = b
        return b[:numel]

    def zeros(self, name, numel, dtype=torch.int32):
        """Like get(), but zero-filled the first time the buffer is created."""
        b = self._bufs.get(name)
        fresh = b is None or b.numel() < max(int(numel), 1) or b.dtype != dtype
        t = self.get(name, numel, dtype)
        if fresh:
            t.zero_()
        return t

    def bytes(self, name, nbytes):
        return self.get(name, (int(nbytes) + 7) // 8, torch.int64)


def grid_from_bytes(t: torch.Tensor) -> dict:
    """Decode an sph_grid struct read back to the host."""
    raw = t.detach().cpu().view(torch.int32)
    f = raw[:4].view(torch.float32)
    i = raw[4:8]
    return {"qmin": (float(f[0]), float(f[1])), "hmax": float(f[2]), "cells_x": int(i[0]),
            "cells_y": int(i[1]), "num_cells": int(i[2])}


def _f2(v):
    if v is None:
        return None
    arr = (ctypes.c_float * 2)(float(v[0]), float(v[1]))
    return ctypes.cast(arr, ctypes.c_void_p)


class CSRNeighbors:
    """Result of one search: sorted SoA, cell table and CSR pairs (all on the device)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)
        self._rank = None

    # n, order, keys, xy, sh, sa, cell_start, counts, offsets, cols, rho, grid, status,
    # cell_capacity, pair_capacity, kernel_support, search_radius (in cells of the grid),
    # cell_ratio (cells per support)

    @property
    def num_pairs(self) -> int:
        return int(self.offsets[self.n].item())

    def flags(self) -> int:
        return int(self.status.item())

    def check(self):
        f = self.flags()
        if f:
            raise N.SPHError(f"neighbor search: {N.decode_flags(f)}")
        if self.num_pairs > self.pair_capacity:
            raise N.SPHError("neighbor search: neighbor pair buffer too small")

    def grid_info(self) -> dict:
        return grid_from_bytes(self.grid)

    @property
    def rank(self):
        if self._rank is None:
            self._rank = torch.empty(self.n, dtype=torch.int32, device=self.order.device)
            N.call("sph_invert_permutation", N.ptr(self.order), self.n, N.ptr(self._rank), N.stream_ptr())
        return self._rank

    def to_original(self, field: torch.Tensor) -> torch.Tensor:
        """A sorted-order float32 field back in original particle order."""
        out = torch.empty(self.n, dtype=torch.float32, device=self.order.device)
        if self.n == 0:
            return out
        N.call("sph_scatter_f32", N.ptr(self.order), N.ptr(field), self.n, N.ptr(out), N.stream_ptr())
        return out

    def density(self) -> torch.Tensor:
        """rho in original particle order."""
        return self.to_original(self.rho)

    def to_coo(self, grad_threshold: float = 1e-7, distances: bool = True):
        """(fluidNeighbors int64 [2,P], fluidDistances [P,2], fluidRadialDistances [P]) in the
        reference layout (src/modules/neighborSearch.py:216-227), pairs ordered by (i, j)."""
        self.check()
        P = self.num_pairs
        dev = self.order.device
        if self.n == 0:
            return (torch.empty((2, 0), dtype=torch.int64, device=dev),
                    torch.empty((0, 2), dtype=torch.float32, device=dev) if distances else None,
                    torch.empty(0, dtype=torch.float32, device=dev) if distances else None)
        st = N.stream_ptr()
        cnt_orig = torch.empty(self.n, dtype=torch.int32, device=dev)
        N.call("sph_scatter_counts", N.ptr(self.order), N.ptr(self.counts), self.n, N.ptr(cnt_orig), st)
        orig_off = torch.empty(self.n + 1, dtype=torch.int64, device=dev)
        scratch = torch.empty((N.load().sph_scan_scratch_bytes(self.n) + 7) // 8, dtype=torch.int64, device=dev)
        N.call("sph_exclusive_scan_i32_to_i64", N.ptr(cnt_orig), N.ptr(orig_off), self.n, N.ptr(scratch),
               scratch.numel() * 8, st)
        pairs = torch.empty((2, P), dtype=torch.int64, device=dev)
        dist = torch.empty((P, 2), dtype=torch.float32, device=dev) if distances else None
        radial = torch.empty(P, dtype=torch.float32, device=dev) if distances else None
        N.call("sph_nl_to_coo", N.ptr(self.xy), self.n, N.ptr(self.order), N.ptr(self.rank),
               N.ptr(self.offsets), N.ptr(self.cols), N.ptr(orig_off), float(grad_threshold),
               float(self.kernel_support or 1.0), N.ptr(pairs), P, N.ptr(dist), N.ptr(radial), st)
        return pairs, dist, radial

    def query(self, qpos: torch.Tensor, qsupport: torch.Tensor, search_radius: int | None = None,
              original_indices: bool = True):
        """Pairs of arbitrary query points against this grid (searchExisting,
        src/modules/neighborSearch.py:231-252): rows = query index, cols = particle index
        (original order by default), predicate |x_q - x_j| < support_q.  search_radius counts
        supports, as in GridSearch.run (the grid's cells are support / cell_ratio)."""
        r = self.search_radius if search_radius is None else int(search_radius) * getattr(self, "cell_ratio", 1)
        m = qpos.shape[0]
        dev = self.order.device
        st = N.stream_ptr()
        qpos = qpos.contiguous()
        qsupport = qsupport.contiguous()
        counts = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
        if m == 0:
            e = torch.empty(0, dtype=torch.int32, device=dev)
            return e, e.clone()
        N.call("sph_nl_query_count", N.ptr(qpos), N.ptr(qsupport), m, N.ptr(self.xy), N.ptr(self.cell_start),
               N.ptr(self.grid), self.cell_capacity, r, N.ptr(counts), st)
        off = torch.empty(m + 1, dtype=torch.int64, device=dev)
        scratch = torch.empty((N.load().sph_scan_scratch_bytes(m) + 7) // 8, dtype=torch.int64, device=dev)
        N.call("sph_exclusive_scan_i32_to_i64", N.ptr(counts), N.ptr(off), m, N.ptr(scratch), scratch.numel() * 8, st)
        P = int(off[m].item())
        rows = torch.empty(P, dtype=torch.int32, device=dev)
        cols = torch.empty(P, dtype=torch.int32, device=dev)
        if P:
            N.call("sph_nl_query_fill", N.ptr(qpos), N.ptr(qsupport), m, N.ptr(self.xy), N.ptr(self.cell_start),
                   N.ptr(self.grid), self.cell_capacity, r, N.ptr(self.order) if original_indices else None,
                   N.ptr(off), N.ptr(rows), N.ptr(cols), st)
        return rows, cols


class GridSearch:
    """Hashed-grid neighbor search with CSR output, reusing its device workspace.

    sort = "counting" (one pass, the digit is the whole cell key) or "radix" (LSD radix
    with `digit_bits` per pass); both give the (key, index) order of a stable sort.
    segments = True: the count pass keeps each particle's accepted candidates as bit masks
    and the fill expands them (one pair test per candidate instead of two); False: the fill
    tests the candidates again.  Both give the same CSR.
    cell_ratio > 1: grid cells of max(support) / cell_ratio, searched cell_ratio times
    search_radius cells out; the same pair set from fewer candidates, each row's pairs in
    the order of the finer cells."""

    def __init__(self, device=None, sort: str = "counting", digit_bits: int = 8, segments: bool = True,
                 cell_ratio: int = 1):
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self.ws = Workspace(self.device)
        if sort not in ("counting", "radix"):
            raise ValueError(sort)
        self.sort = sort
        self.digit_bits = int(digit_bits)
        self.segments = bool(segments)
        if not 1 <= int(cell_ratio) <= 8:
            raise ValueError(cell_ratio)
        self.cell_ratio = int(cell_ratio)

    def grid(self, pos, support, min_coord=None, max_coord=None, cell_capacity=MAX_CELLS):
        """Compute the search grid on the device; returns the device grid bytes."""
        lib = N.load()
        n = pos.shape[0]
        grid = self.ws.get("grid", 8, torch.int32)
        status = self.ws.get("status", 1, torch.int32)
        scratch = self.ws.bytes("grid_scratch", lib.sph_grid_scratch_bytes(n))
        N.call("sph_grid_build_ratio", N.ptr(pos), N.ptr(support), n, _f2(min_coord), _f2(max_coord),
               self.cell_ratio, int(cell_capacity), N.ptr(grid), N.ptr(status), N.ptr(scratch), scratch.numel() * 8,
               N.stream_ptr())
        return grid

    def auto_cell_capacity(self, pos, support, min_coord=None, max_coord=None) -> int:
        """Number of grid cells (one host synchronisation)."""
        status = self.ws.get("status", 1, torch.int32)
        status.zero_()
        g = self.grid(pos, support, min_coord, max_coord, MAX_CELLS)
        info = grid_from_bytes(g)
        flags = int(status.item())
        status.zero_()
        if flags & N.SPH_FLAG_NONFINITE:
            raise N.SPHError("neighbor search: non-finite positions or supports")
        if flags & N.SPH_FLAG_CELL_CAPACITY:
            raise N.SPHError(f"neighbor search: the grid needs more than {MAX_CELLS} cells "
                             f"(domain / support ratio too large for the dense cell table)")
        return max(info["num_cells"], 1)

    def stored_segments(self, n: int) -> int:
        """Segments (start, 32-candidate mask) the last segment search of n particles kept,
        summed over the particles (particles on the dense list count none).  The per-particle
        counts follow the 24 n masks and 24 n starts in the segment scratch."""
        words = self.ws.bytes("segments", N.load().sph_nl_segments_scratch_bytes(n)).view(torch.int32)
        return int(torch.clamp(words[48 * n:49 * n], min=0).sum().item())

    def run(self, pos, support, area=None, kernel_support=None, min_coord=None, max_coord=None,
            search_radius: int = 1, cell_capacity: int | None = None, pair_capacity: int | None = None,
            density: bool = True, sync: bool = True, marks=None) -> CSRNeighbors:
        """One search.  `marks(name)` (optional) is called at each phase boundary, e.g. to
        record CUDA events: "start", "keys", "sort", "gather", "count", "scan", "fill"."""
        lib = N.load()
        mark = marks or (lambda name: None)
        if not (pos.is_cuda and pos.dtype == torch.float32 and pos.dim() == 2 and pos.shape[1] == 2):
            raise N.SPHError("positions must be a float32 CUDA tensor of shape [N, 2]")
        pos = pos.contiguous()
        support = support.contiguous()
        if area is not None:
            area = area.contiguous()
        n = pos.shape[0]
        if n >= (1 << 31) - 1:
            raise N.SPHError("neighbor search: at most 2^31-2 particles")
        st = N.stream_ptr()
        ws = self.ws
        search_radius = int(search_radius) * self.cell_ratio   # in cells of the (finer) grid
        if n == 0:   # no particles: an empty result (no grid to build)
            dev = pos.device
            i32 = lambda m: torch.zeros(m, dtype=torch.int32, device=dev)
            f32 = lambda m: torch.zeros(m, dtype=torch.float32, device=dev)
            return CSRNeighbors(n=0, order=i32(0), keys=i32(0), xy=f32(0).view(0, 2), sh=f32(0),
                                sa=f32(0) if area is not None else None, cell_start=i32(2), counts=i32(0),
                                offsets=i32(1), cols=i32(0), rho=f32(0) if density else None, grid=None,
                                status=i32(1), cell_capacity=0, pair_capacity=0, kernel_support=kernel_support,
                                search_radius=int(search_radius), cell_ratio=self.cell_ratio)
        if cell_capacity is None:
            cell_capacity = self.auto_cell_capacity(pos, support, min_coord, max_coord)
        cap = int(cell_capacity)
        status = ws.get("status", 1, torch.int32)
        status.zero_()
        mark("start")
        grid = self.grid(pos, support, min_coord, max_coord, cap)
        keys = ws.get("keys", n)
        order = ws.get("order", n)
        skeys = ws.get("sorted_keys", n)
        cell_start = ws.get("cell_start", cap + 2)
        if self.sort == "counting":
            cell_count = ws.zeros("cell_count", cap + 1)  # left zeroed by every sort
            N.call("sph_cell_keys", N.ptr(pos), n, N.ptr(grid), cap, N.ptr(keys), None, N.ptr(cell_count),
                   N.ptr(status), st)
            mark("keys")
            cs = ws.bytes("cs_scratch", lib.sph_counting_sort_scratch_bytes(n, cap))
            # positions, supports and areas move into the sorted order in the sort's own launches
            xy = ws.get("xy", 2 * n, torch.float32).view(n, 2)
            sh = ws.get("sorted_support", n, torch.float32)
            sa = ws.get("sorted_area", n, torch.float32) if area is not None else None
            rows = [(pos, xy), (support, sh)] + ([(area, sa)] if area is not None else [])
            k, eb, ins, outs = N.array_set(rows)
            N.call("sph_counting_sort_permute", N.ptr(keys), n, cap, N.ptr(cell_count), N.ptr(cell_start), None,
                   N.ptr(order), N.ptr(skeys), k, eb, ins, outs, N.ptr(status), N.ptr(cs), cs.numel() * 8, st)
        else:
            N.call("sph_cell_keys", N.ptr(pos), n, N.ptr(grid), cap, N.ptr(skeys), N.ptr(order), None,
                   N.ptr(status), st)
            mark("keys")
            rs = ws.bytes("rs_scratch", lib.sph_radix_sort_scratch_bytes(n, self.digit_bits))
            N.call("sph_radix_sort_pairs", N.ptr(skeys), N.ptr(order), n, lib.sph_key_bits(cap), self.digit_bits,
                   N.ptr(rs), rs.numel() * 8, st)
            N.call("sph_cell_starts", N.ptr(skeys), n, cap, N.ptr(cell_start), st)
        mark("sort")
        if self.sort != "counting":
            xy = ws.get("xy", 2 * n, torch.float32).view(n, 2)
            sh = ws.get("sorted_support", n, torch.float32)
            sa = ws.get("sorted_area", n, torch.float32) if area is not None else None
            N.call("sph_gather_sorted", N.ptr(order), n, N.ptr(pos), N.ptr(support), N.ptr(area), N.ptr(xy),
                   N.ptr(sh), N.ptr(sa), st)
        mark("gather")
        counts = ws.get("counts", n)
        rho = ws.get("rho", n, torch.float32) if density else None
        ks = float(kernel_support) if kernel_support is not None else 0.0
        if density and (ks <= 0 or area is None):
            raise N.SPHError("neighbor search: density needs kernel_support > 0 and areas")
        if self.segments:   # one candidate test per pair: the fill expands the stored masks
            seg = ws.bytes("segments", lib.sph_nl_segments_scratch_bytes(n))
            N.call("sph_nl_count_segments", N.ptr(xy), N.ptr(sh), N.ptr(sa), n, N.ptr(skeys), N.ptr(cell_start),
                   N.ptr(grid), cap, int(search_radius), ks, N.ptr(counts), N.ptr(rho), N.ptr(seg), seg.numel() * 8,
                   st)
        else:
            N.call("sph_nl_count", N.ptr(xy), N.ptr(sh), N.ptr(sa), n, N.ptr(skeys), N.ptr(cell_start), N.ptr(grid),
                   cap, int(search_radius), ks, N.ptr(counts), N.ptr(rho), st)
        mark("count")
        offsets = ws.get("offsets", n + 1)
        sc = ws.bytes("scan_scratch", lib.sph_scan_scratch_bytes(n))
        N.call("sph_exclusive_scan_i32", N.ptr(counts), N.ptr(offsets), n, N.ptr(sc), sc.numel() * 8, st)
        mark("scan")
        if pair_capacity is None:
            pair_capacity = int(offsets[n].item())
        cols = ws.get("cols", pair_capacity)
        if self.segments:
            N.call("sph_nl_fill_segments", N.ptr(xy), N.ptr(sh), n, N.ptr(skeys), N.ptr(cell_start), N.ptr(grid), cap,
                   int(search_radius), N.ptr(offsets), int(pair_capacity), N.ptr(cols), N.ptr(status), N.ptr(seg),
                   seg.numel() * 8, st)
        else:
            N.call("sph_nl_fill", N.ptr(xy), N.ptr(sh), n, N.ptr(skeys), N.ptr(cell_start), N.ptr(grid), cap,
                   int(search_radius), N.ptr(offsets), int(pair_capacity), N.ptr(cols), N.ptr(status), st)
        mark("fill")
        res = CSRNeighbors(n=n, order=order, keys=skeys, xy=xy, sh=sh, sa=sa, cell_start=cell_start, counts=counts,
                           offsets=offsets, cols=cols, rho=rho, grid=grid, status=status, cell_capacity=cap,
                           pair_capacity=int(pair_capacity), kernel_support=kernel_support,
                           search_radius=int(search_radius), cell_ratio=self.cell_ratio)
        if sync:
            res.check()
        return res


def next_prime(n: int) -> int:
    """Smallest prime > n (sympy.nextprime semantics, src/modules/neighborSearch.py:95)."""
    def is_prime(k):
        if k < 2:
            return False
        if k % 2 == 0:
            return k == 2
        r = int(math.isqrt(k))
        f = 3
        while f <= r:
            if k % f == 0:
                return False
            f += 2
        return True
    k = n + 1
    while not is_prime(k):
        k += 1
    return k
