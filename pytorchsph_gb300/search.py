"""Native GB300 neighbor search: cell keys -> radix sort -> sorted SoA -> cell table ->
two-pass CSR (count with fused density, scan, fill).

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

    def bytes(self, name, nbytes):
        return self.get(name, (int(nbytes) + 7) // 8, torch.int64)


def grid_from_bytes(t: torch.Tensor) -> dict:
    """Decode an sph_grid struct read back to the host."""
    raw = t.detach().cpu()
    f = raw[:4].view(torch.float32) if raw.dtype == torch.int32 else None
    f = raw.view(torch.int32)[:4].view(torch.float32)
    i = raw.view(torch.int32)[4:8]
    return {"qmin": (float(f[0]), float(f[1])), "hmax": float(f[2]), "cells_x": int(i[0]),
            "cells_y": int(i[1]), "num_cells": int(i[2])}


class CSRNeighbors:
    """Result of one search: sorted SoA, cell table and CSR pairs (all on the device)."""

    def __init__(self, n, order, keys, packed, cell_start, counts, offsets, cols, rho, grid, status,
                 cell_capacity, pair_capacity, kernel_support, search_radius):
        self.n = n
        self.order = order          # int32 [n]: original index of sorted particle s
        self.keys = keys            # int32 [n]: sorted cell keys
        self.packed = packed        # float32 [n, 4]: (x, y, support, area) in sorted order
        self.cell_start = cell_start
        self.counts = counts        # int32 [n]
        self.offsets = offsets      # int32 [n+1]
        self.cols = cols            # int32 [pair_capacity]
        self.rho = rho              # float32 [n] (sorted order) or None
        self.grid = grid            # int32 [8] device bytes of sph_grid
        self.status = status        # int32 [1] device status word
        self.cell_capacity = cell_capacity
        self.pair_capacity = pair_capacity
        self.kernel_support = kernel_support
        self.search_radius = search_radius
        self._rank = None

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

    def density(self) -> torch.Tensor:
        """rho in original particle order."""
        out = torch.empty(self.n, dtype=torch.float32, device=self.order.device)
        N.call("sph_scatter_f32", N.ptr(self.order), N.ptr(self.rho), self.n, N.ptr(out), N.stream_ptr())
        return out

    def to_coo(self, grad_threshold: float = 1e-7, distances: bool = True):
        """(fluidNeighbors int64 [2,P], fluidDistances [P,2], fluidRadialDistances [P]) in the
        reference layout (src/modules/neighborSearch.py:216-227), pairs ordered by (i, j)."""
        self.check()
        P = self.num_pairs
        dev = self.order.device
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
        N.call("sph_nl_to_coo", N.ptr(self.packed), self.n, N.ptr(self.order), N.ptr(self.rank),
               N.ptr(self.offsets), N.ptr(self.cols), N.ptr(orig_off), float(grad_threshold),
               float(self.kernel_support or 1.0), N.ptr(pairs), P, N.ptr(dist), N.ptr(radial), st)
        return pairs, dist, radial


class GridSearch:
    """Hashed-grid neighbor search with CSR output, reusing its device workspace."""

    def __init__(self, device=None, digit_bits: int = 8, threads_per_particle: int = 1):
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self.ws = Workspace(self.device)
        self.digit_bits = int(digit_bits)
        self.threads_per_particle = int(threads_per_particle)

    def grid(self, pos, support, min_coord=None, max_coord=None, cell_capacity=(1 << 31) - 2):
        """Compute the search grid on the device; returns the device grid bytes."""
        lib = N.load()
        n = pos.shape[0]
        grid = self.ws.get("grid", 8, torch.int32)
        status = self.ws.get("status", 1, torch.int32)
        scratch_b = lib.sph_grid_scratch_bytes(n)
        scratch = self.ws.bytes("grid_scratch", scratch_b)
        mn = (ctypes_f2(min_coord) if min_coord is not None else None)
        mx = (ctypes_f2(max_coord) if max_coord is not None else None)
        N.call("sph_grid_build", N.ptr(pos), N.ptr(support), n, mn, mx, int(cell_capacity), N.ptr(grid),
               N.ptr(status), N.ptr(scratch), scratch.numel() * 8, N.stream_ptr())
        return grid

    def run(self, pos, support, area=None, kernel_support=None, min_coord=None, max_coord=None,
            search_radius: int = 1, cell_capacity: int | None = None, pair_capacity: int | None = None,
            density: bool = True, sync: bool = True) -> CSRNeighbors:
        lib = N.load()
        assert pos.is_cuda and pos.dtype == torch.float32 and pos.dim() == 2 and pos.shape[1] == 2
        pos = pos.contiguous()
        support = support.contiguous()
        n = pos.shape[0]
        if n >= (1 << 31) - 1:
            raise N.SPHError("neighbor search: at most 2^31-2 particles")
        st = N.stream_ptr()
        ws = self.ws
        status = ws.get("status", 1, torch.int32)
        status.zero_()
        if cell_capacity is None:
            g = self.grid(pos, support, min_coord, max_coord, MAX_CELLS)
            info = grid_from_bytes(g)
            flags = int(status.item())
            if flags & N.SPH_FLAG_NONFINITE:
                raise N.SPHError("neighbor search: non-finite positions or supports")
            if flags & N.SPH_FLAG_CELL_CAPACITY:
                raise N.SPHError(f"neighbor search: the grid needs more than {MAX_CELLS} cells "
                                 f"(domain / support ratio too large for the dense cell table)")
            cell_capacity = max(info["num_cells"], 1)
            status.zero_()
        grid = self.grid(pos, support, min_coord, max_coord, cell_capacity)
        keys = ws.get("keys", n)
        order = ws.get("order", n)
        N.call("sph_cell_keys", N.ptr(pos), n, N.ptr(grid), int(cell_capacity), N.ptr(keys), N.ptr(order),
               N.ptr(status), st)
        kb = lib.sph_key_bits(int(cell_capacity))
        rs_b = lib.sph_radix_sort_scratch_bytes(n, self.digit_bits)
        rs = ws.bytes("rs_scratch", rs_b)
        N.call("sph_radix_sort_pairs", N.ptr(keys), N.ptr(order), n, kb, self.digit_bits, N.ptr(rs), rs.numel() * 8, st)
        packed = ws.get("packed", 4 * n, torch.float32).view(n, 4)
        N.call("sph_gather_packed", N.ptr(order), n, N.ptr(pos), N.ptr(support), N.ptr(area), N.ptr(packed), st)
        cell_start = ws.get("cell_start", cell_capacity + 1)
        N.call("sph_cell_starts", N.ptr(keys), n, int(cell_capacity), N.ptr(cell_start), st)
        counts = ws.get("counts", n)
        rho = ws.get("rho", n, torch.float32) if density else None
        ks = float(kernel_support) if kernel_support is not None else 0.0
        if density and ks <= 0:
            raise N.SPHError("neighbor search: density needs kernel_support > 0")
        N.call("sph_nl_count", N.ptr(packed), n, N.ptr(keys), N.ptr(cell_start), N.ptr(grid), int(cell_capacity),
               int(search_radius), ks, N.ptr(counts), N.ptr(rho), st)
        offsets = ws.get("offsets", n + 1)
        sc_b = lib.sph_scan_scratch_bytes(n)
        sc = ws.bytes("scan_scratch", sc_b)
        N.call("sph_exclusive_scan_i32", N.ptr(counts), N.ptr(offsets), n, N.ptr(sc), sc.numel() * 8, st)
        if pair_capacity is None:
            pair_capacity = int(offsets[n].item())
        cols = ws.get("cols", pair_capacity)
        N.call("sph_nl_fill", N.ptr(packed), n, N.ptr(keys), N.ptr(cell_start), N.ptr(grid), int(cell_capacity),
               int(search_radius), N.ptr(offsets), int(pair_capacity), N.ptr(cols), N.ptr(status), st)
        res = CSRNeighbors(n, order, keys, packed, cell_start, counts, offsets, cols, rho, grid, status,
                           cell_capacity, pair_capacity, kernel_support, search_radius)
        if sync:
            res.check()
        return res


def ctypes_f2(v):
    import ctypes
    arr = (ctypes.c_float * 2)(float(v[0]), float(v[1]))
    return ctypes.cast(arr, ctypes.c_void_p)


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
