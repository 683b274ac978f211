"""ORACLE — test infrastructure only.  Python front end of `oracle/nsearch_oracle.c`.

The C file is a plain restatement of the reference's neighbor search (sortPositions,
constructHashMap, buildNeighborList*, src/modules/neighborSearch.py:30-171 and
cppSrc/neighSearch.cpp:93-410) and density summation (src/modules/density.py:26-30).
Only the tests, `__graft_entry__.smoke()` and bench.py's CPU-baseline leg use it, as the
checker; the product never imports it.

`build()` compiles the C file with gcc into `oracle/_build/` (plain C + OpenMP, no
architecture-specific flags, -ffp-contract=off) so it builds on x86-64 and aarch64.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nsearch_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libnsearch_oracle.so")

PRED_FMA_XX, PRED_FMA_YY, PRED_UNFUSED, PRED_DOUBLE_SQRT = 0, 1, 2, 3

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               SRC, "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        i64, i32, f32, c_int = ctypes.c_int64, ctypes.c_int32, ctypes.c_float, ctypes.c_int
        _lib.oracle_sort_positions.argtypes = [P, P, i64, P, P, P, P, P, P, P]
        _lib.oracle_sort_positions.restype = c_int
        _lib.oracle_hash_map.argtypes = [P, i64, i32, i32, P, P, P, P]
        _lib.oracle_hash_map.restype = i64
        _lib.oracle_nl_cells.argtypes = [P, P, P, P, P, P, P, i64, i32, i32, i32, c_int, c_int, P, P]
        _lib.oracle_nl_cells.restype = i64
        _lib.oracle_nl_query.argtypes = [P, P, i64, P, P, P, P, P, P, i32, i32, P, f32, i32, c_int,
                                         c_int, P, P]
        _lib.oracle_nl_query.restype = i64
        _lib.oracle_nl_asym.argtypes = [P, P, P, P, P, P, P, i64, P, P, P, P, P, P, i32, i32, c_int,
                                        c_int, P, P]
        _lib.oracle_nl_asym.restype = i64
        _lib.oracle_canonical_csr.argtypes = [P, P, i64, i64, P, P]
        _lib.oracle_canonical_csr.restype = c_int
        _lib.oracle_density.argtypes = [P, P, i64, P, P, f32, c_int, P]
        _lib.oracle_density.restype = c_int
        _lib.oracle_free.argtypes = [P]
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def next_prime(n: int) -> int:
    """Smallest prime > n (sympy.nextprime semantics, src/modules/neighborSearch.py:95)."""
    def is_prime(k):
        if k < 2:
            return False
        if k % 2 == 0:
            return k == 2
        f = 3
        while f * f <= k:
            if k % f == 0:
                return False
            f += 2
        return True
    k = n + 1
    while not is_prime(k):
        k += 1
    return k


class SortInfo:
    """What sortPositions + constructHashMap produce (src/modules/neighborSearch.py:30-88)."""

    def __init__(self, pos, h, min_coord=None, max_coord=None, hash_len=-1):
        L = lib()
        pos = _c(pos, np.float32)
        h = _c(h, np.float32)
        n = pos.shape[0]
        self.n = n
        self.qmin = np.zeros(2, np.float32)
        hmax = np.zeros(1, np.float32)
        cells = np.zeros(2, np.int32)
        lin = np.zeros(n, np.int32)
        order = np.zeros(n, np.int64)
        mn = _c(min_coord, np.float32) if min_coord is not None else None
        mx = _c(max_coord, np.float32) if max_coord is not None else None
        rc = L.oracle_sort_positions(_p(pos), _p(h), n, _p(mn), _p(mx), _p(self.qmin), _p(hmax),
                                     _p(cells), _p(lin), _p(order))
        if rc != 0:
            raise RuntimeError("oracle_sort_positions failed")
        self.hmax = float(hmax[0])
        self.cells = cells
        self.cells_x = int(cells[0])
        self.order = order
        self.sort = order.astype(np.int32)
        self.sorted_lin = lin[order]
        self.sorted_pos = np.ascontiguousarray(pos[order])
        self.sorted_h = np.ascontiguousarray(h[order])
        self.hash_len = next_prime(n) if hash_len == -1 else int(hash_len)
        self.table = np.zeros((self.hash_len, 2), np.int32)
        ci = np.zeros(n, np.int32)
        cc = np.zeros(n, np.int32)
        cs = np.zeros(n, np.int32)
        C = L.oracle_hash_map(_p(self.sorted_lin), n, self.cells_x, self.hash_len, _p(self.table),
                              _p(ci), _p(cc), _p(cs))
        if C < 0:
            raise RuntimeError("oracle_hash_map failed")
        self.cell_indices, self.cum_cell, self.cell_span = ci[:C].copy(), cc[:C].copy(), cs[:C].copy()


def _take_pairs(L, rows_p, cols_p, P):
    if P < 0:
        raise RuntimeError("oracle neighbor list failed")
    rows = np.ctypeslib.as_array(ctypes.cast(rows_p, ctypes.POINTER(ctypes.c_int32)), (max(P, 1),))[:P].copy()
    cols = np.ctypeslib.as_array(ctypes.cast(cols_p, ctypes.POINTER(ctypes.c_int32)), (max(P, 1),))[:P].copy()
    L.oracle_free(rows_p)
    L.oracle_free(cols_p)
    return rows, cols


def nl_cells(si: SortInfo, radius: int = 1, pred: int = PRED_FMA_XX, threads: int = 0):
    """buildNeighborList restated: (rows, cols) int32 original indices, reference order per thread."""
    L = lib()
    rp, cp = ctypes.c_void_p(), ctypes.c_void_p()
    P = L.oracle_nl_cells(_p(si.sorted_pos), _p(si.sorted_h), _p(si.table), _p(si.cell_indices),
                          _p(si.cum_cell), _p(si.cell_span), _p(si.sort), len(si.cell_indices),
                          si.cells_x, si.hash_len, radius, pred, threads, ctypes.byref(rp), ctypes.byref(cp))
    return _take_pairs(L, rp, cp, P)


def nl_query(si: SortInfo, qpos, qh, radius: int = 1, pred: int = PRED_FMA_XX, threads: int = 0):
    """buildNeighborListUnsortedPerParticle restated: rows = query index, cols = original index."""
    L = lib()
    qpos = _c(qpos, np.float32)
    qh = _c(qh, np.float32)
    rp, cp = ctypes.c_void_p(), ctypes.c_void_p()
    P = L.oracle_nl_query(_p(qpos), _p(qh), qpos.shape[0], _p(si.sorted_pos), _p(si.table),
                          _p(si.cell_indices), _p(si.cum_cell), _p(si.cell_span), _p(si.sort),
                          si.cells_x, si.hash_len, _p(si.qmin), si.hmax, radius, pred, threads,
                          ctypes.byref(rp), ctypes.byref(cp))
    return _take_pairs(L, rp, cp, P)


def nl_asym(a: SortInfo, b: SortInfo, pred: int = PRED_FMA_XX, threads: int = 0):
    """buildNeighborListAsymmetric restated (both grids must share cellsX and the table length)."""
    L = lib()
    rp, cp = ctypes.c_void_p(), ctypes.c_void_p()
    P = L.oracle_nl_asym(_p(a.sorted_pos), _p(a.sorted_h), _p(a.table), _p(a.cell_indices),
                         _p(a.cum_cell), _p(a.cell_span), _p(a.sort), len(a.cell_indices),
                         _p(b.sorted_pos), _p(b.table), _p(b.cell_indices), _p(b.cum_cell),
                         _p(b.cell_span), _p(b.sort), a.cells_x, a.hash_len, pred, threads,
                         ctypes.byref(rp), ctypes.byref(cp))
    return _take_pairs(L, rp, cp, P)


def canonical_csr(rows, cols, n_rows):
    """(offsets int64 [n_rows+1], cols int32 [P]) with columns ascending within each row."""
    L = lib()
    rows = _c(rows, np.int32)
    cols = _c(cols, np.int32)
    P = rows.shape[0]
    offsets = np.zeros(n_rows + 1, np.int64)
    out = np.zeros(max(P, 1), np.int32)
    if L.oracle_canonical_csr(_p(rows), _p(cols), P, n_rows, _p(offsets), _p(out)) != 0:
        raise RuntimeError("row index out of range")
    return offsets, out[:P]


def density(offsets, cols, pos, area, support, use_double=False):
    L = lib()
    pos = _c(pos, np.float32)
    area = _c(area, np.float32)
    n = pos.shape[0]
    out = np.zeros(n, np.float64)
    L.oracle_density(_p(_c(offsets, np.int64)), _p(_c(cols, np.int32)), n, _p(pos), _p(area),
                     float(support), int(use_double), _p(out))
    return out if use_double else out.astype(np.float32)


def search(pos, h, min_coord=None, max_coord=None, hash_len=-1, radius=1, pred=PRED_FMA_XX, threads=0):
    """Full fluid search as src/modules/neighborSearch.py:91-116 does it; canonical CSR result."""
    si = SortInfo(pos, h, min_coord, max_coord, hash_len)
    rows, cols = nl_cells(si, radius, pred, threads)
    offsets, c = canonical_csr(rows, cols, si.n)
    return si, offsets, c
