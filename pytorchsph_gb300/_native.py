"""ctypes binding of the C ABI in include/sph_gb300.h (libsph_gb300.so).

The product path has no CPU fallback: if the library is missing or no CUDA device is
present, every entry point raises.  Torch tensors are passed as raw device pointers
(`tensor.data_ptr()`), and work is issued on torch's current CUDA stream so that torch
allocations, CUDA graphs and the library's kernels share one ordering.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import build as _build

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_F32 = ctypes.c_float
_SZ = ctypes.c_size_t

# name -> (restype, argtypes); mirrors include/sph_gb300.h
SIGNATURES = {
    "sph_abi_version": (_I32, []),
    "sph_last_error": (ctypes.c_char_p, []),
    "sph_status_string": (ctypes.c_char_p, [_I32]),
    "sph_scan_scratch_bytes": (_SZ, [_I64]),
    "sph_exclusive_scan_i32": (_I32, [_P, _P, _I64, _P, _SZ, _P]),
    "sph_exclusive_scan_i32_to_i64": (_I32, [_P, _P, _I64, _P, _SZ, _P]),
    "sph_scan_timeouts": (ctypes.c_uint64, []),
    "sph_exclusive_scan_i32_static_max_items": (_I64, []),
    "sph_exclusive_scan_i32_static": (_I32, [_P, _P, _I64, _P]),
    "sph_radix_sort_scratch_bytes": (_SZ, [_I64, _I32]),
    "sph_radix_sort_pairs": (_I32, [_P, _P, _I64, _I32, _I32, _P, _SZ, _P]),
    "sph_grid_scratch_bytes": (_SZ, [_I64]),
    "sph_grid_build": (_I32, [_P, _P, _I64, _P, _P, _I32, _P, _P, _P, _SZ, _P]),
    "sph_grid_build_ratio": (_I32, [_P, _P, _I64, _P, _P, _I32, _I32, _P, _P, _P, _SZ, _P]),
    "sph_grid_build_segments": (_I32, [_P, _P, _P, _I32, _P, _P, _I32, _P, _P, _P]),
    "sph_cell_keys": (_I32, [_P, _I64, _P, _I32, _P, _P, _P, _P, _P]),
    "sph_counting_sort_scratch_bytes": (_SZ, [_I64, _I32]),
    "sph_counting_sort": (_I32, [_P, _I64, _I32, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "sph_key_bits": (_I32, [_I32]),
    "sph_cell_starts": (_I32, [_P, _I64, _I32, _P, _P]),
    "sph_gather_sorted": (_I32, [_P, _I64, _P, _P, _P, _P, _P, _P, _P]),
    "sph_hash_map_scratch_bytes": (_SZ, [_I64, _I32]),
    "sph_hash_map_build": (_I32, [_P, _I64, _I32, _I32, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "sph_nl_count": (_I32, [_P, _P, _P, _I64, _P, _P, _P, _I32, _I32, _F32, _P, _P, _P]),
    "sph_nl_fill": (_I32, [_P, _P, _I64, _P, _P, _P, _I32, _I32, _P, _I64, _P, _P, _P]),
    "sph_nl_segments_scratch_bytes": (_SZ, [_I64]),
    "sph_nl_count_segments": (_I32, [_P, _P, _P, _I64, _P, _P, _P, _I32, _I32, _F32, _P, _P, _P, _SZ, _P]),
    "sph_nl_fill_segments": (_I32, [_P, _P, _I64, _P, _P, _P, _I32, _I32, _P, _I64, _P, _P, _P, _SZ, _P]),
    "sph_scatter_f32": (_I32, [_P, _P, _I64, _P, _P]),
    "sph_nl_to_coo": (_I32, [_P, _I64, _P, _P, _P, _P, _P, _F32, _F32, _P, _I64, _P, _P, _P]),
    "sph_scatter_counts": (_I32, [_P, _P, _I64, _P, _P]),
    "sph_invert_permutation": (_I32, [_P, _I64, _P, _P]),
    "sph_nl_query_count": (_I32, [_P, _P, _I64, _P, _P, _P, _I32, _I32, _P, _P]),
    "sph_nl_query_fill": (_I32, [_P, _P, _I64, _P, _P, _P, _I32, _I32, _P, _P, _P, _P, _P]),
    "sph_nl_hashed_query_count": (_I32, [_P, _P, _I64, _P, _P, _P, _P, _P, _P, _F32, _I32, _I32, _I32, _P, _P]),
    "sph_nl_hashed_query_fill": (_I32, [_P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _F32, _I32, _I32, _I32, _P,
                                        _P, _P, _P]),
    "sph_nl_hashed_cells_count": (_I32, [_P, _P, _P, _P, _P, _P, _I64, _I32, _I32, _I32, _P, _P]),
    "sph_nl_hashed_cells_fill": (_I32, [_P, _P, _P, _P, _P, _P, _P, _I64, _I32, _I32, _I32, _P, _P, _P, _P]),
    "sph_nl_hashed_asym_count": (_I32, [_P, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _I32, _I32, _P, _P]),
    "sph_nl_hashed_asym_fill": (_I32, [_P, _P, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _I32, _I32, _P,
                                       _P, _P, _P]),
}

SIGNATURES.update({  # batch of scenes
    "sph_counting_sort_tie": (_I32, [_P, _I64, _I32, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "sph_counting_sort_permute": (_I32, [_P, _I64, _I32, _P, _P, _P, _P, _P, _I32, _P, _P, _P, _P, _P, _SZ, _P]),
    "sph_scene_bytes": (_SZ, []),
    "sph_scene_encode": (_I32, [_P, _P, _I32, _F32, _P]),
    "sph_batch_cell_keys": (_I32, [_P, _I64, _P, _P, _I32, _P, _P, _P, _P]),
    "sph_batch_nl_count": (_I32, [_P, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "sph_batch_nl_fill": (_I32, [_P, _P, _I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P]),
    "sph_batch_deltasph_step": (_I32, [_P] * 8 + [_I32] + [_P] * 4 + [_I32, _I32, _P, _P, _SZ, _P]),
})

SIGNATURES.update({  # Module-interface terms
    "sph_pair_term": (_I32, [_I32, _P, _P, _P, _I32, _P]),
    "sph_particle_op": (_I32, [_I32, _I64, _P, _P, _P, _P, _I32, _P]),
    "sph_row_offsets": (_I32, [_P, _I64, _I64, _P, _P]),
    "sph_wall_term": (_I32, [_I32, _P, _P, _P, _I32, _P]),
    "sph_transpose_pairs_scratch_bytes": (_SZ, [_I64]),
    "sph_transpose_pairs": (_I32, [_P, _I64, _I64, _P, _P, _P, _SZ, _P]),
    "sph_surface_scratch_bytes": (_SZ, []),
    "sph_arena_set_ids": (_I32, [_P, _P, _I64, _I64, _I32, _P]),
    "sph_arena_extract": (_I32, [_P, _P, _P, _P, _P, _I64, _I32, _P, _P, _P, _P]),
    "sph_arena_extract_many": (_I32, [_P, _P, _P, _P, _P, _I64, _P, _P, _I32, _P, _P, _P, _I32, _P]),
    "sph_arena_retire": (_I32, [_P, _I64, _I32, _P]),
    "sph_periodic_ghosts_scratch_bytes": (_SZ, [_I64]),
    "sph_periodic_ghosts": (_I32, [_P, _I64, _P, _P, _F32, _I32, _I32, _I64, _P, _P, _P, _P, _P, _SZ, _P]),
    "sph_nl_periodic_scratch_bytes": (_SZ, [_I64, _P, _P, _F32]),
    "sph_nl_periodic_count": (_I32, [_P, _P, _I64, _P, _P, _F32, _I32, _I32, _P, _P, _P, _SZ, _P]),
    "sph_nl_periodic_fill": (_I32, [_P, _P, _I64, _P, _P, _F32, _I32, _I32, _P, _I64, _P, _P, _P, _P, _P, _SZ, _P]),
    "sph_surface_term": (_I32, [_I32, _P, _P, _P, _P, _P]),
    "sph_pair_geometry": (_I32, [_P, _P, _I64, _P, _P, _P, _F32, _P, _P, _P]),
})

_D = ctypes.c_double
SIGNATURES.update({  # differentiable rollouts
    "sph_drop_rhs": (_I32, [_I32, _I64] + [_P] * 9 + [_P]),
    "sph_drop_integrate": (_I32, [_I32, _I64] + [_P] * 5 + [_D, _D, _P]),
    "sph_drop_adjoint": (_I32, [_I32, _I64] + [_P] * 7 + [_D] + [_P] * 8),
})

SIGNATURES.update({  # simulation kernels
    "sph_mdbc_wall_density": (_I32, [_P] * 5),
    "sph_deltasph_scratch_bytes": (_SZ, [_I64]),
    "sph_deltasph_segment_lists": (_I32, [_I64, _P, _P, _P, _P]),
    "sph_deltasph_forces": (_I32, [_P] * 8 + [_P, _SZ, _P]),
    "sph_integrate_semi_implicit_euler": (_I32, [_I64] + [_P] * 6 +
                                          [_F32, _I32] + [_P] * 5),
    "sph_rk_axpy": (_I32, [_I64] + [_P] * 7 + [_F32, _F32] +
                    [_P] * 5),
    "sph_rk_accumulate": (_I32, [_I64] + [_P] * 3 + [_F32, _I32] +
                          [_P] * 4),
    "sph_permute": (_I32, [_P, _I64, _I32] + [_P] * 3),
    "sph_permute_arrays": (_I32, [_P, _I64, _I32, _P, _P, _P, _P]),
    "sph_dfsph_partials_count": (_SZ, []),
    "sph_dfsph_wall_wall_term": (_I32, [_P] * 5),
    "sph_dfsph_densities": (_I32, [_P] * 7),
    "sph_dfsph_solve": (_I32, [_P] * 7 + [_I32] + [_P] * 2),
    "sph_dfsph_viscosity": (_I32, [_P] * 7),
    "sph_add_float2": (_I32, [_I64, _P, _P, _P]),
    "sph_fill_float2": (_I32, [_I64, _F32, _F32, _P,
                                         _P]),
    "sph_dt_scratch_bytes": (_SZ, []),
    "sph_update_dt": (_I32, [_I64] + [_P] * 2 + [_F32] * 4 +
                      [_I32, _F32, _F32] + [_P] * 2 +
                      [_SZ, _P]),
})

SPH_PHASE_WALLS, SPH_PHASE_RECORDS, SPH_PHASE_PASS1, SPH_PHASE_DIFFUSION, SPH_PHASE_ALL = 1, 2, 4, 8, 15

SPH_FLAG_OUT_OF_GRID = 1
SPH_FLAG_NONFINITE = 2
SPH_FLAG_PAIR_CAPACITY = 4
SPH_FLAG_CELL_CAPACITY = 8
SPH_FLAG_ITERATION_CAP = 16
SPH_FLAG_CELL_ORDER = 32

FLAG_NAMES = {
    SPH_FLAG_OUT_OF_GRID: "a particle lies outside the search grid",
    SPH_FLAG_NONFINITE: "non-finite value (NaN/Inf) in positions or results",
    SPH_FLAG_PAIR_CAPACITY: "neighbor pair buffer too small",
    SPH_FLAG_CELL_CAPACITY: "search grid has more cells than the cell table holds",
    SPH_FLAG_ITERATION_CAP: "an iterative solve stopped at its maximum iteration count",
    SPH_FLAG_CELL_ORDER: "a cell held more than 2048 particles; their order inside the cell is not reproducible",
}

_lib = None
_lock = threading.Lock()


class SPHError(RuntimeError):
    """Raised when a GB300 kernel reports a failure (the reference raises RuntimeError too)."""


def library_path() -> str:
    return _build.LIB_PATH


def load(require_cuda: bool = True):
    """Load libsph_gb300.so; raises if it is missing (no CPU fallback exists)."""
    global _lib
    if require_cuda and not torch.cuda.is_available():
        raise SPHError("pytorchsph_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU path")
    with _lock:
        if _lib is None:
            path = library_path()
            if not os.path.exists(path):
                raise SPHError(f"GB300 library not built: {path} is missing; run pytorchsph_gb300.build.build()")
            lib = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(status: int, what: str = ""):
    if status != 0:
        lib = load(require_cuda=False)
        msg = lib.sph_last_error().decode(errors="replace")
        kind = lib.sph_status_string(status).decode()
        raise SPHError(f"{what}: {kind}: {msg}")


def call(name: str, *args):
    fn = getattr(load(), name)
    check(fn(*args), name)


def ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def array_set(pairs):
    """(count, row bytes, in pointers, out pointers) of (in, out) tensor pairs of per-particle
    rows, as the C ABI's array-set arguments take them."""
    k = len(pairs)
    row = lambda t: t.element_size() * (t.shape[1] if t.dim() == 2 else 1)
    eb = (ctypes.c_int32 * k)(*[row(t) for t, _ in pairs])
    ins = (ctypes.c_void_p * k)(*[t.data_ptr() for t, _ in pairs])
    outs = (ctypes.c_void_p * k)(*[o.data_ptr() for _, o in pairs])
    return k, eb, ins, outs


def permute_arrays(order, pairs):
    """out[s] = in[order[s]] (a copy when order is None) for up to 8 (in, out) tensor pairs
    of per-particle rows, in one kernel (sph_permute_arrays)."""
    n = pairs[0][0].shape[0] if pairs else 0
    k, eb, ins, outs = array_set(pairs)
    call("sph_permute_arrays", ptr(order), n, k, eb, ins, outs, stream_ptr())


def decode_flags(flags: int) -> str:
    return "; ".join(msg for bit, msg in FLAG_NAMES.items() if flags & bit) or "ok"
