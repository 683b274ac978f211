"""The allocation-free scan entry point, sph_exclusive_scan_i32_static.

Some callers of this library cannot allocate device memory: a host runtime that reaches
the kernels through the C ABI from another language and only receives device pointers from
whoever owns the GPU memory, or a server whose device-memory budget is reserved in full up
front.  For them the scan keeps its tile words in a fixed 64 KiB device array inside the
library instead of caller-provided scratch.  This test calls it through the C ABI and checks
it against the scratch-taking sph_exclusive_scan_i32 (an integer scan: results must be
identical) on calls in a row that reuse the shared array, checks that no look-back wait
gave up, and checks that sizes beyond the fixed array are refused.  The file sorts last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _scan_with_scratch(N, x, n):
    lib = N.load()
    out = torch.empty(n + 1, dtype=torch.int32, device=x.device)
    scratch = torch.empty((lib.sph_scan_scratch_bytes(n) + 7) // 8, dtype=torch.int64, device=x.device)
    N.call("sph_exclusive_scan_i32", N.ptr(x), N.ptr(out), n, N.ptr(scratch), scratch.numel() * 8, N.stream_ptr())
    return out


def test_static_scan_matches_scratch_scan(cuda):
    from pytorchsph_gb300 import _native as N
    lib = N.load()
    g = torch.Generator().manual_seed(1234)
    cases = [1_000_003, 7 * 4096 + 5, 1_000_003, 1]
    timeouts_before = lib.sph_scan_timeouts()
    for n in cases:
        x = torch.randint(0, 97, (n,), generator=g, dtype=torch.int32).to(cuda)
        ref = _scan_with_scratch(N, x, n)
        out = torch.full((n + 1,), -7, dtype=torch.int32, device=cuda)
        status = lib.sph_exclusive_scan_i32_static(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                                   ctypes.c_int64(n), ctypes.c_void_p(N.stream_ptr()))
        assert status == 0, lib.sph_last_error()
        torch.cuda.synchronize()
        assert torch.equal(out, ref), n
        assert int(out[n]) == int(x.sum())
    # every call in a row found the shared tile words in a usable state: no look-back wait
    # ran out (a wait that gave up would count here even if its output happened to be right)
    assert lib.sph_scan_timeouts() == timeouts_before


def test_static_scan_refuses_oversize(cuda):
    from pytorchsph_gb300 import _native as N
    lib = N.load()
    cap = lib.sph_exclusive_scan_i32_static_max_items()
    assert cap == (8192 - 1) * 4096
    x = torch.zeros(4, dtype=torch.int32, device=cuda)
    status = lib.sph_exclusive_scan_i32_static(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                               ctypes.c_int64(cap + 1), ctypes.c_void_p(N.stream_ptr()))
    assert status == 1  # SPH_ERR_INVALID_ARGUMENT, nothing launched
    assert b"exceeds the fixed scratch" in lib.sph_last_error()
    # the largest accepted size works
    n = cap
    y = torch.ones(n, dtype=torch.int32, device=cuda)
    out = torch.empty(n + 1, dtype=torch.int32, device=cuda)
    assert lib.sph_exclusive_scan_i32_static(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_int64(n), ctypes.c_void_p(N.stream_ptr())) == 0
    torch.cuda.synchronize()
    assert int(out[n]) == n and int(out[12345]) == 12345
