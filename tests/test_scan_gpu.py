"""The exclusive scans of the C ABI against torch.cumsum at sizes around the one-block
path's limit (4 tiles of 4096) and the tile size, int32 and int64 outputs; the
single-pass look-back scan above that limit with negative items, unaligned scratch, input
and output pointers, replays of a captured CUDA graph, and no look-back wait that gave up."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 5, 4095, 4096, 4097, 8191, 8192, 8193, 3 * 4096 + 7, 16384, 16385, 65537, 300_001])
def test_exclusive_scans_match_cumsum(cuda, n):
    from pytorchsph_gb300 import _native as N
    lib = N.load()
    g = torch.Generator().manual_seed(n)
    x = torch.randint(0, 1000, (n,), generator=g, dtype=torch.int32).to(cuda)
    ref = torch.cat([torch.zeros(1, dtype=torch.int64, device=cuda), torch.cumsum(x.long(), 0)])
    scratch = torch.empty((lib.sph_scan_scratch_bytes(n) + 7) // 8, dtype=torch.int64, device=cuda)
    o32 = torch.full((n + 1,), -1, dtype=torch.int32, device=cuda)
    N.call("sph_exclusive_scan_i32", N.ptr(x), N.ptr(o32), n, N.ptr(scratch), scratch.numel() * 8, N.stream_ptr())
    o64 = torch.full((n + 1,), -1, dtype=torch.int64, device=cuda)
    N.call("sph_exclusive_scan_i32_to_i64", N.ptr(x), N.ptr(o64), n, N.ptr(scratch), scratch.numel() * 8,
           N.stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(o64, ref)
    assert torch.equal(o32.long(), ref)


def _cumsum(x):
    return torch.cat([torch.zeros(1, dtype=torch.int64, device=x.device), torch.cumsum(x.long(), 0)])


@pytest.mark.parametrize("n", [65537, 1_000_003, 4 * 4096 * 64 + 1, 33_550_336])
def test_lookback_scan_signed_items_unaligned_scratch(cuda, n):
    from pytorchsph_gb300 import _native as N
    lib = N.load()
    g = torch.Generator().manual_seed(n + 1)
    x = torch.randint(-1000, 1000, (n,), generator=g, dtype=torch.int32).to(cuda)
    ref = _cumsum(x)
    nbytes = lib.sph_scan_scratch_bytes(n)
    raw = torch.empty((nbytes + 7) // 8 + 1, dtype=torch.int64, device=cuda)
    before = lib.sph_scan_timeouts()
    for off in (0, 4):   # the scan aligns a scratch pointer that is not on 8 bytes itself
        o64 = torch.full((n + 1,), -1, dtype=torch.int64, device=cuda)
        N.call("sph_exclusive_scan_i32_to_i64", N.ptr(x), N.ptr(o64), n, N.ptr(raw) + off, nbytes, N.stream_ptr())
        torch.cuda.synchronize()
        assert torch.equal(o64, ref)
    assert lib.sph_scan_timeouts() == before


def test_lookback_scan_in_cuda_graph(cuda):
    """The zeroing of the tile words is part of the captured work: every replay scans anew."""
    from pytorchsph_gb300 import _native as N
    lib = N.load()
    n = 777_777
    x = torch.zeros(n, dtype=torch.int32, device=cuda)
    out = torch.empty(n + 1, dtype=torch.int32, device=cuda)
    scratch = torch.empty((lib.sph_scan_scratch_bytes(n) + 7) // 8, dtype=torch.int64, device=cuda)
    s = torch.cuda.Stream(cuda)
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        N.call("sph_exclusive_scan_i32", N.ptr(x), N.ptr(out), n, N.ptr(scratch), scratch.numel() * 8, N.stream_ptr())
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        N.call("sph_exclusive_scan_i32", N.ptr(x), N.ptr(out), n, N.ptr(scratch), scratch.numel() * 8, N.stream_ptr())
    g = torch.Generator().manual_seed(5)
    for _ in range(3):
        x.copy_(torch.randint(0, 50, (n,), generator=g, dtype=torch.int32).to(cuda))
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(out.long(), _cumsum(x))
    assert lib.sph_scan_timeouts() == 0


def test_lookback_scan_unaligned_input_and_output(cuda):
    """Input and output pointers 4 bytes past a 16-byte boundary: the same result."""
    from pytorchsph_gb300 import _native as N
    lib = N.load()
    n = 1_000_001
    g = torch.Generator().manual_seed(3)
    xs = torch.randint(0, 100, (n + 1,), generator=g, dtype=torch.int32).to(cuda)
    x = xs[1:]
    ref = _cumsum(x)
    o = torch.full((n + 2,), -1, dtype=torch.int32, device=cuda)
    scratch = torch.empty((lib.sph_scan_scratch_bytes(n) + 7) // 8, dtype=torch.int64, device=cuda)
    N.call("sph_exclusive_scan_i32", x.data_ptr(), o.data_ptr() + 4, n, N.ptr(scratch), scratch.numel() * 8,
           N.stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(o[1:].long(), ref)
