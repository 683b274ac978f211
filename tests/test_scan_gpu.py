"""The exclusive scans of the C ABI against torch.cumsum at sizes around the one-launch
path's limit (16 tiles of 4096) and the tile size, int32 and int64 outputs."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 5, 4095, 4096, 4097, 3 * 4096 + 7, 65535, 65536, 65537, 300_001])
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
