"""The counting sort that moves per-particle arrays in its in-cell fix
(sph_counting_sort_permute) against sph_counting_sort_tie followed by sph_permute_arrays:
the same order, sorted keys and rows, bit for bit.  Cell sizes cover the one-thread ranking
(<= 48), the shared-memory ranking (<= 1024) and the bitonic sort (<= 2048), with 4-, 8- and
16-byte rows."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sort(N, keys, tie, cap, pairs=None):
    lib = N.load()
    n = keys.numel()
    dev = keys.device
    hist = torch.bincount(keys.long(), minlength=cap + 1).to(torch.int32)
    cell_start = torch.empty(cap + 2, dtype=torch.int32, device=dev)
    order = torch.empty(n, dtype=torch.int32, device=dev)
    skeys = torch.empty(n, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    scratch = torch.empty((lib.sph_counting_sort_scratch_bytes(n, cap) + 7) // 8, dtype=torch.int64, device=dev)
    if pairs is None:
        N.call("sph_counting_sort_tie", N.ptr(keys), n, cap, N.ptr(hist), N.ptr(cell_start), N.ptr(tie), N.ptr(order),
               N.ptr(skeys), N.ptr(status), N.ptr(scratch), scratch.numel() * 8, N.stream_ptr())
    else:
        k, eb, ins, outs = N.array_set(pairs)
        N.call("sph_counting_sort_permute", N.ptr(keys), n, cap, N.ptr(hist), N.ptr(cell_start), N.ptr(tie),
               N.ptr(order), N.ptr(skeys), k, eb, ins, outs, N.ptr(status), N.ptr(scratch), scratch.numel() * 8,
               N.stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert int(hist.abs().sum().item()) == 0   # the sort leaves the histogram zeroed
    return order, skeys, cell_start


def test_counting_sort_permute_matches_sort_then_permute(cuda):
    from pytorchsph_gb300 import _native as N
    g = torch.Generator().manual_seed(11)
    cap = 4000
    parts = [torch.randint(0, cap, (150_000,), generator=g),
             torch.full((60,), 17), torch.full((700,), 123), torch.full((1500,), 2500)]
    keys = torch.cat(parts)
    keys = keys[torch.randperm(keys.numel(), generator=g)].to(torch.int32).to(cuda)
    n = keys.numel()
    tie = torch.randperm(n, generator=g).to(torch.int32).to(cuda)
    x = torch.randn(n, 2, generator=g).to(cuda)
    rho = torch.randn(n, generator=g).to(cuda)
    rec = torch.randn(n, 4, generator=g).to(cuda)
    uid = torch.arange(n, dtype=torch.int32, device=cuda)
    order_a, skeys_a, cs_a = _sort(N, keys, tie, cap)
    outs = [torch.empty_like(t) for t in (x, rho, rec, uid)]
    order_b, skeys_b, cs_b = _sort(N, keys, tie, cap, list(zip((x, rho, rec, uid), outs)))
    assert torch.equal(order_a, order_b) and torch.equal(skeys_a, skeys_b) and torch.equal(cs_a, cs_b)
    o = order_a.long()
    for src, dst in zip((x, rho, rec, uid), outs):
        assert torch.equal(dst, src[o])
    # the order is by (cell, tie) with the cells ascending
    k = keys.long()[o]
    assert torch.all(k[1:] >= k[:-1])
    t = tie.long()[o]
    same = k[1:] == k[:-1]
    assert torch.all(t[1:][same] > t[:-1][same])
