"""The multi-replica plumbing of bench.py on CPU: two gloo ranks, each timing its own
replica; every timed region is bracketed by a barrier and the job's time is the maximum over
ranks (the slowest replica).  The path has no data exchange, so nothing else crosses ranks."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, _ = bench.dist_env()
        assert (r, w) == (rank, world)
        bench.sync_ranks(world)
        out[rank] = bench.max_over_ranks(10.0 * (rank + 1), world)
        bench.sync_ranks(world)
    finally:
        dist.destroy_process_group()


def test_two_replicas_time_is_the_slowest():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert dict(out) == {0: 20.0, 1: 20.0}


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    bench.sync_ranks(1)
