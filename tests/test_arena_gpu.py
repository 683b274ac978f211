"""The pooled serving arena (pytorchsph_gb300.serve.SceneArena): scenes admitted into free
slots and retired from them between steps, with the CUDA graph captured once.  Every scene's
result is bitwise the same as the scene stepped alone, whatever is admitted or retired around
it, also after the arena packs its cell ranges again."""
import numpy as np
import pytest
import torch

from test_serve_gpu import run_batch, same, spec

pytestmark = pytest.mark.gpu


def arena(cuda, **kw):
    from pytorchsph_gb300.serve import SceneArena
    args = dict(particles=40000, walls=20000, cells=400000, slots=8, scheme=2)
    args.update(kw)
    return SceneArena(cuda, **args)


def stepper(a):
    def go(k):
        for _ in range(k):
            if a.graph is None:
                a.capture()
            else:
                a.step()
    return go


def test_arena_scene_equals_alone(cuda):
    A, B, C = spec("dam_break", 3000, 0.7), spec("drop", 2500, 1.5), spec("dam_break", 5000, 1.8)
    a = arena(cuda)
    slots = [a.admit(x) for x in (B, A, C)]
    stepper(a)(6)
    a.check()
    for x, s in zip((B, A, C), slots):
        assert same(run_batch([x], 6, cuda)[0], a.scene_state(s))


def test_admission_and_retirement_midway_change_nothing(cuda):
    A, B, C = spec("dam_break", 3000, 1.2), spec("drop", 2600, 0.8), spec("dam_break", 2500, 0.6)
    a = arena(cuda)
    go = stepper(a)
    sa, sc = a.admit(A), a.admit(C)
    go(2)
    g = a.graph
    sb = a.admit(B)                 # into free slots of the captured batch
    go(2)
    final_c = {k: v.cpu().numpy() for k, v in a.retire(sc).items()}
    go(2)
    a.check()
    assert a.graph is g             # no new capture
    assert same(run_batch([A], 6, cuda)[0], a.scene_state(sa))
    assert same(run_batch([B], 4, cuda)[0], a.scene_state(sb))
    assert same(run_batch([C], 4, cuda)[0], final_c)


def test_cell_ranges_packed_again_change_nothing(cuda):
    from pytorchsph_gb300.serve import ArenaFull
    A, B, C = spec("dam_break", 2500, 1.0), spec("dam_break", 2500, 1.0), spec("drop", 2400, 1.0)
    D = spec("dam_break", 3200, 1.4)
    probe = arena(cuda)
    need = [probe.admit(x) for x in (A, B, C)]
    cells = {k: probe.slots[k]["ncells"] for k in need}
    nd = D.on_device(cuda)["grid"].num_cells + 1
    # room for A, C and D only after the ranges are packed: B's gap is too small for D
    a = arena(cuda, cells=cells[need[0]] + cells[need[2]] + max(nd, cells[need[1]]) + 8)
    go = stepper(a)
    sa, sb, sc = a.admit(A), a.admit(B), a.admit(C)
    go(2)
    a.retire(sb)
    sd = a.admit(D)
    go(3)
    a.check()
    assert same(run_batch([A], 5, cuda)[0], a.scene_state(sa))
    assert same(run_batch([C], 5, cuda)[0], a.scene_state(sc))
    assert same(run_batch([D], 3, cuda)[0], a.scene_state(sd))
    small = arena(cuda, particles=7000)
    small.admit(A)
    small.admit(B)
    with pytest.raises(ArenaFull):
        small.admit(C)


def test_pooled_server_grows_and_matches_alone(cuda):
    """The request loop on the arena: it grows past its first capacity (the one rebuild),
    every request completes its steps, and results equal the scenes run alone."""
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.serve import Request, Server
    trace = workloads.serving_trace(8, rate=400.0, n_min=8000, n_max=20000, steps=9, seed=5)
    reqs = [Request(t["rid"], t["arrival"], spec(t["kind"], t["n"], t["shape"], steps=t["steps"])) for t in trace]
    srv = Server(cuda)
    srv.run(reqs, time_scale=1.0, max_wall=120)
    assert srv.pooled and srv.arena_grows >= 1
    assert all(r.steps_done == r.spec.steps and r.error is None for r in reqs)
    for r in (reqs[0], reqs[5]):
        assert same(run_batch([r.spec], r.spec.steps, cuda)[0], r.final)
    p = srv.latency_percentiles()
    assert p[50] is not None and p[99] >= p[50] > 0


def test_admit_many_equals_one_by_one(cuda):
    """Admitting several scenes in one call (one copy per field for scenes uploaded side by
    side) gives bitwise the states of admitting them one by one; when they do not all fit it
    admits none and says so."""
    A, B, C = spec("dam_break", 2600, 0.9), spec("drop", 2300, 1.3), spec("dam_break", 3100, 1.6)
    a1 = arena(cuda)
    s1 = a1.admit_many([A, B, C])
    assert s1 is not None and len(set(s1)) == 3
    stepper(a1)(4)
    a1.check()
    for x in (A, B, C):
        x.dev = None                  # upload again, one scene at a time
    a2 = arena(cuda)
    s2 = [a2.admit(x) for x in (A, B, C)]
    stepper(a2)(4)
    for p, q in zip(s1, s2):
        assert same(a1.scene_state(p), a2.scene_state(q))
    small = arena(cuda, particles=6000)
    assert small.admit_many([A, B, C]) is None and not small.slots and small.occupied == 0


def test_retire_many_equals_retire(cuda):
    """Retiring several scenes in one pass gives each its state in its own particle order, as
    retire() does, and frees their particles, walls and slots; the scene left behind is
    unaffected."""
    A, B, C = spec("dam_break", 2600, 1.1), spec("drop", 2300, 0.9), spec("dam_break", 2900, 1.4)
    a1, a2 = arena(cuda), arena(cuda)
    s1 = [a1.admit(x) for x in (A, B, C)]
    s2 = [a2.admit(x) for x in (A, B, C)]
    stepper(a1)(3)
    stepper(a2)(3)
    one = {sl: {k: v.cpu().numpy() for k, v in a1.retire(sl).items()} for sl in (s1[0], s1[2])}
    rows, out = a2.retire_many([s2[0], s2[2]])
    for sl1, sl2 in ((s1[0], s2[0]), (s1[2], s2[2])):
        r0, n = rows[sl2]
        got = {"x": out[0][r0:r0 + n].cpu().numpy(), "v": out[1][r0:r0 + n].cpu().numpy(),
               "rho": out[2][r0:r0 + n].cpu().numpy()}
        assert same(got, one[sl1])
    assert sorted(a2.slots) == [s2[1]] and a2.live_n == a1.live_n and a2.walls_n == a1.walls_n
    stepper(a1)(2)
    stepper(a2)(2)
    a2.check()
    assert same(a1.scene_state(s1[1]), a2.scene_state(s2[1]))


def test_extent_shrinks_and_grows_without_changing_results(cuda):
    """With a small extent quantum the arena steps only its occupied slots: retiring scenes
    shrinks the extent, admitting grows it again over slots that an earlier extent left
    stale; every scene still equals the scene run alone."""
    A, B, C = spec("dam_break", 3000, 1.2), spec("drop", 2600, 0.8), spec("dam_break", 4200, 1.5)
    D, E = spec("drop", 2400, 1.4), spec("dam_break", 2800, 0.9)
    a = arena(cuda, extent_quantum=2048)
    go = stepper(a)
    sa, sb, sc = a.admit(A), a.admit(B), a.admit(C)
    go(2)
    assert a.n == 10240 and len(a._graphs) == 1
    final_b = {k: v.cpu().numpy() for k, v in a.retire(sb).items()}
    final_c = {k: v.cpu().numpy() for k, v in a.retire(sc).items()}
    go(2)                                  # A alone: the extent shrinks to 4096
    assert a.n == 4096
    sd, se = a.admit(D), a.admit(E)        # grows over slots that held B and C
    go(3)
    a.check()
    assert a.n == 8192 and len(a._graphs) >= 3   # particle extents 10240, 4096, 8192
    assert same(run_batch([A], 7, cuda)[0], a.scene_state(sa))
    assert same(run_batch([B], 2, cuda)[0], final_b)
    assert same(run_batch([C], 2, cuda)[0], final_c)
    assert same(run_batch([D], 3, cuda)[0], a.scene_state(sd))
    assert same(run_batch([E], 3, cuda)[0], a.scene_state(se))
