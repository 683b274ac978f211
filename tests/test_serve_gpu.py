"""Batched serving (pytorchsph_gb300.serve): every scene gives the same result alone and in
any mix of scenes (bitwise: scenes share no data and each cell is ordered by particle id),
a batch of one equals the single-scene engine, pairs taken from the cell rows equal pairs
from a CSR list, a captured CUDA graph equals eager launches, rebuilding the batch mid-run
changes nothing, and the request loop completes a trace."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def spec(kind, n, shape, steps=5):
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.serve import SceneSpec
    from pytorchsph_gb300.sim import SimConfig
    sc, p = workloads.make_request_scene({"kind": kind, "n": n, "shape": shape})
    cfg = SimConfig(solver="deltaSPH", integration="semiImplicitEuler", dt=p["dt"], c0=p["c0"], gravity=p["gravity"],
                    point_source=p["point_source"], density_diffusion=p["diffusion"])
    return SceneSpec(sc, cfg, steps)


def run_batch(specs, steps, dev, graph=False, pairs="cells"):
    from pytorchsph_gb300.serve import SceneBatch
    b = SceneBatch(specs, dev, pairs=pairs)
    if graph:
        b.capture()
        steps -= 1
    for _ in range(steps):
        b.step()
    b.check()
    return [b.scene_state(s) for s in range(len(specs))]


def same(a, b):
    return all(np.array_equal(a[k], b[k]) for k in ("x", "v", "rho"))


def test_alone_equals_in_mix(cuda):
    A = spec("dam_break", 3000, 0.7)
    B = spec("drop", 2500, 1.5)
    C = spec("dam_break", 5000, 1.8)
    alone = run_batch([A], 6, cuda)[0]
    mix = run_batch([B, A, C], 6, cuda)
    assert same(alone, mix[1])
    alone_b = run_batch([B], 6, cuda)[0]
    assert same(alone_b, mix[0])


def test_batch_of_one_equals_single_scene_engine(cuda):
    from pytorchsph_gb300.sim import Simulation
    A = spec("dam_break", 4000, 1.0)
    sim = Simulation(A.scene, A.cfg, cuda)
    for _ in range(6):
        sim.step()
    s = sim.state()
    b = run_batch([A], 6, cuda)[0]
    assert same(s, b)


def test_cell_pairs_equal_csr_pairs(cuda):
    """Both pair sources visit the same pairs in the same order: bitwise equal states, for
    renormalized and MOG scenes in one batch."""
    import dataclasses
    A, B = spec("dam_break", 3000, 1.2), spec("drop", 2600, 0.8)
    C = spec("dam_break", 2500, 0.6)
    C = dataclasses.replace(C, cfg=dataclasses.replace(C.cfg, density_diffusion="MOG"))
    cells = run_batch([A, B, C], 6, cuda, pairs="cells")
    csr = run_batch([A, B, C], 6, cuda, pairs="csr")
    assert all(same(x, y) for x, y in zip(cells, csr))


def test_segment_overflow_takes_the_cell_rows(cuda):
    """Particles with more non-empty segments than a segment list holds (a dam-break block
    compressed to 0.45 of its spacing: ~140 neighbors, over 8 segments of 32 candidates)
    take their pairs from the cell rows in both force passes: bitwise the states of the CSR
    list, with the drop beside it unaffected."""
    import ctypes
    import dataclasses
    from pytorchsph_gb300 import _native as N
    from pytorchsph_gb300.serve import SceneBatch
    A = spec("dam_break", 3000, 1.0)
    sc = dict(A.scene)
    lo = sc["pos"].min(0)
    sc["pos"] = (lo + (sc["pos"] - lo) * 0.45).astype(np.float32)
    A = dataclasses.replace(A, scene=sc)
    B = spec("drop", 2500, 1.0)
    b = SceneBatch([A, B], cuda, pairs="cells")
    for _ in range(3):
        b.step()
    b.check()
    mo, so, co, ms = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int32()
    N.call("sph_deltasph_segment_lists", b.n, ctypes.byref(mo), ctypes.byref(so), ctypes.byref(co),
           ctypes.byref(ms))
    counts = b.forces_scratch.view(torch.int32)[co.value // 4:co.value // 4 + b.n].cpu().numpy()
    assert (counts == -1).sum() > 500 and counts.max() <= ms.value
    cells = [b.scene_state(s) for s in range(2)]
    csr = run_batch([A, B], 3, cuda, pairs="csr")
    assert all(same(x, y) for x, y in zip(cells, csr))
    assert same(cells[1], run_batch([B], 3, cuda)[0])


def test_graph_replay_equals_eager(cuda):
    A, B = spec("dam_break", 3000, 1.2), spec("drop", 3000, 0.8)
    e = run_batch([A, B], 7, cuda, graph=False)
    g = run_batch([A, B], 7, cuda, graph=True)
    assert all(same(x, y) for x, y in zip(e, g))


def test_rebuild_midway_changes_nothing(cuda):
    from pytorchsph_gb300.serve import SceneBatch
    A, B = spec("dam_break", 3000, 1.2), spec("drop", 3000, 0.8)
    straight = run_batch([A, B], 8, cuda)
    b1 = SceneBatch([A, B], cuda)
    for _ in range(3):
        b1.step()
    states = [b1.scene_state(0), b1.scene_state(1)]
    b2 = SceneBatch([B, A], cuda, states=[states[1], states[0]])
    for _ in range(5):
        b2.step()
    assert same(straight[0], b2.scene_state(1))
    assert same(straight[1], b2.scene_state(0))


def test_server_completes_small_trace(cuda):
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.serve import Request, Server, SceneSpec
    from pytorchsph_gb300.sim import SimConfig
    trace = workloads.serving_trace(6, rate=200.0, n_min=2048, n_max=6000, steps=12, seed=3)
    reqs = []
    for t in trace:
        s = spec(t["kind"], t["n"], t["shape"], steps=t["steps"])
        reqs.append(Request(t["rid"], t["arrival"], s))
    srv = Server(cuda, rebuild_every=4)
    srv.run(reqs, time_scale=1.0, max_wall=120)
    assert all(r.steps_done == r.spec.steps for r in reqs), [(r.rid, r.steps_done) for r in reqs]
    # a request's result equals the same scene run alone for its step count
    r = reqs[2]
    alone = run_batch([r.spec], r.spec.steps, cuda)[0]
    assert r.final is not None and same(alone, r.final)


def test_particle_leaving_its_grid_keeps_scenes_apart(cuda):
    """A particle thrown out of its scene's grid goes to that scene's outside slot: the scene
    keeps its own particle range, the particle has no neighbors, and the scene's result is
    still the same alone and in a mix."""
    from pytorchsph_gb300 import _native as N
    from pytorchsph_gb300.serve import SceneBatch, SceneSpec
    A = spec("dam_break", 3000, 0.7)
    B = spec("drop", 2500, 1.5)
    sc = dict(B.scene)
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    pos[7] = (1.45, 0.0)                       # alone near the edge of the grid (domain +-1.5)
    vel[7] = (200.0, 0.0)                      # ~0.1 m per step: outside after two steps
    sc["pos"], sc["vel"] = pos, vel
    Bx = SceneSpec(sc, B.cfg, B.steps)
    b = SceneBatch([Bx, A], cuda)
    for _ in range(6):
        b.step()
    b.check()                                  # leaving the grid is reported, not an error
    assert b.flags() & N.SPH_FLAG_OUT_OF_GRID
    esc = b.escaped()
    assert list(esc) == [1, 0]
    mix = [b.scene_state(0), b.scene_state(1)]
    g = b.grids[0]
    hi = g.qmin[0] + g.cells_x * g.hmax
    assert mix[0]["x"][7, 0] > hi and np.isfinite(mix[0]["x"]).all()
    assert same(run_batch([A], 6, cuda)[0], mix[1])
    assert same(run_batch([Bx], 6, cuda)[0], mix[0])


def test_pair_overflow_holds_the_step(cuda):
    """With a column buffer too small for the neighbor list the fill writes only whole rows
    that fit, no kernel reads past it, and the update leaves the state unchanged."""
    from pytorchsph_gb300 import _native as N
    from pytorchsph_gb300.serve import SceneBatch
    A = spec("dam_break", 3000, 1.0)
    b = SceneBatch([A], cuda, pair_headroom=0.5, pairs="csr")
    before = b.scene_state(0)
    b.step()
    assert b.flags() & N.SPH_FLAG_PAIR_CAPACITY
    assert same(before, b.scene_state(0))
    with pytest.raises(N.SPHError):
        b.check()


def test_server_recovers_from_pair_overflow(cuda):
    """The request loop reruns a step the device did not apply, after a rebuild with more
    pair headroom; results equal the scenes run alone."""
    from pytorchsph_gb300.serve import Request, Server
    A, B = spec("dam_break", 3000, 1.2, steps=5), spec("drop", 2600, 0.9, steps=7)
    reqs = [Request(0, 0.0, A), Request(1, 0.0, B)]
    srv = Server(cuda, rebuild_every=4, pair_headroom=0.5, pairs="csr")
    srv.run(reqs, time_scale=1.0, max_wall=120)
    assert srv.pair_overflows >= 1
    assert all(r.steps_done == r.spec.steps and r.error is None for r in reqs)
    for r in reqs:
        assert same(run_batch([r.spec], r.spec.steps, cuda)[0], r.final)


def close(a, b, tol):
    """Max |a - b| of each field within tol[field] of the field's largest magnitude."""
    return all(np.abs(a[k].astype(np.float64) - b[k]).max() <= tol[k] * max(np.abs(b[k]).max(), 1e-30)
               for k in ("x", "v", "rho"))


# Another summation order moves a step by float32 rounding: positions and densities hardly,
# velocities more, because pressure and wall terms are small remainders of large sums (one
# float32 step is 2e-3 of max |v| from the float64 step on these dam breaks).
REORDER_TOL = {"x": 1e-6, "v": 5e-3, "rho": 1e-5}


def configured(spec, ratio, tpp):
    import dataclasses
    return dataclasses.replace(spec, cell_ratio=ratio, tpp=tpp, dev=None)


def test_lanes_per_particle_and_cell_ratio_keep_the_pairs(cuda):
    """Splitting a particle's segments over 2 or 4 lanes, or searching cells of h/2 two cells
    out, visits the same pairs in another order: after 6 steps the states agree with one lane
    and cells of h within float32 rounding (REORDER_TOL), and a configured scene is still
    bitwise the same alone and in a mix of differently configured scenes."""
    A, B = spec("dam_break", 3000, 1.2), spec("drop", 2600, 0.8)
    base = run_batch([A, B], 6, cuda)
    for ratio, tpp in ((1, 2), (1, 4), (2, 1), (2, 2)):
        got = run_batch([configured(A, ratio, tpp), configured(B, ratio, tpp)], 6, cuda)
        assert close(got[0], base[0], REORDER_TOL) and close(got[1], base[1], REORDER_TOL), (ratio, tpp)
    A2, B4, C = configured(A, 2, 2), configured(B, 1, 4), spec("dam_break", 2500, 0.6)
    mix = run_batch([C, B4, A2], 6, cuda, graph=True)
    assert same(run_batch([A2], 6, cuda)[0], mix[2])
    assert same(run_batch([B4], 6, cuda)[0], mix[1])
    assert same(run_batch([C], 6, cuda)[0], mix[0])


def test_autotuner_picks_a_measured_configuration(cuda):
    from pytorchsph_gb300.serve import SceneBatch
    from pytorchsph_gb300.tune import Autotuner, Tuning
    tuner = Autotuner(cuda)
    t = Tuning(serving=tuner.tune_serving(sizes=(2048,), batch_particles=8192, steps=2,
                                          candidates=((1, 1), (2, 2))))
    e = t.serving[11]
    assert (e["cell_ratio"], e["tpp"]) in ((1, 1), (2, 2)) and len(e["measured"]) == 2
    best = min(e["measured"].values(), key=lambda m: m["ms_per_step"])
    assert e["measured"][f'{e["cell_ratio"]},{e["tpp"]}'] is best
    A = spec("drop", 2600, 0.8)
    b = SceneBatch([A], cuda, tuning=t)
    assert (A.cell_ratio, A.tpp) == (e["cell_ratio"], e["tpp"])
    b.step()
    b.check()
