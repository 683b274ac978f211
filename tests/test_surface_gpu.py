"""GPU delta+ surface detection and shifting (pytorchsph_gb300.modules.deltaPlusModule on
sph_surface_term) against the reference's own detectSurface / shift
(tests/golden/surface_golden.npz) and against the float64 restatement (oracle/sph_torch.py).

Inputs are the reference's own pair lists, put in (i, j) order (the Module interface's pair
order; the reference sums the same pairs by scatter in its search order).  Tolerances,
relative to the field's maximum: lambda, eigenvalues, matrices and the lambda gradient 1e-4
(float32 summation order); the normal 5e-3 (it normalises a gradient that is small in the
bulk; the reference's own float32 normal differs from its float64 one by 6e-4); the shift
1e-4; the surface masks must be identical."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "surface_golden.npz")


def rel(a, b):
    a = a.detach().double().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


class Driver:
    def sync(self, t):
        return


def _ordered(pairs, *vals):
    """Pairs (and their per-pair values) sorted by (row, col)."""
    key = pairs[0].astype(np.int64) * (1 << 32) + pairs[1].astype(np.int64)
    o = np.argsort(key, kind="stable")
    return (pairs[:, o],) + tuple(v[o] for v in vals)


def _setup(g, m, part, cuda):
    from pytorchsph_gb300 import modules as M
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=cuda)
    G = lambda k: g[f"{part}/in_{k}"]
    nb, d, q = _ordered(G("fluidNeighbors"), G("fluidDistances"), G("fluidRadialDistances"))
    st = {"fluidPosition": t(G("fluidPosition")), "fluidVelocity": t(G("fluidVelocity")),
          "fluidDensity": t(G("fluidDensity")), "fluidArea": t(G("fluidArea")), "fluidVolume": t(G("fluidVolume")),
          "fluidNeighbors": t(nb.astype(np.int64)), "fluidDistances": t(d), "fluidRadialDistances": t(q),
          "numParticles": len(G("fluidPosition"))}
    cfg = {"particle": {"support": np.float32(m["h"]), "packing": m["packing"]},
           "fluid": {"restDensity": m["rho0"], "c0": m["c0"], "backgroundPressure": False},
           "diffusion": {"densityScheme": "deltaSPH", "alpha": m["alpha"], "delta": m["delta"], "kinematic": 0.001,
                         "boundaryDiffusion": True},
           "pressure": {"gamma": 7.0, "kappa": 1.0, "fluidPressureTerm": "TaitEOS", "boundaryPressureTerm": "PBSPH"},
           "compute": {"precision": torch.float32, "device": "cuda", "maxNeighbors": 256},
           "simulation": {"densityScheme": "continuum", "scheme": "deltaPlus", "boundaryScheme": "solid",
                          "bodyForces": True},
           "shifting": {"enabled": True, "scheme": "deltaPlus"},
           "solidBoundary": {"recomputeBoundary": False, "layers": 3},
           "neighborSearch": {"gradientThreshold": 1e-7, "supportScale": 1.0, "sortNeighborhoods": True},
           "domain": {"virtualMin": [float(v) for v in g["scene_vmin"]],
                      "virtualMax": [float(v) for v in g["scene_vmax"]]}}
    sim = Driver()
    sim.config = cfg
    bm = M.solidBoundaryModule()
    for p in bm.getParameters():
        p.parseConfig(cfg)
    bm.initialize(cfg, st)
    bm.resetState(st)
    bm.setWalls(t(G("boundaryPositions")), t(G("boundaryPositions")), t(G("boundaryVolume")))
    bp, bd, bq = _ordered(G("boundaryToFluidNeighbors"), G("boundaryToFluidNeighborDistances"),
                          G("boundaryToFluidNeighborRadialDistances"))
    bm.boundaryToFluidNeighbors = t(bp.astype(np.int64))
    bm.boundaryToFluidNeighborDistances = t(bd)
    bm.boundaryToFluidNeighborRadialDistances = t(bq)
    bm._bf = M._WallPairs(bm.boundaryToFluidNeighbors, t(bd), t(bq), bm.numPtcls, st["numParticles"])
    if f"{part}/in_boundaryToBoundaryNeighbors" in g.files:
        wp, wd, wq = _ordered(G("boundaryToBoundaryNeighbors"), G("boundaryToBoundaryNeighborDistances"),
                              G("boundaryToBoundaryNeighborRadialDistances"))
        rows = t(wp[0].astype(np.int64))
        off = torch.empty(bm.numPtcls + 1, dtype=torch.int32, device=cuda)
        from pytorchsph_gb300 import _native as N
        N.call("sph_row_offsets", N.ptr(rows), rows.shape[0], bm.numPtcls, N.ptr(off), N.stream_ptr())
        bm._ww = (off, t(wp[1].astype(np.int64)), t(wd), t(wq))
    bm.boundaryDensity = t(G("boundaryDensity"))
    sim.boundaryModule = bm
    dp = M.deltaPlusModule()
    dp.initialize(cfg, st)
    return st, sim, dp


@pytest.fixture(scope="module")
def gold():
    g = np.load(GOLDEN)
    return g, json.loads(str(g["meta"]))


def test_detect_surface_matches_reference(cuda, gold):
    g, m = gold
    st, sim, dp = _setup(g, m, "surface", cuda)
    dp.detectSurface(st, sim)
    torch.cuda.synchronize()
    R = lambda k: g[f"surface/out_{k}"]
    for k in ("normalizationMatrix", "fluidL", "eigVals", "fluidLambda", "lambdaGrad"):
        assert rel(st[k], R(k)) < 1e-4, k
    assert rel(st["fluidNormal"], R("fluidNormal")) < 5e-3
    assert rel(sim.boundaryModule.normalizationMatrix, R("boundaryNormalizationMatrix")) < 1e-4
    assert rel(sim.boundaryModule.eigVals, R("boundaryEigVals")) < 1e-4
    assert np.array_equal(st["fluidSurfaceMask"].cpu().numpy(), R("fluidSurfaceMask"))
    # the error against the reference's float64 run, beside the float32 reference's own
    for k in ("fluidLambda", "fluidNormal"):
        e_gpu = rel(st[k], g[f"f64_surface/out_{k}"])
        e_ref = rel(R(k), g[f"f64_surface/out_{k}"])
        assert e_gpu <= 10 * e_ref + 1e-6, (k, e_gpu, e_ref)


def test_shift_matches_reference(cuda, gold):
    g, m = gold
    st, sim, dp = _setup(g, m, "shift", cuda)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=cuda)
    st["fluidNormal"] = t(g["shift/in_fluidNormal"])
    st["fluidSurfaceMask"] = t(g["shift/in_fluidSurfaceMask"])
    dp.computeShiftAmount(st, sim)
    raw = st["shiftAmount"].clone()
    dp.adjustShiftingAmount(st, sim)
    torch.cuda.synchronize()
    assert rel(raw, g["shift/out_shiftAmount"]) < 1e-4
    assert rel(st["fluidUpdate"], g["shift/out_fluidUpdate"]) < 1e-4
    assert np.array_equal(st["fluidSurfaceMask"].cpu().numpy(), g["shift/out_fluidSurfaceMask"])


def test_detect_surface_from_own_search(cuda, gold):
    """The whole path on the GPU: neighbor search, wall search, densities, detectSurface on the
    golden's scene; the pair sets are the reference's, so the mask must be the reference's."""
    from pytorchsph_gb300 import modules as M
    g, m = gold
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=cuda)
    st0, sim, dp = _setup(g, m, "surface", cuda)
    G = lambda k: g[f"surface/in_{k}"]
    n = len(G("fluidPosition"))
    st = {"fluidPosition": t(G("fluidPosition")), "fluidVelocity": t(G("fluidVelocity")),
          "fluidDensity": t(G("fluidDensity")), "fluidArea": t(G("fluidArea")),
          "fluidSupport": torch.full((n,), float(np.float32(m["h"])), device=cuda), "numParticles": n}
    cfg = sim.config
    ns = M.neighborSearchModule()
    for p in ns.getParameters():
        p.parseConfig(cfg)
    ns.initialize(cfg, st)
    dens = M.densityModule()
    dens.initialize(cfg, st)
    sim.neighborSearch = ns
    bm = sim.boundaryModule
    bm.boundaryDensity = t(G("boundaryDensity"))
    ns.search(st, sim)
    bm.boundaryNeighborhoodSearch(st, sim)
    dens.evaluate(st, sim)
    bm.boundaryDensity = t(G("boundaryDensity"))      # the reference's mDBC densities of this state
    dp.detectSurface(st, sim)
    torch.cuda.synchronize()
    assert rel(st["fluidLambda"], g["surface/out_fluidLambda"]) < 1e-4
    assert np.array_equal(st["fluidSurfaceMask"].cpu().numpy(), g["surface/out_fluidSurfaceMask"])


def test_wall_index_past_fluid_raises(cuda, gold):
    """deltaPlus.py:150 reads fluidArea[b] for wall b: with more walls than fluid particles the
    reference raises IndexError, and so does the module."""
    g, m = gold
    st, sim, dp = _setup(g, m, "surface", cuda)
    keep = 100
    for k in ("fluidPosition", "fluidVelocity", "fluidDensity", "fluidArea", "fluidVolume"):
        st[k] = st[k][:keep].contiguous()
    nb = st["fluidNeighbors"]
    sel = (nb[0] < keep) & (nb[1] < keep)
    st["fluidNeighbors"] = nb[:, sel].contiguous()
    st["fluidDistances"] = st["fluidDistances"][sel].contiguous()
    st["fluidRadialDistances"] = st["fluidRadialDistances"][sel].contiguous()
    st["numParticles"] = keep
    bm = sim.boundaryModule
    from pytorchsph_gb300 import modules as M
    bp = bm.boundaryToFluidNeighbors
    sel = bp[1] < keep
    bm.boundaryToFluidNeighbors = bp[:, sel].contiguous()
    bm._bf = M._WallPairs(bm.boundaryToFluidNeighbors, bm.boundaryToFluidNeighborDistances[sel].contiguous(),
                          bm.boundaryToFluidNeighborRadialDistances[sel].contiguous(), bm.numPtcls, keep)
    dp.computeNormalizationmatrix(st, sim)
    with pytest.raises(IndexError):
        dp.computeFluidNormal(st, sim)


def test_deltaplus_timestep_matches_reference(cuda, gold):
    """The deltaSPH timestep with the delta+ module (src/deltaSPH.py:146-200 with
    simulation.scheme = 'deltaPlus': surface detection at step 5 and the surface-switched
    pressure term computePressureAccelDeltaPlus, pressure.py:31-51, fluid and wall parts),
    driven through the Module interface from the neighbor search on, against the reference's
    first right-hand side: the error against the reference's float64 run at most 3x its float32
    run's own error plus 1e-6 of the maximum."""
    from pytorchsph_gb300 import modules as M
    g, m = gold
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=cuda)
    _, sim, dp = _setup(g, m, "surface", cuda)
    cfg = sim.config
    cfg["gravity"] = {"magnitude": 9.81, "direction": [0.0, -1.0], "pointSource": False, "potentialField": True,
                      "center": [0.0, 0.0]}
    pos = g["scene_pos"]
    n = len(pos)
    st = {"fluidPosition": t(pos), "fluidVelocity": t(g["scene_vel"]), "fluidDensity": t(g["scene_rho"]),
          "fluidArea": t(g["scene_area"]), "fluidSupport": torch.full((n,), float(np.float32(m["h"])), device=cuda),
          "numParticles": n, "fluidRestDensity": torch.full((n,), m["rho0"], device=cuda)}
    sim.neighborSearch = M.neighborSearchModule()
    bm = M.solidBoundaryModule()
    sim.boundaryModule = bm
    sim.densityDiffusionModule = M.densityDiffusionModule()
    sim.pressureModule = M.pressureModule()
    mods = [sim.neighborSearch, bm, sim.densityDiffusionModule, sim.pressureModule, M.densityModule(),
            M.gravityModule(), M.momentumModule(), M.diffusionModule(), M.laminarViscosityModule(), dp]
    for mod in mods:
        for p in mod.getParameters() or []:
            p.parseConfig(cfg)
        mod.initialize(cfg, st)
        mod.resetState(st)
    dens, grav, mom, visc, lam = mods[4:9]
    bm.setWalls(t(g["scene_wall_pos"]), t(g["scene_ghost_pos"]), t(g["scene_wall_area"]))
    sim.neighborSearch.search(st, sim)                                   # 2
    bm.boundaryNeighborhoodSearch(st, sim)                               # 3
    dens.evaluate(st, sim)                                               # 4
    bm.evalBoundaryDensity(st, sim)
    dp.detectSurface(st, sim)                                            # 5
    st["fluidAcceleration"] = torch.zeros_like(st["fluidVelocity"])      # 6
    grav.evaluate(st, sim)                                               # 7
    mom.computeDpDt(st, sim)                                             # 8
    sim.densityDiffusionModule.computeDensityDiffusion(st, sim)          # 9
    sim.pressureModule.computePressure(st, sim)                          # 10
    sim.pressureModule.computePressureAcceleration(st, sim)
    visc.evaluate(st, sim)                                               # 11
    lam.computeLaminarViscosity(st, sim)                                 # 12
    torch.cuda.synchronize()
    assert np.array_equal(st["fluidSurfaceMask"].cpu().numpy(), g["surface/out_fluidSurfaceMask"])
    for key, field in (("fluidAcceleration", "fluidAcceleration"), ("dpdt", "dpdt")):
        e_gpu = rel(st[field], g[f"f64_step/out_{key}"])
        e_ref = rel(g[f"step/out_{key}"], g[f"f64_step/out_{key}"])
        assert e_gpu <= 3 * e_ref + 1e-6, (key, e_gpu, e_ref)
        assert rel(st[field], g[f"step/out_{key}"]) < 2e-2, key
