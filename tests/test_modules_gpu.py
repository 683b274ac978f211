"""The Module interface (pytorchsph_gb300.modules) driven in the reference's timestep order
(src/deltaSPH.py:146-200) on GPU kernels, against the restated reference step in float64
(oracle/sph_torch.py) and against the fused engine (pytorchsph_gb300.sim.Simulation).

A fluid-only oscillating drop is used, with a boundary module that adds nothing, so the
reference's own module composition (`x += simulation.boundaryModule...`) is exercised
without walls.  Tolerances are relative to each field's maximum: pairs bit-exact,
acceleration and dpdt within 5e-3 of float64 (the float32 bar of the solver tests), and
within 1e-4 of the fused engine (same float32 formulas, different summation grouping)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


class ZeroBoundary:
    """The wall hooks deltaSPH calls, all returning zero contributions (no walls)."""

    def __init__(self, n, dev):
        self.n, self.dev = n, dev

    def computeDpDt(self, st, sim):
        return torch.zeros(self.n, device=self.dev)

    def computeNormalizationMatrices(self, st, sim):
        return torch.zeros((self.n, 2, 2), device=self.dev)

    def computeRenormalizedDensityGradient(self, st, sim):
        return torch.zeros((self.n, 2), device=self.dev)

    def computePressure(self, st, sim):
        return None

    def computePressureAcceleration(self, st, sim):
        return torch.zeros((self.n, 2), device=self.dev)

    def computeVelocityDiffusion(self, st, sim):
        return torch.zeros((self.n, 2), device=self.dev)


class Driver:
    def __init__(self, n, dev):
        self.boundaryModule = ZeroBoundary(n, dev)

    def sync(self, t):
        return


def config(sc, diffusion, c0):
    return {
        "particle": {"support": sc["h"], "packing": 0.4},
        "fluid": {"restDensity": 1000.0, "c0": c0, "backgroundPressure": 0.0},
        "pressure": {"gamma": 7.0, "kappa": 1.0, "fluidPressureTerm": "TaitEOS"},
        "diffusion": {"alpha": 0.01, "delta": 0.1, "kinematic": 0.001, "boundaryDiffusion": True,
                      "densityScheme": diffusion},
        "compute": {"precision": torch.float32, "device": "cuda", "maxNeighbors": 256},
        "neighborSearch": {"gradientThreshold": 1e-7, "supportScale": 1.0, "sortNeighborhoods": True},
        "domain": {"virtualMin": [float(v) for v in sc["vmin"]], "virtualMax": [float(v) for v in sc["vmax"]]},
        "simulation": {"densityScheme": "continuum", "scheme": "deltaSPH", "boundaryScheme": "solid",
                       "bodyForces": True},
        "gravity": {"magnitude": 1.0, "direction": [0.0, -1.0], "pointSource": True, "potentialField": True,
                    "center": [0.0, 0.0]},
    }


def module_timestep(sc, diffusion, c0, dev):
    from pytorchsph_gb300 import modules as M
    n = len(sc["pos"])
    t = lambda a: torch.as_tensor(np.asarray(a, np.float32), device=dev).contiguous()
    rng = np.random.default_rng(5)
    rho = (1.0 + 1e-3 * rng.standard_normal(n)).astype(np.float32)   # a non-trivial density field
    st = {"fluidPosition": t(sc["pos"]), "fluidVelocity": t(sc["vel"]), "fluidDensity": t(rho),
          "fluidArea": t(sc["area"]), "fluidSupport": t(sc["support"])}
    cfg = config(sc, diffusion, c0)
    mods = [M.neighborSearchModule(), M.densityModule(), M.gravityModule(), M.momentumModule(),
            M.densityDiffusionModule(), M.pressureModule(), M.diffusionModule(), M.laminarViscosityModule()]
    for m in mods:
        for p in m.getParameters() or []:
            p.parseConfig(cfg)
        m.initialize(cfg, st)
        m.resetState(st)
    ns, dens, grav, mom, ddiff, pres, visc, lam = mods
    sim = Driver(n, dev)
    ns.search(st, sim)                                     # 2
    dens.evaluate(st, sim)                                 # 4
    st["fluidAcceleration"] = torch.zeros_like(st["fluidVelocity"])   # 6
    grav.evaluate(st, sim)                                 # 7
    mom.computeDpDt(st, sim)                               # 8
    ddiff.computeDensityDiffusion(st, sim)                 # 9
    pres.computePressure(st, sim)                          # 10
    pres.computePressureAcceleration(st, sim)
    visc.evaluate(st, sim)                                 # 11
    lam.computeLaminarViscosity(st, sim)                   # 12
    torch.cuda.synchronize()
    return st, rho


@pytest.mark.parametrize("diffusion", ["MOG", "deltaSPH"])
def test_module_timestep_matches_reference_step(cuda, diffusion):
    import sph_torch as S
    from pytorchsph_gb300 import workloads
    sc = workloads.oscillating_drop(3000, 0.5, 1.3)
    st, rho = module_timestep(sc, diffusion, 10.0, cuda)
    p = S.Params(h=sc["h"], c0=10.0, diffusion=diffusion, vmin=sc["vmin"], vmax=sc["vmax"], gravity=(0.0, 0.0),
                 point_source=True, kinematic=0.001)
    x32 = torch.from_numpy(sc["pos"])
    nb = S.search(x32, None, sc["h"], sc["vmin"], sc["vmax"], torch.float64)
    # the module search returns the reference pair set in (i, j) order
    pairs = st["fluidNeighbors"].cpu().numpy()
    assert np.array_equal(pairs[0], nb.ff.i.numpy()) and np.array_equal(pairs[1], nb.ff.j.numpy())
    ref = {"x": x32.double(), "v": torch.from_numpy(sc["vel"]).double(), "rho": torch.from_numpy(rho).double(),
           "area": torch.from_numpy(sc["area"]).double()}
    acc, _, dpdt, ex = S.deltasph_rhs(ref, None, nb, p, torch.float64)
    assert rel(st["fluidAcceleration"].cpu(), acc) < 5e-3
    assert rel(st["dpdt"].cpu(), dpdt) < 5e-3
    assert rel(st["fluidPressure"].cpu(), ex["pressure"]) < 1e-4
    assert rel(st["fluidVolume"].cpu(), ref["area"] / ref["rho"]) < 1e-6


def test_module_timestep_matches_fused_engine(cuda):
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.sim import Simulation, SimConfig
    sc = workloads.oscillating_drop(3000, 0.5, 1.3)
    st, rho = module_timestep(sc, "deltaSPH", 10.0, cuda)
    scene = dict(sc)
    scene["rho"] = rho
    cfg = SimConfig(solver="deltaSPH", integration="semiImplicitEuler", dt=1e-4, c0=10.0, gravity=(0.0, 0.0),
                    point_source=True, density_diffusion="deltaSPH", kinematic=0.001)
    sim = Simulation(scene, cfg, cuda)
    acc, _, dpdt = sim.rhs()
    to_orig = lambda t: sim._orig(t).cpu()
    assert rel(to_orig(acc), st["fluidAcceleration"].cpu()) < 1e-4
    assert rel(to_orig(dpdt), st["dpdt"].cpu()) < 1e-4


def test_summation_density_and_search_existing(cuda):
    import sph_torch as S
    from pytorchsph_gb300 import modules as M
    from pytorchsph_gb300 import workloads
    sc = workloads.dam_break(40, 60, 0.01, (4.0, 2.0))
    n = len(sc["pos"])
    t = lambda a: torch.as_tensor(np.asarray(a, np.float32), device=cuda).contiguous()
    st = {"fluidPosition": t(sc["pos"]), "fluidVelocity": t(sc["vel"]), "fluidDensity": t(sc["rho"]),
          "fluidArea": t(sc["area"]), "fluidSupport": t(sc["support"])}
    cfg = config(sc, "MOG", 10.0)
    cfg["simulation"]["densityScheme"] = "summation"
    ns, dens = M.neighborSearchModule(), M.densityModule()
    for m in (ns, dens):
        for p in m.getParameters() or []:
            p.parseConfig(cfg)
        m.initialize(cfg, st)
    ns.search(st, Driver(n, cuda))
    dens.evaluate(st, Driver(n, cuda))
    nb = S.search(torch.from_numpy(sc["pos"]), S.Walls(torch.from_numpy(sc["wall_pos"]),
                                                        torch.from_numpy(sc["ghost_pos"]),
                                                        torch.from_numpy(sc["wall_area"])),
                  sc["h"], sc["vmin"], sc["vmax"], torch.float64)
    F = nb.ff
    rho_ref = S.ssum(S.W(F.q, sc["h"]) * torch.from_numpy(sc["area"]).double()[F.j], F.i, n)
    assert rel(st["fluidDensity"].cpu(), rho_ref) < 1e-5
    # searchExisting: wall query points, the query's own support, distances / query support
    wq = t(sc["wall_pos"])
    wh = t(np.full(len(sc["wall_pos"]), sc["h"], np.float32))
    pairs, dist, radial = ns.searchExisting(wq, wh, st, Driver(n, cuda))
    key = lambda r, c: np.sort(np.asarray(r, np.int64) * (1 << 32) + np.asarray(c, np.int64))
    p = pairs.cpu().numpy()
    assert np.array_equal(key(p[0], p[1]), key(nb.bf.i.numpy(), nb.bf.j.numpy()))
    o = np.lexsort((p[1], p[0]))
    r_ref = nb.bf.q.numpy() * 1.0
    oref = np.lexsort((nb.bf.j.numpy(), nb.bf.i.numpy()))
    assert np.allclose(radial.cpu().numpy()[o], r_ref[oref], rtol=0, atol=1e-6)
    assert np.allclose(dist.cpu().numpy()[o], nb.bf.e.numpy()[oref], rtol=0, atol=1e-6)
