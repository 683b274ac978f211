"""Test infrastructure only (oracle): run the reference's own deltaSPH / DFSPH time steps.

Builds `deltaSPHSimulation` / `dfsphSimulation` objects of wi-re/pytorchSPH
(src/deltaSPH.py:74-140, src/dfsph.py:70-125) around a scene from
`pytorchsph_gb300.workloads` and steps them with the reference's own `integrate()`
(src/simulationBase.py:632-782) on CPU.  Scene setup that the reference derives through
Nelder-Mead packing and skimage contours (src/simulationBase.py:832-979,
src/ghostParticles.py:97-139) is replaced by the scene's exact arrays:
* SPHSimulation.__init__ is bypassed; the config entries it derives (particle area,
  support, packing, virtual domain, wall polygon) are filled in directly;
* solidBoundary's `samplePolygon` returns the scene's wall / ghost layers.
Everything on the hot path — neighbor search, every summation, mDBC, the solvers, the
integrators — is the reference's own code.  Only the development container has the
reference; the vectors it produces are committed under tests/golden/.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import ref_harness  # noqa: E402


def _modules():
    R = ref_harness.load()
    import importlib
    deltaSPH = importlib.import_module("src.deltaSPH")
    dfsph = importlib.import_module("src.dfsph")
    sb = importlib.import_module("src.simulationBase")
    return R, deltaSPH, dfsph, sb


def base_config(scene, scheme="deltaSPH", diffusion="MOG", integration="semiImplicitEuler", dt=None, c0=None,
                rho0=1000.0, alpha=0.01, delta=0.1, kinematic=0.001, gravity=9.81, point_source=False,
                point_center=(0.0, 0.0), dfsph=None, cfl_fixed=True, boundary_diffusion=True,
                boundary_pressure="PBSPH"):
    dx = scene["dx"]
    h = np.float32(scene["h"])
    W, H = scene.get("tank", (None, None))
    if c0 is None:
        c0 = 10.0 * math.sqrt(2.0 * 9.81 * scene["column_height"])
    if dt is None:
        dt = 0.25 * float(h) / c0
    radius = dx / math.sqrt(math.pi)
    cfg = {
        "particle": {"radius": radius},
        "simulation": {"scheme": scheme, "boundaryScheme": "solid", "verbose": False,
                       "densityScheme": "continuum" if scheme != "dfsph" else "summation", "mode": "default"},
        "pressure": {"fluidPressureTerm": "TaitEOS", "boundaryPressureTerm": boundary_pressure, "gamma": 7.0},
        "diffusion": {"velocityScheme": "deltaSPH", "densityScheme": diffusion, "alpha": alpha, "delta": delta,
                      "kinematic": kinematic, "boundaryDiffusion": boundary_diffusion},
        "integration": {"scheme": integration, "dt": dt},
        "fluid": {"restDensity": rho0, "c0": c0},
        "gravity": {"magnitude": gravity, "direction": [0, -1], "pointSource": point_source, "potentialField": True,
                    "center": [float(point_center[0]), float(point_center[1])]},
        "timestep": {"fixed": cfl_fixed, "min": dt if cfl_fixed else 1e-6, "max": dt if cfl_fixed else 1e-2,
                     "CFLNumber": 0.4},
        "domain": {"min": [0.0, 0.0], "max": [W, H], "adjustDomain": False, "adjustParticle": False},
        "compute": {"device": "cpu", "floatprecision": "single"},
        "export": {"active": False, "staticBoundary": True},
        "shifting": {"enabled": False, "scheme": "deltaPlus"},
        "periodicBC": {"periodicX": False, "periodicY": False, "buffer": 2},
        "solidBoundary": {"layers": 3},
        "kernel": {"targetNeighbors": 9 * math.pi},
    }
    if dfsph:
        cfg["dfsph"] = dict(dfsph)
    return cfg


def _derive(cfg, scene, sb):
    """What SPHSimulation.__init__ derives (src/simulationBase.py:832-979), set exactly."""
    sim_params = sb.SPHSimulation.getBasicParameters(None)
    for p in sim_params:
        p.parseConfig(cfg)
    cfg["compute"]["precision"] = torch.float32
    cfg["compute"]["maxValue"] = torch.finfo(torch.float32).max
    dx = scene["dx"]
    h = np.float32(scene["h"])
    cfg["particle"]["area"] = np.float32(dx * dx)
    cfg["particle"]["support"] = h
    cfg["particle"]["packing"] = dx / float(h)
    cfg["particle"]["spacing"] = cfg["particle"]["packing"]
    buf = float(h) * cfg["periodicBC"]["buffer"]
    dmin = np.array(cfg["domain"]["min"], dtype=np.float64)
    dmax = np.array(cfg["domain"]["max"], dtype=np.float64)
    cfg["domain"]["virtualMin"] = dmin - buf
    cfg["domain"]["virtualMax"] = dmax + buf
    W, H = scene["tank"]
    cfg["solidBC"] = {"domainBoundary": {"vertices": [[0.0, 0.0], [W, 0.0], [W, H], [0.0, H]], "inverted": True}}
    cfg["solidBC"]["domainBoundary"]["polygon"] = torch.tensor(cfg["solidBC"]["domainBoundary"]["vertices"],
                                                               dtype=torch.float32)
    return sim_params


class _Float32Search:
    """The reference's neighbor-search extension takes float32 tensors only (accessor<float>);
    for a float64 run of the reference's summations the positions are handed to it as float32
    (exact: the scene's positions are float32 values)."""

    def __init__(self, ext):
        self.ext = ext

    def __getattr__(self, name):
        fn = getattr(self.ext, name)

        def call(*args):
            args = [a.to(torch.float32) if isinstance(a, torch.Tensor) and a.dtype == torch.float64 else a
                    for a in args]
            return fn(*args)
        return call


def _precompute_mls_renamed(util):
    """precomputeMLS (src/util.py:332-384) with its local `kernel` renamed.

    The reference assigns `kernel = kernel(radialDistances, support)` inside the function that
    calls the module-level `kernel` (:357), so every call raises UnboundLocalError and the
    ghostMLS / deltaMLS wall pressures cannot run.  This recompiles the reference's own source
    with every use of that local (not the call) renamed; nothing else changes."""
    import ast
    import inspect
    import textwrap
    tree = ast.parse(textwrap.dedent(inspect.getsource(util.precomputeMLS)))
    fn = tree.body[0]
    fn.decorator_list = []
    called = {id(c.func) for c in ast.walk(fn) if isinstance(c, ast.Call) and isinstance(c.func, ast.Name)}
    for node in ast.walk(fn):
        if isinstance(node, ast.Name) and node.id == "kernel" and id(node) not in called:
            node.id = "kernelValue"
    out = {}
    exec(compile(ast.fix_missing_locations(tree), util.__file__, "exec"), util.__dict__, out)
    return out["precomputeMLS"]


class _FluidVolumeView:
    """solidBoundary.py:782 reads `self.deltaSPH.fluidVolume`, an attribute nothing in the
    reference sets (MLSPressure raises AttributeError there); the harness points it at the
    state's fluidVolume, the fluid's area that evalMLSBoundaries is given right after (:802)."""

    def __init__(self, sim):
        self.sim = sim

    @property
    def fluidVolume(self):
        return self.sim.simulationState["fluidVolume"]


def make_simulation(scene, precision="single", **kw):
    """A reference simulation object around `scene`, initialised like initializeSimulation.
    precision="double" runs the reference's own summations in float64."""
    R, deltaSPH, dfsph, sb = _modules()
    cfg = base_config(scene, **kw)
    params = _derive(cfg, scene, sb)
    dtype = torch.float64 if precision == "double" else torch.float32
    cfg["compute"]["precision"] = dtype
    cfg["compute"]["floatprecision"] = precision
    poly = cfg["solidBC"]["domainBoundary"]
    poly["polygon"] = poly["polygon"].to(dtype)
    if precision == "double":
        if not isinstance(R.neighborSearch.neighborSearch, _Float32Search):
            R.neighborSearch.neighborSearch = _Float32Search(R.neighborSearch.neighborSearch)
    elif isinstance(R.neighborSearch.neighborSearch, _Float32Search):
        R.neighborSearch.neighborSearch = R.neighborSearch.neighborSearch.ext
    cls = dfsph.dfsphSimulation if cfg["simulation"]["scheme"] == "dfsph" else deltaSPH.deltaSPHSimulation

    orig_init = sb.SPHSimulation.__init__

    def light_init(self, config):
        self.verbose = False
        self.config = config
        self.parameters = params
        self.kernel, self.kernelGrad = R.kernels.getKernelFunctions("wendland2")
        self.dtype = dtype
        self.device = "cpu"

    sb.SPHSimulation.__init__ = light_init
    try:
        sim = cls(cfg)
    finally:
        sb.SPHSimulation.__init__ = orig_init

    # wall layers from the scene instead of skimage contours
    from pytorchsph_gb300 import workloads
    dx = scene["dx"]
    W, H = scene["tank"]
    layers = {}
    for k in range(cfg["solidBoundary"]["layers"]):
        layers[k] = workloads.tank_walls(W, H, dx, layers=k + 1)
    counts = [0] + [len(layers[k][0]) for k in range(len(layers))]

    def sample_polygon(poly, spacing, support, offset=0, mirrored=False, inverted=False):
        k = int(round(offset / dx - 0.5))
        w, g = layers[k]
        w, g = w[counts[k]:], g[counts[k]:]
        return w.astype(np.float64), torch.from_numpy(g).to(dtype)

    R.solidBoundary.samplePolygon = sample_polygon
    if cfg["pressure"]["boundaryPressureTerm"] in ("ghostMLS", "deltaMLS"):
        R.solidBoundary.precomputeMLS = _precompute_mls_renamed(R.util)

    n = len(scene["pos"])
    T = lambda a: torch.from_numpy(a.copy()).to(dtype)
    st = {
        "fluidPosition": T(scene["pos"]),
        "UID": torch.arange(n, dtype=torch.int64),
        "ghostIndices": torch.full((n,), -1, dtype=torch.int64),
        "fluidDensity": T(scene["rho"]),
        "fluidArea": T(scene["area"]),
        "fluidSupport": T(scene["support"]),
        "fluidVelocity": T(scene["vel"]),
        "fluidAcceleration": torch.zeros(n, 2, dtype=dtype),
        "fluidPressure": torch.zeros(n, dtype=dtype),
        "fluidRestDensity": torch.full((n,), float(cfg["fluid"]["restDensity"]), dtype=dtype),
        "dpdt": torch.zeros(n, dtype=dtype),
        "numParticles": n, "realParticles": n, "time": 0.0, "timestep": 0,
        "dt": cfg["integration"]["dt"],
    }
    sim.simulationState = st
    for m in sim.modules:
        m.initialize(sim.config, sim.simulationState)
    sim.perennialState = sim.saveState(copy=False)
    sim.simulationState = sim.setupSimulationState(sim.perennialState)
    # walls must be exactly the scene's (the reference keeps its own copies)
    bm = sim.boundaryModule
    if cfg["pressure"]["boundaryPressureTerm"] == "MLSPressure":
        bm.deltaSPH = _FluidVolumeView(sim)
    assert np.array_equal(bm.boundaryPositions.to(torch.float32).numpy(), scene["wall_pos"])
    return sim


def snapshot(sim):
    s = sim.simulationState
    out = {k: s[k].detach().clone().numpy() for k in ("fluidPosition", "fluidVelocity", "fluidDensity")}
    for k in ("dpdt", "fluidAcceleration", "fluidPressure", "fluidAlpha", "fluidSourceTerm"):
        if k in s and isinstance(s[k], torch.Tensor):
            out[k] = s[k].detach().clone().numpy()
    bm = sim.boundaryModule
    out["boundaryDensity"] = bm.boundaryDensity.detach().clone().numpy()
    if isinstance(getattr(bm, "pressure", None), torch.Tensor):
        out["boundaryPressure"] = bm.pressure.detach().clone().numpy()
    out["dt"] = float(s["dt"])
    for k in ("densityIterations", "divergenceIterations"):
        if k in s:
            out[k] = np.asarray(s[k], np.float64)
    return out
