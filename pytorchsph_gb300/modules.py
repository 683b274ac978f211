"""The reference's Module interface (src/module.py) for the neighbor search and the deltaSPH
summations, computed by the GB300 kernels.

Each class has the reference module's name, constructor, `getParameters`, `initialize`
(reading the same configuration keys), `resetState` (dropping the same state keys) and hot
methods with the same signatures and the same simulationState reads and writes, so a
reference driver (`deltaSPHSimulation.timestep`, src/deltaSPH.py:146-200) runs unchanged
with these modules in place of its own.  Wall contributions still come from
`simulation.boundaryModule`, as in the reference.

The arrays stay torch CUDA tensors in original particle order; every summation is one
kernel launch over the (i, j)-ordered pair list (`sph_pair_term`), with no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from .search import GridSearch
from .sim import SphParamsC


class Parameter:
    """A configuration parameter (src/parameter.py:3-22)."""

    def __init__(self, namespace, name, datatype, defaultValue, required=False, hint='', export=True):
        self.namespace = namespace
        self.name = name
        self.datatype = datatype
        self.defaultValue = defaultValue
        self.required = required
        self.hint = hint
        self.export = export

    def parseConfig(self, config):
        if self.required and self.namespace not in config:
            raise Exception('Parameter Namespace %s missing for required parameter %s.%s' %
                            (self.namespace, self.namespace, self.name))
        config.setdefault(self.namespace, {})
        if self.required and self.name not in config[self.namespace]:
            raise Exception('Required parameter %s.%s is missing' % (self.namespace, self.name))
        config[self.namespace].setdefault(self.name, self.defaultValue)


class Module:
    """Base class of all modules (src/module.py:4-24): every hook is a no-op by default."""

    def getParameters(self):
        return None

    def initialize(self, config, state):
        return

    def finalize(self):
        return

    def resetState(self, simulationState):
        return

    def saveState(self, perennialState, copy):
        return

    def exportState(self, simulationState, simulation, group, mask):
        return

    def setupSimulationState(self, perennialState):
        return

    def __init__(self, identifier, moduleDescription):
        self.description = moduleDescription
        self.name = identifier


class BoundaryModule(Module):
    """Boundary hooks the solvers require (src/module.py:27-56); unimplemented ones raise."""

    def __init__(self, identifier, moduleDescription):
        super().__init__(identifier, moduleDescription)

    def _missing(self, what):
        raise Exception('Operation %s not implemented for ' % what, self.name)

    def dfsphPrepareSolver(self, simulationState, simulation, density):
        self._missing('dfsphPrepareSolver')

    def dfsphBoundaryAccelTerm(self, simulationState, simulation, density):
        self._missing('dfsphBoundaryAccelTerm')

    def dfsphBoundaryPressureSum(self, simulationState, simulation, density):
        self._missing('dfsphBoundaryPressureSum')

    def dfsphBoundaryAlphaTerm(self, simulationState, simulation, density):
        self._missing('dfsphBoundaryAlphaTerm')

    def dfsphBoundarySourceTerm(self, simulationState, simulation, density):
        self._missing('dfsphBoundarySourceTerm')

    def evalBoundaryPressure(self, simulationState, simulation, density):
        self._missing('boundaryPressure')

    def evalBoundaryDensity(self, simulationState, simulation):
        self._missing('boundaryDensity')

    def evalBoundaryFriction(self, simulationState, simulation):
        self._missing('boundaryFriction')

    def boundaryNeighborhoodSearch(self, simulationState, simulation):
        self._missing('boundaryNeighborsearch')

    def boundaryFilterNeighborhoods(self, simulationState, simulation):
        return


# ----------------------------------------------------------------------------- kernel plumbing
class PairTermsC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("offsets", "cols", "dist", "radial", "pos", "vel", "rho", "volume",
                                                "area", "pressure", "L", "grad_rho", "actual_area", "pred_accel",
                                                "pred_vel")] + [("dt", ctypes.c_double), ("n", ctypes.c_int64)]


class WallTermsC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in (
        "wall_offsets", "rows", "cols", "dist", "radial", "fluid_offsets", "fluid_pairs", "pos", "vel", "rho", "area",
        "volume", "pressure", "L", "actual_area", "pred_accel", "pred_vel", "wall_pos", "wall_ghost", "wall_area",
        "wall_rho", "wall_volume", "wall_pressure", "wall_actual_area", "wall_term")] + [
        ("dt", ctypes.c_double), ("n", ctypes.c_int64), ("nb", ctypes.c_int64)]


TERM = {"density": 0, "divergence": 1, "mog": 2, "normalization": 3, "renormalized_gradient": 4,
        "delta_diffusion": 5, "pressure_accel": 6, "velocity_diffusion": 7, "laminar": 8, "dfsph_alpha": 9,
        "dfsph_source": 10, "dfsph_pressure_sum": 11, "dfsph_accel": 12}
WALL = {"density": 0, "dpdt": 1, "normalization": 2, "renormalized_gradient": 3, "pressure_accel": 4,
        "velocity_diffusion": 5, "dfsph_alpha": 6, "dfsph_source": 7, "dfsph_pressure_sum": 8, "dfsph_accel": 9,
        "b_density": 20, "b_mdbc": 21, "b_dfsph_alpha": 22, "b_dfsph_source": 23, "b_dfsph_pressure_sum": 24,
        "b_ghost_mls_pressure": 25, "b_delta_mls_pressure": 26, "b_mls_pressure": 27}
WALL_WIDTH = {"density": 1, "dpdt": 1, "normalization": 4, "renormalized_gradient": 2, "pressure_accel": 2,
              "velocity_diffusion": 2, "dfsph_alpha": 4, "dfsph_source": 1, "dfsph_pressure_sum": 1,
              "dfsph_accel": 2}
OP = {"tait": 0, "volume": 1, "pinv2x2": 2, "gravity": 3}
WIDTH = {"density": 1, "divergence": 1, "mog": 1, "normalization": 4, "renormalized_gradient": 2,
         "delta_diffusion": 1, "pressure_accel": 2, "velocity_diffusion": 2, "laminar": 2, "dfsph_alpha": 4,
         "dfsph_source": 1, "dfsph_pressure_sum": 1, "dfsph_accel": 2}


def _f32(t):
    if t is None:
        return None
    if not (t.is_cuda and t.dtype == torch.float32):
        raise N.SPHError("module state arrays must be float32 CUDA tensors")
    return t.contiguous()


def _params(support, restDensity=1000.0, c0=10.0, gamma=7.0, alpha=0.01, delta=0.1, kinematic=0.01,
            gravity=(0.0, 0.0), pointSource=False, magnitude=1.0, center=(0.0, 0.0)):
    P = SphParamsC()
    P.support = float(support)
    P.rest_density = float(restDensity)
    P.c0 = float(c0)
    P.gamma = float(gamma)
    P.alpha = float(alpha)
    P.delta = float(delta)
    P.kinematic = float(kinematic)
    P.gravity[0], P.gravity[1] = float(gravity[0]), float(gravity[1])
    P.point_source = int(bool(pointSource))
    P.point_magnitude = float(magnitude)
    P.point_center[0], P.point_center[1] = float(center[0]), float(center[1])
    P.search_radius = 1
    return P


def row_offsets(simulationState):
    """int32 [n+1] row offsets of fluidNeighbors (kept in the state beside the pairs)."""
    nb = simulationState['fluidNeighbors']
    n = simulationState['fluidPosition'].shape[0]
    cached = simulationState.get('fluidNeighborOffsets')
    if cached is not None and cached.shape[0] == n + 1:
        return cached
    rows = nb[0].contiguous()
    off = torch.empty(n + 1, dtype=torch.int32, device=rows.device)
    N.call("sph_row_offsets", N.ptr(rows), rows.shape[0], n, N.ptr(off), N.stream_ptr())
    simulationState['fluidNeighborOffsets'] = off
    return off


def pair_term(term, simulationState, P, pressure=None, L=None, grad_rho=None, out=None, accumulate=False,
              actual_area=None, pred_accel=None, pred_vel=None, dt=0.0):
    """One summation of `term` over the state's pairs; returns [n], [n,2] or [n,2,2]."""
    st = simulationState
    n = st['fluidPosition'].shape[0]
    off = row_offsets(st)
    nb = st['fluidNeighbors']
    cols = nb[1].contiguous()
    vol = st.get('fluidVolume')
    keep = [off, cols]
    arrays = {"dist": st.get('fluidDistances'), "radial": st.get('fluidRadialDistances'),
              "pos": st.get('fluidPosition'), "vel": st.get('fluidVelocity'), "rho": st.get('fluidDensity'),
              "volume": vol, "area": st.get('fluidArea'), "pressure": pressure, "L": L, "grad_rho": grad_rho,
              "actual_area": actual_area, "pred_accel": pred_accel, "pred_vel": pred_vel}
    ptrs = {}
    for k, t in arrays.items():
        t = _f32(t)
        keep.append(t)
        ptrs[k] = N.ptr(t)
    inp = PairTermsC(N.ptr(off), N.ptr(cols), *[ptrs[k] for k in (
        "dist", "radial", "pos", "vel", "rho", "volume", "area", "pressure", "L", "grad_rho", "actual_area",
        "pred_accel", "pred_vel")], float(dt), n)
    w = WIDTH[term]
    if out is None:
        out = torch.zeros((n,) if w == 1 else (n, w), dtype=torch.float32, device=st['fluidPosition'].device)
    N.call("sph_pair_term", TERM[term], ctypes.byref(inp), ctypes.byref(P), N.ptr(out), int(accumulate),
           N.stream_ptr())
    return out.view(n, 2, 2) if term == "normalization" else out


def particle_op(op, a, b, P, out, accumulate=False):
    a = _f32(a)
    b = _f32(b)
    N.call("sph_particle_op", OP[op], a.shape[0], N.ptr(a), N.ptr(b), ctypes.byref(P), N.ptr(out), int(accumulate),
           N.stream_ptr())
    return out


def _c0(cfg):
    """The c0 default every deltaSPH module applies (e.g. src/modules/momentum.py:62-67)."""
    if cfg['fluid']['c0'] < 0:
        cfg['fluid']['c0'] = 10.0 * np.sqrt(2.0 * 9.81 * 0.3)
    return cfg['fluid']['c0']


class _SummationModule(Module):
    """Shared configuration of the summation modules (the keys their initialize reads)."""

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')

    def initialize(self, simulationConfig, simulationState):
        cfg = simulationConfig
        self.support = cfg['particle']['support']
        self.restDensity = cfg['fluid']['restDensity']
        self.gamma = cfg['pressure']['gamma']
        self.dtype = cfg['compute']['precision']
        self.device = cfg['compute']['device']
        self.alpha = cfg['diffusion']['alpha']
        self.delta = cfg['diffusion']['delta']
        self.c0 = _c0(cfg)
        self.eps = self.support ** 2 * 0.1
        self.kinematic = cfg['diffusion'].get('kinematic', 0.01)
        self.P = _params(self.support, self.restDensity, self.c0, self.gamma, self.alpha, self.delta, self.kinematic)


# ----------------------------------------------------------------------------- neighbor search
class neighborSearchModule(Module):
    """src/modules/neighborSearch.py:174-252 on the GB300 search (sorted SoA + CSR inside)."""

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')

    def getParameters(self):
        return [
            Parameter('neighborSearch', 'gradientThreshold', 'float', 1e-7, required=False, export=True, hint=''),
            Parameter('neighborSearch', 'supportScale', 'float', 1.0, required=False, export=True, hint=''),
            Parameter('neighborSearch', 'sortNeighborhoods', 'bool', True, required=False, export=True, hint=''),
        ]

    def initialize(self, simulationConfig, simulationState):
        self.support = simulationConfig['particle']['support']
        self.maxNeighbors = simulationConfig['compute']['maxNeighbors']
        self.threshold = simulationConfig['neighborSearch']['gradientThreshold']
        self.supportScale = simulationConfig['neighborSearch']['supportScale']
        self.sortNeighborhoods = simulationConfig['neighborSearch']['sortNeighborhoods']
        self.dtype = simulationConfig['compute']['precision']
        self.device = simulationConfig['compute']['device']
        self.minDomain = simulationConfig['domain']['virtualMin']
        self.maxDomain = simulationConfig['domain']['virtualMax']
        self.engine = None
        self.csr = None

    def resetState(self, simulationState):
        simulationState.pop('fluidNeighbors', None)
        simulationState.pop('fluidDistances', None)
        simulationState.pop('fluidRadialDistances', None)
        simulationState.pop('fluidNeighborOffsets', None)

    def search(self, simulationState, simulation):
        pos = _f32(simulationState['fluidPosition'])
        sup = _f32(simulationState['fluidSupport'])
        if self.engine is None:
            self.engine = GridSearch(pos.device)
        self.csr = self.engine.run(pos, sup, kernel_support=float(self.support), density=False,
                                   min_coord=np.asarray(self.minDomain, np.float32),
                                   max_coord=np.asarray(self.maxDomain, np.float32))
        fluidNeighbors, fluidDistances, fluidRadialDistances = self.csr.to_coo(self.threshold)
        simulationState['fluidNeighbors'] = fluidNeighbors
        simulationState['fluidDistances'] = fluidDistances
        simulationState['fluidRadialDistances'] = fluidRadialDistances
        simulationState.pop('fluidNeighborOffsets', None)
        row_offsets(simulationState)
        return fluidNeighbors, fluidDistances, fluidRadialDistances

    def searchExisting(self, queryPositions, querySupports, simulationState, simulation, searchRadius: int = 1):
        if self.csr is None:
            raise N.SPHError("searchExisting needs a prior search() of the fluid")
        q = _f32(queryPositions)
        hq = _f32(querySupports)
        rows, cols = self.csr.query(q, hq, searchRadius)
        P = rows.shape[0]
        dist = torch.empty((P, 2), dtype=torch.float32, device=q.device)
        radial = torch.empty(P, dtype=torch.float32, device=q.device)
        N.call("sph_pair_geometry", N.ptr(rows), N.ptr(cols), P, N.ptr(q),
               N.ptr(_f32(simulationState['fluidPosition'])), N.ptr(hq), float(self.threshold), N.ptr(dist),
               N.ptr(radial), N.stream_ptr())
        fluidNeighbors = torch.stack([rows.long(), cols.long()], dim=0)
        return fluidNeighbors, dist, radial


# ----------------------------------------------------------------------------- summations
class densityModule(Module):
    """src/modules/density.py:33-55."""

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')

    def initialize(self, simulationConfig, simulationState):
        self.support = simulationConfig['particle']['support']
        self.scheme = simulationConfig['simulation']['densityScheme']
        self.P = _params(self.support)

    def resetState(self, simulationState):
        simulationState.pop('fluidVolume', None)

    def evaluate(self, simulationState, simulation):
        if self.scheme == 'summation':
            simulationState['fluidDensity'] = pair_term("density", simulationState, self.P)
        area = simulationState['fluidArea']
        vol = torch.empty_like(area)
        simulationState['fluidVolume'] = particle_op("volume", area, simulationState['fluidDensity'], self.P, vol)


class momentumModule(_SummationModule):
    """src/modules/momentum.py:41-90: dpdt = continuity (+ walls)."""

    def resetState(self, simulationState):
        self.divergenceTerm = None
        self.dpdt = None
        simulationState.pop('dpdt', None)

    def computeDpDt(self, simulationState, simulation):
        self.divergenceTerm = pair_term("divergence", simulationState, self.P)
        self.divergenceTerm += simulation.boundaryModule.computeDpDt(simulationState, simulation)
        self.dpdt = self.divergenceTerm
        simulationState['dpdt'] = self.dpdt
        simulation.sync(simulationState['dpdt'])


class densityDiffusionModule(_SummationModule):
    """src/modules/densityDiffusion.py:86-180: MOG or renormalized deltaSPH density diffusion."""

    def getParameters(self):
        return [Parameter('deltaSPH', 'HughesGrahamCorrection', 'bool', True, required=False, export=True, hint='')]

    def initialize(self, simulationConfig, simulationState):
        super().initialize(simulationConfig, simulationState)
        self.scheme = simulationConfig['diffusion']['densityScheme']

    def resetState(self, simulationState):
        self.normalizationMatrix = None
        self.fluidL = None
        self.eigVals = None
        self.densityDiffusion = None

    def computeNormalizationMatrices(self, simulationState, simulation):
        self.normalizationMatrix = pair_term("normalization", simulationState, self.P)
        self.normalizationMatrix += simulation.boundaryModule.computeNormalizationMatrices(simulationState, simulation)
        self.fluidL, self.eigVals = pinv2x2(self.normalizationMatrix, self.P)

    def computeRenormalizedDensityGradient(self, simulationState, simulation):
        n = self.fluidL.shape[0]
        self.renormalizedGrad = None   # per-pair L_i gradW is folded into the row sums
        self.renormalizedDensityGradient = pair_term("renormalized_gradient", simulationState, self.P,
                                                     L=self.fluidL.reshape(n, 4))
        self.renormalizedDensityGradient += simulation.boundaryModule.computeRenormalizedDensityGradient(
            simulationState, simulation)

    def computeDensityDiffusion(self, simulationState, simulation):
        if self.scheme == 'deltaSPH':
            if 'fluidL' in simulationState:
                self.normalizationMatrix = simulationState['normalizationMatrix']
                self.fluidL = simulationState['fluidL']
                self.eigVals = simulationState['eigVals']
            else:
                self.computeNormalizationMatrices(simulationState, simulation)
            self.computeRenormalizedDensityGradient(simulationState, simulation)
            self.densityDiffusion = pair_term("delta_diffusion", simulationState, self.P,
                                              grad_rho=self.renormalizedDensityGradient)
            simulationState['dpdt'] += self.densityDiffusion
        elif self.scheme == 'MOG':
            self.densityDiffusion = pair_term("mog", simulationState, self.P)
            simulationState['dpdt'] += self.densityDiffusion
        simulation.sync(simulationState['dpdt'])


class pressureModule(_SummationModule):
    """src/modules/pressure.py:54-140: Tait pressure and the pressure acceleration."""

    def getParameters(self):
        return [Parameter('pressure', 'HughesGrahamCorrection', 'bool', True, required=False, export=True, hint='')]

    def initialize(self, simulationConfig, simulationState):
        super().initialize(simulationConfig, simulationState)
        self.kappa = simulationConfig['pressure']['kappa']
        self.simulationScheme = simulationConfig['simulation']['scheme']
        self.fluidPressureScheme = simulationConfig['pressure']['fluidPressureTerm']

    def resetState(self, simulationState):
        self.pressure = None
        self.pressureAccel = None

    def computePressure(self, simulationState, simulation):
        if self.fluidPressureScheme != "TaitEOS":
            raise N.SPHError("pressureModule: only the TaitEOS pressure term runs on this path")
        rho = simulationState['fluidDensity']
        self.pressure = particle_op("tait", rho, None, self.P, torch.empty_like(rho))
        simulation.boundaryModule.computePressure(simulationState, simulation)
        simulationState['fluidPressure'] = self.pressure
        simulation.sync(simulationState['fluidPressure'])
        return self.pressure

    def computePressureAcceleration(self, simulationState, simulation):
        st = simulationState
        if self.simulationScheme == 'deltaPlus':     # computePressureAccelDeltaPlus (pressure.py:31-51)
            n = st['fluidPosition'].shape[0]
            self.pressureAccel = torch.empty((n, 2), dtype=torch.float32, device=st['fluidPosition'].device)
            surface_term("pressure_accel", self.P, n, out=self.pressureAccel, fluid=st, pressure=self.pressure,
                         mask=st['fluidSurfaceMask'], volume=st['fluidVolume'], rho=st['fluidDensity'])
        else:
            self.pressureAccel = pair_term("pressure_accel", st, self.P, pressure=self.pressure)
        self.pressureAccel += simulation.boundaryModule.computePressureAcceleration(simulationState, simulation)
        simulationState['fluidAcceleration'] += self.pressureAccel
        simulation.sync(simulationState['fluidAcceleration'])


class diffusionModule(_SummationModule):
    """src/modules/diffusion.py:47-93: artificial viscosity (+ walls when boundaryDiffusion)."""

    def initialize(self, simulationConfig, simulationState):
        super().initialize(simulationConfig, simulationState)
        self.boundaryDiffusion = simulationConfig['diffusion']['boundaryDiffusion']

    def resetState(self, simulationState):
        self.velocityDiffusion = None

    def evaluate(self, simulationState, simulation):
        self.velocityDiffusion = pair_term("velocity_diffusion", simulationState, self.P)
        if self.boundaryDiffusion:
            self.velocityDiffusion += simulation.boundaryModule.computeVelocityDiffusion(simulationState, simulation)
        simulationState['fluidAcceleration'] += self.velocityDiffusion
        simulation.sync(simulationState['fluidAcceleration'])


class laminarViscosityModule(_SummationModule):
    """src/modules/laminar.py:49-100."""

    def initialize(self, simulationConfig, simulationState):
        super().initialize(simulationConfig, simulationState)
        self.boundaryDiffusion = simulationConfig['diffusion']['boundaryDiffusion']
        self.kinematic = simulationConfig['diffusion']['kinematic']
        self.P = _params(self.support, self.restDensity, self.c0, self.gamma, self.alpha, self.delta, self.kinematic)

    def resetState(self, simulationState):
        self.laminarViscosity = None

    def computeLaminarViscosity(self, simulationState, simulation):
        self.laminarViscosity = pair_term("laminar", simulationState, self.P)
        simulationState['fluidAcceleration'] += self.laminarViscosity
        simulation.sync(simulationState['fluidAcceleration'])


class gravityModule(Module):
    """src/modules/gravity.py:23-57: constant gravity or the point source (potential field)."""

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')

    def getParameters(self):
        return [
            Parameter('gravity', 'magnitude', 'float', 9.81, required=False, export=True, hint=''),
            Parameter('gravity', 'direction', 'float array', [0, -1], required=False, export=True, hint=''),
            Parameter('gravity', 'pointSource', 'bool', False, required=False, export=True, hint=''),
            Parameter('gravity', 'potentialField', 'bool', True, required=False, export=True, hint=''),
            Parameter('gravity', 'center', 'float array', [0, 0], required=False, export=True, hint=''),
        ]

    def initialize(self, simulationConfig, simulationState):
        g = simulationConfig['gravity']
        self.magnitude = g['magnitude']
        self.direction = g['direction']
        self.pointSource = g['pointSource']
        self.potentialField = g['potentialField']
        self.center = g['center']
        self.dtype = simulationConfig['compute']['precision']
        self.device = simulationConfig['compute']['device']
        if self.pointSource and not self.potentialField:
            raise N.SPHError("gravityModule: the point source runs as a potential field on this path")
        self.P = _params(1.0, gravity=(self.magnitude * self.direction[0], self.magnitude * self.direction[1]),
                         pointSource=self.pointSource, magnitude=self.magnitude, center=self.center)

    def evaluate(self, simulationState, simulation):
        particle_op("gravity", simulationState['fluidPosition'], None, self.P, simulationState['fluidAcceleration'])


# ----------------------------------------------------------------------------- solid walls
class _WallPairs:
    """A wall -> fluid pair list of searchExisting (rows = wall, cols = fluid particle) with
    its grouping by wall (row offsets) and by fluid particle (sph_transpose_pairs)."""

    def __init__(self, neighbors, dist, radial, nb, n):
        self.rows = neighbors[0].contiguous()
        self.cols = neighbors[1].contiguous()
        self.dist = _f32(dist)
        self.radial = _f32(radial)
        P = self.rows.shape[0]
        dev = self.rows.device
        st = N.stream_ptr()
        self.woff = torch.empty(nb + 1, dtype=torch.int32, device=dev)
        N.call("sph_row_offsets", N.ptr(self.rows), P, nb, N.ptr(self.woff), st)
        self.foff = torch.empty(n + 1, dtype=torch.int32, device=dev)
        self.fpairs = torch.empty(max(P, 1), dtype=torch.int32, device=dev)
        scr = torch.empty((N.load().sph_transpose_pairs_scratch_bytes(n) + 7) // 8, dtype=torch.int64, device=dev)
        N.call("sph_transpose_pairs", N.ptr(self.cols), P, n, N.ptr(self.foff), N.ptr(self.fpairs), N.ptr(scr),
               scr.numel() * 8, st)


def wall_term(term, pairs, P, n, nb, out=None, accumulate=False, dt=0.0, **arrays):
    """One wall sum (sph_wall_term): fluid side -> [n], [n,2] or [n,4]; wall side -> [nb]."""
    keep = {k: _f32(v) for k, v in arrays.items()}
    names = ("pos", "vel", "rho", "area", "volume", "pressure", "L", "actual_area", "pred_accel", "pred_vel",
             "wall_pos", "wall_ghost", "wall_area", "wall_rho", "wall_volume", "wall_pressure", "wall_actual_area",
             "wall_term")
    unknown = set(keep) - set(names)
    if unknown:
        raise N.SPHError(f"wall_term: unknown arrays {sorted(unknown)}")
    inp = WallTermsC(N.ptr(pairs.woff), N.ptr(pairs.rows), N.ptr(pairs.cols), N.ptr(pairs.dist),
                     N.ptr(pairs.radial), N.ptr(pairs.foff), N.ptr(pairs.fpairs),
                     *[N.ptr(keep.get(k)) for k in names], float(dt), n, nb)
    if out is None:
        dev = pairs.rows.device
        if WALL[term] >= 20:
            out = torch.zeros(nb, dtype=torch.float32, device=dev)
        else:
            w = WALL_WIDTH[term]
            out = torch.zeros((n,) if w == 1 else (n, w), dtype=torch.float32, device=dev)
    N.call("sph_wall_term", WALL[term], ctypes.byref(inp), ctypes.byref(P), N.ptr(out), int(accumulate),
           N.stream_ptr())
    return out


class SurfaceC(ctypes.Structure):
    """sph_surface_in (include/sph_gb300.h)."""
    _fields_ = [(k, ctypes.c_void_p) for k in (
        "offsets", "cols", "dist", "radial", "wall_offsets", "wall_rows", "wall_cols", "wall_dist", "wall_radial",
        "fluid_wall_offsets", "fluid_wall_pairs", "ww_offsets", "ww_cols", "ww_dist", "ww_radial", "pos", "vel",
        "rho", "area", "volume", "matrix", "L", "lambda_", "normal", "mask", "shift", "wall_pos", "wall_area",
        "wall_rho", "wall_volume", "wall_lambda", "pressure", "wall_pressure")] + [
        ("packing", ctypes.c_float), ("cfl", ctypes.c_float), ("n", ctypes.c_int64), ("nb", ctypes.c_int64)]


SURF = {"pinv_eig": 0, "wall_normalization": 1, "normal": 2, "angle_mask": 3, "classify": 4, "shift": 5,
        "shift_adjust": 6, "pressure_accel": 7, "wall_pressure_accel": 8}


def surface_term(term, P, n, nb=0, out=None, out2=None, fluid=None, walls=None, wall_walls=None, packing=0.0,
                 cfl=1.5, **arrays):
    """One call of sph_surface_term.  fluid: the state whose fluidNeighbors / distances give
    the fluid pairs; walls: a _WallPairs (wall -> fluid); wall_walls: (offsets, cols, dist,
    radial) of the wall-wall pairs; arrays: the named per-particle arrays."""
    keep = []
    ptr = {}
    if fluid is not None:
        off = row_offsets(fluid)
        cols = fluid['fluidNeighbors'][1].contiguous()
        keep += [off, cols]
        ptr.update(offsets=N.ptr(off), cols=N.ptr(cols), dist=N.ptr(_f32(fluid['fluidDistances'])),
                   radial=N.ptr(_f32(fluid['fluidRadialDistances'])))
    if walls is not None:
        ptr.update(wall_offsets=N.ptr(walls.woff), wall_rows=N.ptr(walls.rows), wall_cols=N.ptr(walls.cols),
                   wall_dist=N.ptr(walls.dist), wall_radial=N.ptr(walls.radial), fluid_wall_offsets=N.ptr(walls.foff),
                   fluid_wall_pairs=N.ptr(walls.fpairs))
    if wall_walls is not None:
        wo, wc, wd, wr = wall_walls
        ptr.update(ww_offsets=N.ptr(wo), ww_cols=N.ptr(wc), ww_dist=N.ptr(_f32(wd)), ww_radial=N.ptr(_f32(wr)))
    for k, v in arrays.items():
        name = "lambda_" if k in ("lambda", "lambda_") else k
        if name not in [f[0] for f in SurfaceC._fields_]:
            raise N.SPHError(f"surface_term: unknown array {k}")
        t = _f32(v.reshape(-1) if v is not None else None)
        keep.append(t)
        ptr[name] = N.ptr(t)
    inp = SurfaceC(**ptr, packing=float(packing), cfl=float(cfl), n=int(n), nb=int(nb))
    N.call("sph_surface_term", SURF[term], ctypes.byref(inp), ctypes.byref(P), N.ptr(out), N.ptr(out2),
           N.stream_ptr())
    return out, out2


def pinv2x2(M, P):
    """(pinv2x2(M) [n,2,2], its eigVals [n,2]) of src/util.py:386-433 for matrices M [n,2,2]."""
    n = M.shape[0]
    dev = M.device
    L = torch.empty((n, 2, 2), dtype=torch.float32, device=dev)
    eig = torch.empty((n, 2), dtype=torch.float32, device=dev)
    surface_term("pinv_eig", P, n, out=L, out2=eig, matrix=M.contiguous())
    return L, eig


class solidBoundaryModule(BoundaryModule):
    """src/modules/solidBoundary.py on GPU kernels: ghost-particle solid walls with mDBC wall
    densities and the PBSPH pressure scheme (deltaSPH: continuity, L, <grad rho>, pressure
    acceleration and velocity diffusion wall parts; DFSPH: summation wall density and the
    alpha, source, pressure-sum and acceleration wall parts with the walls' own relaxed-Jacobi
    pressures).  The wall particles come as arrays through `setWalls` (positions, mirrored
    ghost positions, areas); sampling them from SDF or polygon descriptions
    (solidBoundary.py:113-211) is scene set-up, outside this path."""

    MLSscale = 1

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')
        self.active = False
        self.boundaryToFluidNeighbors = None
        self.ghostToFluidNeighbors = None

    def getParameters(self):
        return [
            Parameter('solidBoundary', 'recomputeBoundary', 'bool', False, required=False, export=True, hint=''),
            Parameter('solidBoundary', 'layers', 'int', 3, required=False, export=True, hint=''),
        ]

    def initialize(self, simulationConfig, simulationState):
        cfg = simulationConfig
        self.support = cfg['particle']['support']
        self.threshold = cfg['neighborSearch']['gradientThreshold']
        self.dtype = cfg['compute']['precision']
        self.device = cfg['compute']['device']
        self.layers = cfg['solidBoundary']['layers']
        self.recomputeBoundary = cfg['solidBoundary']['recomputeBoundary']
        self.boundaryPressureScheme = cfg['pressure']['boundaryPressureTerm']
        self.fluidPressureScheme = cfg['pressure']['fluidPressureTerm']
        self.relaxedJacobiOmega = cfg['dfsph']['relaxedJacobiOmega'] if 'dfsph' in cfg else 0.5
        self.backgroundPressure = cfg['fluid']['backgroundPressure']
        self.alpha = cfg['diffusion']['alpha']
        self.delta = cfg['diffusion']['delta']
        self.simulationDensityScheme = cfg['simulation']['densityScheme']
        self.simulationScheme = cfg['simulation']['scheme']
        self.gamma = cfg['pressure']['gamma']
        self.c0 = _c0(cfg)
        self.eps = self.support ** 2 * 0.1
        self.restDensity = cfg['fluid']['restDensity']
        if self.boundaryPressureScheme not in ('PBSPH', 'ghostMLS', 'deltaMLS', 'MLSPressure') or \
                self.fluidPressureScheme != 'TaitEOS':
            raise N.SPHError("solidBoundaryModule: the PBSPH, ghostMLS, deltaMLS and MLSPressure boundary pressures "
                             "with TaitEOS run on this path")
        self.P = _params(self.support, self.restDensity, self.c0, self.gamma, self.alpha, self.delta)

    def setWalls(self, positions, ghostPositions, volumes):
        """Wall particles (float32 CUDA [nb, 2], [nb, 2], [nb]); the walls are static."""
        self.boundaryPositions = _f32(positions)
        self.boundaryGhostPositions = _f32(ghostPositions)
        self.boundaryVolume = _f32(volumes)
        self.numPtcls = self.boundaryPositions.shape[0]
        dev = self.boundaryPositions.device
        self.boundarySupport = torch.full((self.numPtcls,), float(self.support), dtype=torch.float32, device=dev)
        self.boundaryDensity = torch.ones(self.numPtcls, dtype=torch.float32, device=dev)
        self.boundaryVelocity = torch.zeros((self.numPtcls, 2), dtype=torch.float32, device=dev)
        self.boundaryAcceleration = torch.zeros((self.numPtcls, 2), dtype=torch.float32, device=dev)
        self.boundaryRestDensity = torch.full((self.numPtcls,), float(self.restDensity), dtype=torch.float32,
                                              device=dev)
        self.staticBoundary = True
        self.active = True
        # static wall-wall density term sum_b' W A_b' (solidBoundary.py:180-200): a search of the
        # walls among themselves with the density sum fused
        res = GridSearch(dev).run(self.boundaryPositions, self.boundarySupport, self.boundaryVolume,
                                  kernel_support=float(self.support))
        self.boundaryDensityTerm = res.density()
        # the wall-wall pair lists of solidBoundary.py:180-191 from the same search, with the
        # reference's sign of the distances, (x_col - x_row) / r
        nbrs, dist, radial = res.to_coo()
        self.boundaryToBoundaryNeighbors = nbrs
        self.boundaryToBoundaryNeighborDistances = (-dist).contiguous()
        self.boundaryToBoundaryNeighborRadialDistances = radial
        ww_off = torch.empty(self.numPtcls + 1, dtype=torch.int32, device=dev)
        rows = nbrs[0].contiguous()
        N.call("sph_row_offsets", N.ptr(rows), rows.shape[0], self.numPtcls, N.ptr(ww_off), N.stream_ptr())
        self._ww = (ww_off, nbrs[1].contiguous(), self.boundaryToBoundaryNeighborDistances, radial)
        self.normalizationMatrix = None
        self.fluidL = None
        self.eigVals = None

    def resetState(self, simulationState):
        for k in ("boundaryPressure", "boundaryPressure2", "boundaryActualArea", "boundaryPredictedVelocity",
                  "boundaryResidual", "boundaryAlpha", "boundarySource", "boundaryDensityContribution",
                  "boundaryToFluidNeighbors", "boundaryToFluidNeighborDistances",
                  "boundaryToFluidNeighborRadialDistances", "ghostToFluidNeighbors", "ghostToFluidNeighborDistances",
                  "ghostToFluidNeighborRadialDistances", "fluidVolume", "pressure", "divergenceTerm", "dpdt"):
            setattr(self, k, None)

    # ------------------------------------------------------------------ neighborhoods
    def boundaryNeighborhoodSearch(self, simulationState, simulation):
        if not self.active:
            return
        n = simulationState['fluidPosition'].shape[0]
        ns = simulation.neighborSearch
        (self.boundaryToFluidNeighbors, self.boundaryToFluidNeighborDistances,
         self.boundaryToFluidNeighborRadialDistances) = ns.searchExisting(
            self.boundaryPositions, self.boundarySupport, simulationState, simulation)
        # the ghost pair list; the deltaMLS and MLSPressure wall pressures query it from the wall
        # positions instead (solidBoundary.py:639-640), and mDBC then uses those pairs too
        query = self.boundaryPositions if self.boundaryPressureScheme in ('deltaMLS', 'MLSPressure') \
            else self.boundaryGhostPositions
        (self.ghostToFluidNeighbors, self.ghostToFluidNeighborDistances,
         self.ghostToFluidNeighborRadialDistances) = ns.searchExisting(
            query, self.boundarySupport * self.MLSscale, simulationState, simulation, searchRadius=self.MLSscale)
        self._bf = _WallPairs(self.boundaryToFluidNeighbors, self.boundaryToFluidNeighborDistances,
                              self.boundaryToFluidNeighborRadialDistances, self.numPtcls, n)
        self._gf = _WallPairs(self.ghostToFluidNeighbors, self.ghostToFluidNeighborDistances,
                              self.ghostToFluidNeighborRadialDistances, self.numPtcls, n)

    def _wall_volume(self):
        out = torch.empty_like(self.boundaryVolume)
        return particle_op("volume", self.boundaryVolume, self.boundaryDensity, self.P, out)

    def _sum(self, term, st, pairs=None, out=None, **arrays):
        n = st['fluidPosition'].shape[0]
        return wall_term(term, pairs or self._bf, self.P, n, self.numPtcls, out=out,
                         dt=float(st.get('dt', 0.0)), **arrays)

    # ------------------------------------------------------------------ densities
    def evalBoundaryDensity(self, simulationState, simulation):
        if self.simulationDensityScheme == 'summation':
            self.evalBoundaryDensitySummation(simulationState, simulation)
        elif self.simulationDensityScheme == 'continuum':
            self.computeBoundaryDensitymDBC(simulationState, simulation)

    def evalBoundaryDensitySummation(self, simulationState, simulation):
        st = simulationState
        if self.boundaryToFluidNeighbors is None:
            return torch.zeros_like(st['fluidDensity'])
        self.boundaryDensityContribution = self._sum("density", st, wall_area=self.boundaryVolume)
        self.boundaryDensity = self._sum("b_density", st, area=st['fluidArea'], wall_term=self.boundaryDensityTerm)
        self.fluidVolume = self._wall_volume()
        st['fluidDensity'] += self.boundaryDensityContribution

    def computeBoundaryDensitymDBC(self, simulationState, simulation):
        st = simulationState
        self.boundaryDensity = self._sum("b_mdbc", st, pairs=self._gf, pos=st['fluidPosition'],
                                         area=st['fluidArea'], volume=st['fluidVolume'],
                                         wall_pos=self.boundaryPositions, wall_ghost=self.boundaryGhostPositions)

    # ------------------------------------------------------------------ deltaSPH wall parts
    def computeDpDt(self, simulationState, simulation):
        st = simulationState
        self.fluidVolume = self._wall_volume()
        return self._sum("dpdt", st, vel=st['fluidVelocity'], wall_volume=self.fluidVolume,
                         wall_rho=self.boundaryDensity)

    def computeNormalizationMatrices(self, simulationState, simulation):
        """solidBoundary.py:676-694: the walls' own matrices (wall -> fluid and wall -> wall
        pairs) with their pseudo-inverses and singular values, and the fluid's wall part."""
        st = simulationState
        n = st['fluidPosition'].shape[0]
        self.fluidVolume = self._wall_volume()
        M = torch.empty((self.numPtcls, 2, 2), dtype=torch.float32, device=self.boundaryPositions.device)
        surface_term("wall_normalization", self.P, n, self.numPtcls, out=M, walls=self._bf, wall_walls=self._ww,
                     pos=st['fluidPosition'], volume=st['fluidVolume'], wall_pos=self.boundaryPositions,
                     wall_volume=self.fluidVolume)
        self.normalizationMatrix = M
        self.fluidL, self.eigVals = pinv2x2(M, self.P)
        out = self._sum("normalization", st, pos=st['fluidPosition'], wall_pos=self.boundaryPositions,
                        wall_volume=self.fluidVolume)
        return out.view(n, 2, 2)

    def computeRenormalizedDensityGradient(self, simulationState, simulation):
        st = simulationState
        n = st['fluidPosition'].shape[0]
        L = simulation.densityDiffusionModule.fluidL.reshape(n, 4)
        return self._sum("renormalized_gradient", st, L=L, rho=st['fluidDensity'], wall_rho=self.boundaryDensity,
                         wall_volume=self._wall_volume())

    def computePressure(self, simulationState, simulation):
        """solidBoundary.py:772-808: PBSPH = Tait of the mDBC density; the MLS schemes
        interpolate the fluid pressure (pressureModule.pressure) at the ghost / wall position."""
        st = simulationState
        scheme = self.boundaryPressureScheme
        if scheme == 'PBSPH':
            self.pressure = particle_op("tait", self.boundaryDensity, None, self.P,
                                        torch.empty_like(self.boundaryDensity))
        elif scheme in ('ghostMLS', 'deltaMLS'):
            self.pressure = self._sum("b_ghost_mls_pressure" if scheme == 'ghostMLS' else "b_delta_mls_pressure", st,
                                      pairs=self._gf, pos=st['fluidPosition'], area=st['fluidArea'],
                                      rho=st['fluidDensity'], pressure=simulation.pressureModule.pressure,
                                      wall_pos=self.boundaryPositions, wall_ghost=self.boundaryGhostPositions)
        else:
            self.pressure = self._sum("b_mls_pressure", st, pairs=self._gf, pos=st['fluidPosition'],
                                      volume=st['fluidVolume'], pressure=simulation.pressureModule.pressure,
                                      wall_pos=self.boundaryPositions)
        return self.pressure

    def computeVelocityDiffusion(self, simulationState, simulation):
        st = simulationState
        return self._sum("velocity_diffusion", st, pos=st['fluidPosition'], vel=st['fluidVelocity'],
                         rho=st['fluidDensity'], wall_pos=self.boundaryPositions, wall_volume=self._wall_volume(),
                         wall_rho=self.boundaryDensity)

    def computePressureAcceleration(self, simulationState, simulation):
        st = simulationState
        self.fluidVolume = self._wall_volume()
        if self.simulationScheme == 'deltaPlus':     # computePressureAccelDeltaPlus (solidBoundary.py:876-884)
            n = st['fluidPosition'].shape[0]
            out = torch.empty((n, 2), dtype=torch.float32, device=st['fluidPosition'].device)
            surface_term("wall_pressure_accel", self.P, n, self.numPtcls, out=out, walls=self._bf,
                         pressure=simulation.pressureModule.pressure, wall_pressure=self.pressure,
                         mask=st['fluidSurfaceMask'], rho=st['fluidDensity'], wall_volume=self.fluidVolume)
            return out
        return self._sum("pressure_accel", st, rho=st['fluidDensity'], pressure=st['fluidPressure'],
                         wall_pressure=self.pressure, wall_volume=self.fluidVolume)

    # ------------------------------------------------------------------ DFSPH wall parts (PBSPH)
    def dfsphPrepareSolver(self, simulationState, simulation, density=True):
        if not density or self.boundaryToFluidNeighbors is None:
            return
        self.boundaryPressure = torch.zeros_like(self.boundaryVolume)
        self.boundaryPressure2 = torch.zeros_like(self.boundaryVolume)
        self.boundaryActualArea = self._wall_volume()
        self.boundaryPredictedVelocity = torch.zeros_like(self.boundaryPositions)   # static walls

    def dfsphBoundaryAccelTerm(self, simulationState, simulation, density):
        st = simulationState
        if not density or self.boundaryToFluidNeighbors is None:
            return torch.zeros_like(st['fluidPosition'])
        return self._sum("dfsph_accel", st, rho=st['fluidDensity'], pressure=st['fluidPressure2'],
                         wall_area=self.boundaryVolume, wall_rho=self.boundaryDensity,
                         wall_pressure=self.boundaryPressure)

    def dfsphBoundaryPressureSum(self, simulationState, simulation, density):
        st = simulationState
        if not density or self.boundaryToFluidNeighbors is None:
            return torch.zeros_like(st['fluidDensity'])
        ksum = self._sum("b_dfsph_pressure_sum", st, actual_area=st['fluidActualArea'], pred_accel=st['fluidPredAccel'])
        self.boundaryResidual = ksum - self.boundarySource
        p = self.boundaryPressure - self.relaxedJacobiOmega * self.boundaryResidual / self.boundaryAlpha
        p = torch.clamp(p, min=0.)
        if self.backgroundPressure:
            p = torch.clamp(p, min=(5 ** 2) * self.restDensity)
        self.boundaryPressure = p
        return self._sum("dfsph_pressure_sum", st, pred_accel=st['fluidPredAccel'],
                         wall_actual_area=self.boundaryActualArea)

    def dfsphBoundaryAlphaTerm(self, simulationState, simulation, density):
        st = simulationState
        n = st['fluidPosition'].shape[0]
        if not density or self.boundaryToFluidNeighbors is None:
            return (torch.zeros((n, 2), dtype=torch.float32, device=st['fluidPosition'].device),
                    torch.zeros(n, dtype=torch.float32, device=st['fluidPosition'].device))
        k = self._sum("dfsph_alpha", st, wall_actual_area=self.boundaryActualArea, wall_area=self.boundaryVolume)
        self.boundaryAlpha = self._sum("b_dfsph_alpha", st, actual_area=st['fluidActualArea'], area=st['fluidArea'],
                                       wall_actual_area=self.boundaryActualArea)
        return k[:, 0:2], k[:, 2]

    def dfsphBoundarySourceTerm(self, simulationState, simulation, density):
        st = simulationState
        if not density or self.boundaryToFluidNeighbors is None:
            return torch.zeros_like(st['fluidDensity'])
        self.boundarySource = self._sum("b_dfsph_source", st, actual_area=st['fluidActualArea'],
                                        pred_vel=st['fluidPredictedVelocity'], wall_rho=self.boundaryDensity)
        return self._sum("dfsph_source", st, pred_vel=st['fluidPredictedVelocity'],
                         wall_actual_area=self.boundaryActualArea)


# ----------------------------------------------------------------------------- DFSPH
class dfsphModule(Module):
    """src/modules/dfsph.py:102-320: the divergence-free and constant-density solves of DFSPH,
    each relaxed-Jacobi sweep one kernel per fluid term plus the boundary module's hooks, with
    the reference's loop, error and iteration-count rules (the fused cooperative solver of
    `pytorchsph_gb300.sim.Simulation` is the fast path)."""

    def getParameters(self):
        return [
            Parameter('dfsph', 'minDensitySolverIterations', 'int', 2, required=False, export=True, hint=''),
            Parameter('dfsph', 'minDivergenceSolverIterations', 'int', 2, required=False, export=True, hint=''),
            Parameter('dfsph', 'maxDensitySolverIterations', 'int', 256, required=False, export=True, hint=''),
            Parameter('dfsph', 'maxDivergenceSolverIterations', 'int', 8, required=False, export=True, hint=''),
            Parameter('dfsph', 'densityThreshold', 'float', 1e-3, required=False, export=True, hint=''),
            Parameter('dfsph', 'divergenceThreshold', 'float', 1e-2, required=False, export=True, hint=''),
            Parameter('dfsph', 'divergenceSolver', 'bool', True, required=False, export=True, hint=''),
            Parameter('dfsph', 'relaxedJacobiOmega', 'float', 0.5, required=False, export=True, hint=''),
        ]

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')

    def initialize(self, simulationConfig, simulationState):
        cfg = simulationConfig
        self.support = cfg['particle']['support']
        d = cfg['dfsph']
        self.minDensitySolverIterations = d['minDensitySolverIterations']
        self.minDivergenceSolverIterations = d['minDivergenceSolverIterations']
        self.maxDensitySolverIterations = d['maxDensitySolverIterations']
        self.maxDivergenceSolverIterations = d['maxDivergenceSolverIterations']
        self.densityThreshold = d['densityThreshold']
        self.divergenceThreshold = d['divergenceThreshold']
        self.relaxedJacobiOmega = d['relaxedJacobiOmega'] if 'dfsph' in cfg else 0.5
        self.backgroundPressure = cfg['fluid']['backgroundPressure']
        self.pressureScheme = cfg['pressure']['boundaryPressureTerm']
        self.P = _params(self.support, cfg['fluid']['restDensity'])

    def _dt(self, st):
        return float(st['dt'])

    def computeAlpha(self, simulationState, simulation, density=True):
        st = simulationState
        k = pair_term("dfsph_alpha", st, self.P, actual_area=st['fluidActualArea'])
        bk1, bk2 = simulation.boundaryModule.dfsphBoundaryAlphaTerm(st, simulation, density)
        kSum1 = k[:, 0:2] + bk1
        kSum2 = k[:, 2] + bk2
        dt = self._dt(st)
        fac = -dt ** 2 * st['fluidActualArea']
        mass = st['fluidArea'] * st['fluidRestDensity']
        alpha = fac / mass * torch.einsum('nd, nd -> n', kSum1, kSum1) + fac * kSum2
        return torch.clamp(alpha, -1, -1e-7)

    def computeSourceTerm(self, simulationState, simulation, density=True):
        st = simulationState
        source = pair_term("dfsph_source", st, self.P, actual_area=st['fluidActualArea'],
                           pred_vel=st['fluidPredictedVelocity'], dt=self._dt(st))
        source = source + simulation.boundaryModule.dfsphBoundarySourceTerm(st, simulation, density)
        return 1. - st['fluidDensity'] + source if density else source

    def computeUpdatedPressure(self, simulationState, simulation, density=True):
        st = simulationState
        kernelSum = pair_term("dfsph_pressure_sum", st, self.P, actual_area=st['fluidActualArea'],
                              pred_accel=st['fluidPredAccel'], dt=self._dt(st))
        kernelSum += simulation.boundaryModule.dfsphBoundaryPressureSum(st, simulation, density)
        residual = kernelSum - st['fluidSourceTerm']
        pressure = st['fluidPressure'] - 0.3 * residual / st['fluidAlpha']
        pressure = torch.clamp(pressure, min=0.) if density else pressure
        if density and self.backgroundPressure:
            pressure = torch.clamp(pressure, min=(5 ** 2) * st['fluidRestDensity'])
        if not bool(torch.isfinite(pressure).all()):
            raise Exception('Pressure solver became unstable!')
        return pressure, residual

    def computeAcceleration(self, simulationState, simulation, density=True):
        st = simulationState
        a = pair_term("dfsph_accel", st, self.P, pressure=st['fluidPressure2'])
        return a + simulation.boundaryModule.dfsphBoundaryAccelTerm(st, simulation, density)

    def _solve(self, st, simulation, density):
        errors = []
        i = 0
        error = 0.
        if density:
            minIters, maxIters, thr = (self.minDensitySolverIterations, self.maxDensitySolverIterations,
                                       self.densityThreshold)
            if 'densityErrors' in st:
                minIters = max(minIters, len(st['densityErrors']) * 0.75)
        else:
            minIters, maxIters, thr = (self.minDivergenceSolverIterations, self.maxDivergenceSolverIterations,
                                       self.divergenceThreshold)
        while (i < minIters or error > thr) and i <= maxIters:
            st['fluidPredAccel'] = self.computeAcceleration(st, simulation, density)
            st['fluidPressure'][:] = st['fluidPressure2'][:]
            st['fluidPressure2'], st['residual'] = self.computeUpdatedPressure(st, simulation, density)
            if density and self.pressureScheme == 'PBSPH':
                bm = simulation.boundaryModule
                fluidError = torch.sum(torch.clamp(st['residual'], min=-thr))
                boundaryError = torch.sum(torch.clamp(bm.boundaryResidual, min=-thr)) \
                    if getattr(bm, 'boundaryResidual', None) is not None else 0.
                error = (fluidError + boundaryError) / (getattr(bm, 'numPtcls', 0) + st['residual'].shape[0])
            else:
                error = torch.mean(torch.clamp(st['residual'], min=-thr))
            errors.append(float(error))
            error = float(error)
            i += 1
        return errors

    def densitySolve(self, simulationState, simulation):
        errors = self._solve(simulationState, simulation, True)
        simulationState['densityErrors'] = errors
        simulationState['densitySolverPressure'] = simulationState['fluidPressure']
        return errors

    def divergenceSolve(self, simulationState, simulation):
        errors = self._solve(simulationState, simulation, False)
        simulationState['divergenceErrors'] = errors
        simulationState['divergenceSolverPressure'] = simulationState['fluidPressure']
        return errors

    def DFSPH(self, simulationState, simulation, density=True):
        st = simulationState
        x = st['fluidPosition']
        st['fluidPredAccel'] = torch.zeros_like(x)
        st['fluidPredictedVelocity'] = st['fluidVelocity'] + float(st['dt']) * st['fluidAcceleration']
        st['fluidActualArea'] = st['fluidArea'] / st['fluidDensity']
        simulation.boundaryModule.dfsphPrepareSolver(st, simulation, density)
        st['fluidAlpha'] = self.computeAlpha(st, simulation, density)
        st['fluidSourceTerm'] = self.computeSourceTerm(st, simulation, density)
        n = st['numParticles']
        st['fluidPressure2'] = torch.zeros(n, dtype=x.dtype, device=x.device)
        st['fluidPressure'] = torch.zeros(n, dtype=x.dtype, device=x.device)
        errors = self.densitySolve(st, simulation) if density else self.divergenceSolve(st, simulation)
        st['fluidPredAccel'] = self.computeAcceleration(st, simulation, density)
        st['fluidPressure'][:] = st['fluidPressure2'][:]
        st['fluidPredictedVelocity'] += float(st['dt']) * st['fluidPredAccel']
        return errors

    def incompressibleSolver(self, simulationState, simulation):
        return self.DFSPH(simulationState, simulation, True)

    def divergenceSolver(self, simulationState, simulation):
        return self.DFSPH(simulationState, simulation, False)


# ----------------------------------------------------------------------------- delta+ surface / shifting
class deltaPlusModule(Module):
    """src/modules/deltaPlus.py:36-251 on GPU kernels (sph_surface_term): surface detection
    (normalization matrix with its singular values, the lambda gradient and the fluid normal,
    the angle test and the surface classification) and the delta+ particle shift.

    What the reference does and this keeps: the wall part of the lambda gradient takes the wall
    particle's volume as fluidArea[b] / fluidDensity[b], indexing the fluid arrays with the
    wall index (deltaPlus.py:150), so a wall index at or above the fluid count raises
    IndexError as it does there; the shift evaluates W at the packing ratio for its k0
    (deltaPlus.py:90), which the reference can only evaluate once the ratio is a tensor."""

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')

    def exportState(self, simulationState, simulation, grp, mask):
        if simulation.config['shifting']['enabled']:
            grp.create_dataset('fluidShifting', data=simulationState['fluidUpdate'].detach().cpu().numpy())

    def initialize(self, simulationConfig, simulationState):
        cfg = simulationConfig
        self.support = cfg['particle']['support']
        self.packing = cfg['particle']['packing']
        self.restDensity = cfg['fluid']['restDensity']
        self.scheme = cfg['diffusion']['densityScheme']
        self.alpha = cfg['diffusion']['alpha']
        self.delta = cfg['diffusion']['delta']
        self.c0 = _c0(cfg)
        self.eps = self.support ** 2 * 0.1
        self.dtype = cfg['compute']['precision']
        self.device = cfg['compute']['device']
        self.P = _params(self.support, self.restDensity, self.c0, alpha=self.alpha, delta=self.delta)

    @staticmethod
    def _walls(simulation, n):
        bm = getattr(simulation, 'boundaryModule', None)
        if bm is None or not getattr(bm, 'active', False) or getattr(bm, '_bf', None) is None:
            return None, None, 0
        return bm, bm._bf, bm.numPtcls

    def computeShiftAmount(self, simulationState, simulation):
        st = simulationState
        n = st['fluidPosition'].shape[0]
        cfg = getattr(simulation, 'config', None)
        c0 = cfg['fluid']['c0'] if cfg else self.c0
        packing = cfg['particle']['packing'] if cfg else self.packing
        bm, walls, nb = self._walls(simulation, n)
        P = _params(self.support, self.restDensity, c0)
        out = torch.empty((n, 2), dtype=torch.float32, device=st['fluidPosition'].device)
        scratch = torch.empty((N.load().sph_surface_scratch_bytes() + 3) // 4, dtype=torch.float32, device=out.device)
        surface_term("shift", P, n, nb, out=out, out2=scratch, fluid=st, walls=walls, packing=packing, cfl=1.5,
                     vel=st['fluidVelocity'], area=st['fluidArea'], rho=st['fluidDensity'],
                     wall_area=bm.boundaryVolume if bm else None, wall_rho=bm.boundaryDensity if bm else None)
        st['shiftAmount'] = out

    def computeNormalizationmatrix(self, simulationState, simulation):
        st = simulationState
        if 'fluidL' in st:
            self.normalizationMatrix = st['normalizationMatrix']
            self.fluidL = st['fluidL']
            self.eigVals = st['eigVals']
        else:
            M = pair_term("normalization", st, self.P)
            bm = getattr(simulation, 'boundaryModule', None)
            if bm is not None and getattr(bm, 'active', False):
                M += bm.computeNormalizationMatrices(st, simulation)
            st['normalizationMatrix'] = M
            st['fluidL'], st['eigVals'] = pinv2x2(M, self.P)
        st['fluidLambda'] = st['eigVals'][:, 1]

    def computeFluidNormal(self, simulationState, simulation):
        st = simulationState
        n = st['fluidPosition'].shape[0]
        bm, walls, nb = self._walls(simulation, n)
        if walls is not None and walls.rows.numel() > 0 and int(walls.rows.max()) >= n:
            # fluidArea[bb] of deltaPlus.py:150 with a wall index past the fluid arrays
            raise IndexError(f"index {int(walls.rows.max())} is out of bounds for dimension 0 with size {n}")
        dev = st['fluidPosition'].device
        grad = torch.empty((n, 2), dtype=torch.float32, device=dev)
        normal = torch.empty((n, 2), dtype=torch.float32, device=dev)
        surface_term("normal", self.P, n, nb, out=grad, out2=normal, fluid=st, walls=walls, area=st['fluidArea'],
                     rho=st['fluidDensity'], L=st['fluidL'].contiguous(), lambda_=st['fluidLambda'].contiguous(),
                     wall_lambda=bm.eigVals[:, 1].contiguous() if bm is not None else None)
        st['lambdaGrad'] = grad
        st['fluidNormal'] = normal

    def detectFluidSurface(self, simulationState, simulation):
        st = simulationState
        n = st['fluidPosition'].shape[0]
        bm, walls, nb = self._walls(simulation, n)
        dev = st['fluidPosition'].device
        lam = st['fluidLambda'].contiguous()
        mask = torch.empty(n, dtype=torch.float32, device=dev)
        angles = torch.empty((n, 2), dtype=torch.float32, device=dev)
        surface_term("angle_mask", self.P, n, nb, out=mask, out2=angles, fluid=st, walls=walls,
                     normal=st['fluidNormal'], lambda_=lam)
        st['angleMin'] = angles[:, 0]
        st['angleMax'] = angles[:, 1]
        surf = torch.empty(n, dtype=torch.float32, device=dev)
        surface_term("classify", self.P, n, nb, out=surf, fluid=st, mask=mask, lambda_=lam)
        st['fluidSurfaceMask'] = surf

    def adjustShiftingAmount(self, simulationState, simulation):
        st = simulationState
        n = st['fluidPosition'].shape[0]
        dev = st['fluidPosition'].device
        update = torch.empty((n, 2), dtype=torch.float32, device=dev)
        mask = torch.empty(n, dtype=torch.float32, device=dev)
        surface_term("shift_adjust", self.P, n, out=update, out2=mask, shift=st['shiftAmount'],
                     mask=st['fluidSurfaceMask'], normal=st['fluidNormal'])
        st['shiftAmount'] = update       # the reference adjusts shiftAmount in place
        st['fluidUpdate'] = update
        st['fluidSurfaceMask'] = mask

    def detectSurface(self, simulationState, simulation):
        self.computeNormalizationmatrix(simulationState, simulation)
        self.computeFluidNormal(simulationState, simulation)
        self.detectFluidSurface(simulationState, simulation)

    def shift(self, simulationState, simulation):
        if 'fluidSurfaceMask' not in simulationState:
            self.detectSurface(simulationState, simulation)
        self.computeShiftAmount(simulationState, simulation)
        self.adjustShiftingAmount(simulationState, simulation)
