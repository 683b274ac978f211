"""GB300 simulation engine for the deltaSPH and DFSPH steps of pytorchSPH.

The whole per-step hot path runs in libsph_gb300.so: re-sort of the particle state by cell
key, CSR neighbor search, mDBC wall density, the summations and the integrator.  The
particle state lives on the device in cell-sorted order between steps (every array is
permuted together with the sort), `uid` carries each particle's original index, and
`Simulation.state()` returns fields in the original order.

Mirrors `deltaSPHSimulation` / `dfsphSimulation` (src/deltaSPH.py:74-200,
src/dfsph.py:70-202) with `SPHSimulation.integrate` (src/simulationBase.py:632-782) for the
semiImplicitEuler and RK4 schemes, solid ghost-particle walls (`solidBoundaryModule`) and
the adaptive time step (src/modules/adaptiveDT.py:59-95).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as N
from .search import MAX_CELLS, Workspace, grid_from_bytes, _f2


# ----------------------------------------------------------------------------- C structs
class SphParamsC(ctypes.Structure):
    _fields_ = [("support", ctypes.c_float), ("rest_density", ctypes.c_float), ("c0", ctypes.c_float),
                ("gamma", ctypes.c_float), ("alpha", ctypes.c_float), ("delta", ctypes.c_float),
                ("kinematic", ctypes.c_float), ("gravity", ctypes.c_float * 2), ("point_source", ctypes.c_int32),
                ("point_magnitude", ctypes.c_float), ("point_center", ctypes.c_float * 2),
                ("density_diffusion", ctypes.c_int32), ("boundary_diffusion", ctypes.c_int32),
                ("search_radius", ctypes.c_int32), ("cell_capacity", ctypes.c_int32),
                ("min_density_iters", ctypes.c_int32), ("max_density_iters", ctypes.c_int32),
                ("min_divergence_iters", ctypes.c_int32), ("max_divergence_iters", ctypes.c_int32),
                ("density_threshold", ctypes.c_float), ("divergence_threshold", ctypes.c_float),
                ("omega_boundary", ctypes.c_float), ("omega_fluid", ctypes.c_float)]


class FluidViewC(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("v", ctypes.c_void_p), ("rho", ctypes.c_void_p), ("area", ctypes.c_void_p),
                ("keys", ctypes.c_void_p), ("offsets", ctypes.c_void_p), ("cols", ctypes.c_void_p),
                ("cell_start", ctypes.c_void_p), ("n", ctypes.c_int64), ("pair_capacity", ctypes.c_int64)]


class WallViewC(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("ghost", ctypes.c_void_p), ("area", ctypes.c_void_p),
                ("cell_start", ctypes.c_void_p), ("n", ctypes.c_int64), ("rho", ctypes.c_void_p),
                ("volume", ctypes.c_void_p), ("pressure", ctypes.c_void_p)]


class DfsphBuffersC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in (
        "rho", "volume", "actual_area", "vstar", "alpha", "source", "pressure", "pred_accel", "residual", "wall_rho",
        "wall_actual_area", "wall_alpha", "wall_source", "wall_pressure", "wall_residual", "wall_density_term",
        "partials", "errors", "iters", "records")]




def _ref(s):
    return ctypes.byref(s)


# ----------------------------------------------------------------------------- configuration
@dataclass
class SimConfig:
    """Scene parameters (names follow the reference's TOML keys)."""
    solver: str = "deltaSPH"                 # simulation.scheme: "deltaSPH" | "dfsph"
    integration: str = "semiImplicitEuler"    # integration.scheme: "semiImplicitEuler" | "RK4"
    dt: float = 1e-4                          # integration.dt (initial)
    rest_density: float = 1000.0              # fluid.restDensity
    c0: float = 10.0                          # fluid.c0
    gamma: float = 7.0                        # pressure.gamma
    alpha: float = 0.01                       # diffusion.alpha
    delta: float = 0.1                        # diffusion.delta
    kinematic: float = 0.001                  # diffusion.kinematic
    density_diffusion: str = "MOG"            # diffusion.densityScheme: "MOG" | "deltaSPH" | "none"
    boundary_diffusion: bool = True           # diffusion.boundaryDiffusion
    gravity: tuple = (0.0, -9.81)             # gravity.magnitude * gravity.direction
    point_source: bool = False                # gravity.pointSource (potential field)
    point_magnitude: float = 1.0
    point_center: tuple = (0.0, 0.0)
    fixed_dt: bool = True                     # timestep.fixed
    dt_min: float = 1e-6                      # timestep.min
    dt_max: float = 1e-2                      # timestep.max
    cfl: float = 0.4                          # timestep.CFLNumber
    min_density_iters: int = 2                # dfsph.*
    max_density_iters: int = 100
    density_threshold: float = 1e-4
    divergence_solver: bool = True
    min_divergence_iters: int = 2
    max_divergence_iters: int = 100
    divergence_threshold: float = 1e-3
    omega_boundary: float = 0.5
    omega_fluid: float = 0.3
    search_radius: int = 1
    pair_headroom: float = 1.3


DIFFUSION = {"none": 0, "MOG": 1, "deltaSPH": 2}


class Simulation:
    """One scene on the GPU.  `scene` holds numpy arrays (pos, vel, rho, area, support,
    wall_pos, ghost_pos, wall_area, vmin, vmax), e.g. from pytorchsph_gb300.workloads."""

    def __init__(self, scene: dict, cfg: SimConfig, device=None):
        self.lib = N.load()
        self.cfg = cfg
        self.device = torch.device(device or torch.device("cuda", torch.cuda.current_device()))
        dev = self.device
        self.ws = Workspace(dev)
        f32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float32), device=dev)
        n = len(scene["pos"])
        self.n = n
        h = float(np.float32(scene["support"][0]))
        if not np.all(scene["support"] == np.float32(h)):
            raise N.SPHError("the GB300 engine needs a uniform support radius")
        self.h = h
        self.vmin = np.asarray(scene["vmin"], np.float32)
        self.vmax = np.asarray(scene["vmax"], np.float32)
        # particle state (original order at start; kept in cell-sorted order afterwards)
        self.arr = {
            "x": f32(scene["pos"]).reshape(n, 2), "v": f32(scene["vel"]).reshape(n, 2), "rho": f32(scene["rho"]),
            "area": f32(scene["area"]), "uid": torch.arange(n, dtype=torch.int32, device=dev),
        }
        self.support_arr = torch.full((n,), h, dtype=torch.float32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.dt = torch.tensor([cfg.dt], dtype=torch.float32, device=dev)
        self.time = torch.zeros(1, dtype=torch.float64, device=dev)   # simulated time, kept on the device
        self.steps = 0
        # grid (constant: given domain, uniform support)
        self.grid = torch.empty(8, dtype=torch.int32, device=dev)
        self.cap = self._grid_capacity()
        self._build_grid(self.cap)
        self.params = self._params()
        # walls, sorted once by their cell in the fluid grid
        self.nb = len(scene.get("wall_pos", ()))
        self._setup_walls(scene)
        self.pair_cap = 0
        self.cols = None
        self.extra = {}
        self.last = {}
        self.graph = None

    # ------------------------------------------------------------------ set-up
    def _grid_capacity(self):
        st = N.stream_ptr()
        scratch = self.ws.bytes("grid_scratch", self.lib.sph_grid_scratch_bytes(self.n))
        self.status.zero_()
        N.call("sph_grid_build", N.ptr(self.arr["x"]), N.ptr(self.support_arr), self.n, _f2(self.vmin),
               _f2(self.vmax), MAX_CELLS, N.ptr(self.grid), N.ptr(self.status), N.ptr(scratch), scratch.numel() * 8, st)
        flags = int(self.status.item())
        if flags:
            raise N.SPHError(f"search grid: {N.decode_flags(flags)}")
        return max(grid_from_bytes(self.grid)["num_cells"], 1)

    def _build_grid(self, cap):
        scratch = self.ws.bytes("grid_scratch", self.lib.sph_grid_scratch_bytes(self.n))
        N.call("sph_grid_build", N.ptr(self.arr["x"]), N.ptr(self.support_arr), self.n, _f2(self.vmin),
               _f2(self.vmax), int(cap), N.ptr(self.grid), N.ptr(self.status), N.ptr(scratch), scratch.numel() * 8,
               N.stream_ptr())

    def _params(self):
        c = self.cfg
        P = SphParamsC()
        P.support = self.h
        P.rest_density = c.rest_density
        P.c0 = c.c0
        P.gamma = c.gamma
        P.alpha = c.alpha
        P.delta = c.delta
        P.kinematic = c.kinematic
        P.gravity[0], P.gravity[1] = c.gravity
        P.point_source = int(c.point_source)
        P.point_magnitude = c.point_magnitude
        P.point_center[0], P.point_center[1] = c.point_center
        P.density_diffusion = DIFFUSION[c.density_diffusion]
        P.boundary_diffusion = int(bool(c.boundary_diffusion))
        P.search_radius = c.search_radius
        P.cell_capacity = self.cap
        P.min_density_iters = c.min_density_iters
        P.max_density_iters = c.max_density_iters
        P.min_divergence_iters = c.min_divergence_iters
        P.max_divergence_iters = c.max_divergence_iters
        P.density_threshold = c.density_threshold
        P.divergence_threshold = c.divergence_threshold
        P.omega_boundary = c.omega_boundary
        P.omega_fluid = c.omega_fluid
        return P

    def _sort_keys(self, x, n, prefix, tie=None):
        """Counting sort of `n` positions by cell key (inside a cell by `tie`, e.g. the
        particle id, then index); returns (order, sorted_keys, cell_start)."""
        st = N.stream_ptr()
        ws = self.ws
        keys = ws.get(prefix + "keys", n)
        order = ws.get(prefix + "order", n)
        skeys = ws.get(prefix + "skeys", n)
        cs = ws.get(prefix + "cell_start", self.cap + 2)
        hist = ws.zeros(prefix + "hist", self.cap + 1)
        N.call("sph_cell_keys", N.ptr(x), n, N.ptr(self.grid), self.cap, N.ptr(keys), None, N.ptr(hist),
               N.ptr(self.status), st)
        scratch = ws.bytes(prefix + "cs_scratch", self.lib.sph_counting_sort_scratch_bytes(n, self.cap))
        N.call("sph_counting_sort_tie", N.ptr(keys), n, self.cap, N.ptr(hist), N.ptr(cs), N.ptr(tie), N.ptr(order),
               N.ptr(skeys), N.ptr(self.status), N.ptr(scratch), scratch.numel() * 8, st)
        return order, skeys, cs

    def _permute(self, order, t):
        out = torch.empty_like(t)
        eb = t.element_size() * (t.shape[1] if t.dim() == 2 else 1)
        N.call("sph_permute", N.ptr(order), t.shape[0], eb, N.ptr(t), N.ptr(out), N.stream_ptr())
        return out

    def _setup_walls(self, scene):
        dev = self.device
        nb = self.nb
        z = lambda k: torch.zeros(max(nb, 1), dtype=torch.float32, device=dev)
        if nb == 0:
            self.walls = {"x": torch.zeros((1, 2), device=dev), "ghost": torch.zeros((1, 2), device=dev),
                          "area": z(0), "cell_start": torch.zeros(self.cap + 2, dtype=torch.int32, device=dev),
                          "rho": z(0), "volume": z(0), "pressure": z(0), "order": None}
        else:
            self.scene_walls = {"pos": np.ascontiguousarray(scene["wall_pos"], np.float32),
                                "ghost": np.ascontiguousarray(scene["ghost_pos"], np.float32),
                                "area": np.ascontiguousarray(scene["wall_area"], np.float32)}
            wx = torch.as_tensor(np.ascontiguousarray(scene["wall_pos"], np.float32), device=dev)
            order, _, cs = self._sort_keys(wx, nb, "w_")
            self.walls = {"x": self._permute(order, wx),
                          "ghost": self._permute(order, torch.as_tensor(np.ascontiguousarray(scene["ghost_pos"], np.float32), device=dev)),
                          "area": self._permute(order, torch.as_tensor(np.ascontiguousarray(scene["wall_area"], np.float32), device=dev)),
                          "cell_start": cs.clone(), "rho": torch.ones(nb, device=dev), "volume": z(0),
                          "pressure": z(0), "order": order.clone()}
        self.wall_view = WallViewC(N.ptr(self.walls["x"]), N.ptr(self.walls["ghost"]), N.ptr(self.walls["area"]),
                                   N.ptr(self.walls["cell_start"]), nb, N.ptr(self.walls["rho"]),
                                   N.ptr(self.walls["volume"]), N.ptr(self.walls["pressure"]))
        if self.cfg.solver == "dfsph":
            self.wall_term = torch.zeros(max(nb, 1), dtype=torch.float32, device=dev)
            if nb:
                N.call("sph_dfsph_wall_wall_term", _ref(self.wall_view), N.ptr(self.grid), _ref(self.params),
                       N.ptr(self.wall_term), N.stream_ptr())

    # ------------------------------------------------------------------ one right-hand side
    def _search(self, sync):
        """Re-sort every particle array by cell key and build the CSR neighbor list."""
        st = N.stream_ptr()
        n = self.n
        order, skeys, cs = self._sort_keys(self.arr["x"], n, "f_", tie=self.arr["uid"])
        for k in list(self.arr):
            self.arr[k] = self._permute(order, self.arr[k])
        for k in list(self.extra):
            self.extra[k] = self._permute(order, self.extra[k])
        self.skeys, self.cell_start = skeys, cs
        counts = self.ws.get("counts", n)
        rho_fluid = self.ws.get("rho_fluid", n, torch.float32)
        dens = self.cfg.solver == "dfsph"
        N.call("sph_nl_count", N.ptr(self.arr["x"]), N.ptr(self.support_arr), N.ptr(self.arr["area"]), n, N.ptr(skeys),
               N.ptr(cs), N.ptr(self.grid), self.cap, self.cfg.search_radius, self.h if dens else 0.0, N.ptr(counts),
               N.ptr(rho_fluid) if dens else None, st)
        offsets = self.ws.get("offsets", n + 1)
        sc = self.ws.bytes("scan_scratch", self.lib.sph_scan_scratch_bytes(n))
        N.call("sph_exclusive_scan_i32", N.ptr(counts), N.ptr(offsets), n, N.ptr(sc), sc.numel() * 8, st)
        if sync or self.cols is None:
            P = int(offsets[n].item())
            if P > self.pair_cap:
                self.pair_cap = int(P * self.cfg.pair_headroom) + 1024
                self.cols = torch.empty(self.pair_cap, dtype=torch.int32, device=self.device)
        N.call("sph_nl_fill", N.ptr(self.arr["x"]), N.ptr(self.support_arr), n, N.ptr(skeys), N.ptr(cs), N.ptr(self.grid),
               self.cap, self.cfg.search_radius, N.ptr(offsets), self.pair_cap, N.ptr(self.cols), N.ptr(self.status), st)
        self.offsets = offsets
        self.rho_fluid = rho_fluid
        self.fluid_view = FluidViewC(N.ptr(self.arr["x"]), N.ptr(self.arr["v"]), N.ptr(self.arr["rho"]),
                                     N.ptr(self.arr["area"]), N.ptr(skeys), N.ptr(offsets), N.ptr(self.cols), N.ptr(cs), n,
                                     self.pair_cap)

    def rhs(self, sync=True):
        """Evaluate one timestep() at the current state; returns (acc, vel, dpdt or None)."""
        self._search(sync)
        st = N.stream_ptr()
        n = self.n
        acc = torch.empty((n, 2), dtype=torch.float32, device=self.device)
        if self.cfg.solver == "dfsph":
            return self._dfsph_rhs(acc, st)
        dpdt = torch.empty(n, dtype=torch.float32, device=self.device)
        if self.nb:
            N.call("sph_mdbc_wall_density", _ref(self.fluid_view), _ref(self.wall_view), N.ptr(self.grid),
                   _ref(self.params), st)
        gr = self.ws.get("grad_rho", 2 * n, torch.float32) if self.cfg.density_diffusion == "deltaSPH" else None
        scr = self.ws.bytes("forces_scratch", self.lib.sph_deltasph_scratch_bytes(n))
        N.call("sph_deltasph_forces", _ref(self.fluid_view), _ref(self.wall_view), N.ptr(self.grid), _ref(self.params),
               N.ptr(dpdt), N.ptr(acc), None, N.ptr(gr), N.ptr(scr), scr.numel() * 8, st)
        self.last = {"acc": acc, "dpdt": dpdt}
        return acc, self.arr["v"], dpdt

    def _dfsph_bufs(self):
        n, nb = self.n, max(self.nb, 1)
        g = lambda k, m, dt=torch.float32: self.ws.get("dfsph_" + k, m, dt)
        maxit = max(self.cfg.max_density_iters, self.cfg.max_divergence_iters) + 2
        b = {"rho": g("rho", n), "volume": g("volume", n), "actual_area": g("aact", n), "vstar": g("vstar", 2 * n),
             "alpha": g("alpha", n), "source": g("source", n), "pressure": g("p", n), "pred_accel": g("pa", 2 * n),
             "residual": g("res", n), "wall_rho": g("wrho", nb), "wall_actual_area": g("waact", nb),
             "wall_alpha": g("walpha", nb), "wall_source": g("wsrc", nb), "wall_pressure": g("wp", nb),
             "wall_residual": g("wres", nb), "wall_density_term": self.wall_term,
             "partials": g("partials", int(self.lib.sph_dfsph_partials_count()), torch.float64),
             "errors": g("errors", maxit), "iters": g("iters", 1, torch.int32), "records": g("records", 9 * n)}
        self.dfsph_arrays = b
        return DfsphBuffersC(*[N.ptr(b[k]) for k, _ in DfsphBuffersC._fields_])

    def _dfsph_rhs(self, acc, st):
        n = self.n
        B = self._dfsph_bufs()
        b = self.dfsph_arrays
        N.call("sph_dfsph_densities", _ref(self.fluid_view), _ref(self.wall_view), N.ptr(self.grid), _ref(self.params),
               N.ptr(self.rho_fluid), _ref(B), st)
        # the solver works with the summation density (incl. walls) as fluidDensity
        self.arr["rho"].copy_(b["rho"])
        c = self.cfg
        N.call("sph_fill_float2", n, c.gravity[0], c.gravity[1], N.ptr(acc), st)
        info = {}
        if c.divergence_solver:
            N.call("sph_dfsph_solve", _ref(self.fluid_view), _ref(self.wall_view), N.ptr(self.grid), _ref(self.params),
                   _ref(B), N.ptr(acc), N.ptr(self.dt), 0, N.ptr(self.status), st)
            N.call("sph_add_float2", n, N.ptr(b["pred_accel"]), N.ptr(acc), st)
            info["divergence_iters"] = b["iters"].clone()
            info["divergence_errors"] = b["errors"].clone()
        N.call("sph_dfsph_solve", _ref(self.fluid_view), _ref(self.wall_view), N.ptr(self.grid), _ref(self.params),
               _ref(B), N.ptr(acc), N.ptr(self.dt), 1, N.ptr(self.status), st)
        N.call("sph_add_float2", n, N.ptr(b["pred_accel"]), N.ptr(acc), st)
        info["density_iters"] = b["iters"].clone()
        info["density_errors"] = b["errors"].clone()
        N.call("sph_dfsph_viscosity", _ref(self.fluid_view), _ref(self.wall_view), N.ptr(self.grid), _ref(self.params),
               _ref(B), N.ptr(acc), st)
        self.last = {"acc": acc, "pressure": b["pressure"], "alpha": b["alpha"], "source": b["source"], **info}
        return acc, self.arr["v"], None

    # ------------------------------------------------------------------ integration
    def capture(self):
        """Record one step() in a CUDA graph; every later step() replays it (one launch of
        the whole step instead of ~20 host calls).  The state arrays become fixed device
        buffers: the recorded step ends by copying its new state into them.  Needs one eager
        step first (it sizes the neighbor buffer; a step that overflows it raises at check())."""
        if self.cols is None:
            raise N.SPHError("capture: run one step first")
        torch.cuda.synchronize(self.device)
        inputs = dict(self.arr)
        g = torch.cuda.CUDAGraph()
        steps, last = self.steps, self.last
        try:
            with torch.cuda.graph(g):
                self._step_kernels()
                for k, t in inputs.items():
                    t.copy_(self.arr[k])
        except Exception:
            self.arr, self.last = inputs, last
            raise
        self.arr = inputs
        self.steps = steps
        self.graph = g

    def step(self, sync=True):
        """One integrate() (src/simulationBase.py:632-782)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._step_kernels(sync)   # sync: the neighbor buffer grows to the step's pair count
        self.steps += 1
        if sync:
            self.check()

    def _step_kernels(self, sync=False):
        st = N.stream_ptr()
        n = self.n
        c = self.cfg
        cont = c.solver != "dfsph"
        if c.integration == "semiImplicitEuler":
            acc, vel, dpdt = self.rhs(sync)
            xo = torch.empty_like(self.arr["x"])
            vo = torch.empty_like(self.arr["v"])
            ro = torch.empty_like(self.arr["rho"])
            N.call("sph_integrate_semi_implicit_euler", n, N.ptr(self.arr["x"]), N.ptr(vel), N.ptr(self.arr["rho"]),
                   N.ptr(acc), N.ptr(dpdt), N.ptr(self.dt), c.rest_density, int(cont), N.ptr(xo), N.ptr(vo),
                   N.ptr(ro), N.ptr(self.status), st)
            self.last["eval"] = {"x": self.arr["x"], "v": self.arr["v"], "rho": self.arr["rho"]}
            self.arr["x"], self.arr["v"], self.arr["rho"] = xo, vo, ro
            self.last["acc_final"] = acc
        elif c.integration == "RK4":
            if not cont:
                raise N.SPHError("RK4 is implemented for the continuum-density deltaSPH solver")
            self.extra = {"x0": self.arr["x"].clone(), "v0": self.arr["v"].clone(), "r0": self.arr["rho"].clone()}
            self.extra["su"] = torch.empty_like(self.arr["x"])
            self.extra["sa"] = torch.empty_like(self.arr["x"])
            self.extra["sd"] = torch.empty_like(self.arr["rho"])
            for k, (cstage, w) in enumerate([(0.5, 1.0), (0.5, 2.0), (1.0, 2.0), (None, 1.0)]):
                acc, vel, dpdt = self.rhs(sync)
                e = self.extra
                N.call("sph_rk_accumulate", n, N.ptr(vel), N.ptr(acc), N.ptr(dpdt), w, int(k == 0), N.ptr(e["su"]),
                       N.ptr(e["sa"]), N.ptr(e["sd"]), st)
                if cstage is not None:
                    xo = torch.empty_like(self.arr["x"])
                    vo = torch.empty_like(self.arr["v"])
                    ro = torch.empty_like(self.arr["rho"])
                    N.call("sph_rk_axpy", n, N.ptr(e["x0"]), N.ptr(e["v0"]), N.ptr(e["r0"]), N.ptr(vel), N.ptr(acc),
                           N.ptr(dpdt), N.ptr(self.dt), cstage, c.rest_density, N.ptr(xo), N.ptr(vo), N.ptr(ro),
                           N.ptr(self.status), st)
                    self.arr["x"], self.arr["v"], self.arr["rho"] = xo, vo, ro
            e = self.extra
            xo = torch.empty_like(self.arr["x"])
            vo = torch.empty_like(self.arr["v"])
            ro = torch.empty_like(self.arr["rho"])
            N.call("sph_rk_axpy", n, N.ptr(e["x0"]), N.ptr(e["v0"]), N.ptr(e["r0"]), N.ptr(e["su"]), N.ptr(e["sa"]),
                   N.ptr(e["sd"]), N.ptr(self.dt), 1.0 / 6.0, c.rest_density, N.ptr(xo), N.ptr(vo), N.ptr(ro),
                   N.ptr(self.status), st)
            self.last["eval"] = {"x": self.arr["x"], "v": self.arr["v"], "rho": self.arr["rho"]}
            self.arr["x"], self.arr["v"], self.arr["rho"] = xo, vo, ro
            self.last["acc_final"] = e["sa"]
            self.extra = {}
        else:
            raise N.SPHError(f"integration scheme {c.integration!r} is not on the GB300 path")
        self.time += self.dt
        if not c.fixed_dt:
            self.last["dt_used"] = self.dt.clone()
            sc = self.ws.bytes("dt_scratch", self.lib.sph_dt_scratch_bytes())
            N.call("sph_update_dt", n, N.ptr(self.arr["v"]), N.ptr(self.last["acc_final"]), self.h, c.kinematic, c.cfl,
                   c.c0, int(c.solver in ("deltaSPH", "deltaPlus")), c.dt_min, c.dt_max, N.ptr(self.dt), N.ptr(sc),
                   sc.numel() * 8, st)

    def check(self):
        f = int(self.status.item())
        if f:
            raise N.SPHError(f"simulation step: {N.decode_flags(f)}")
        if self.cols is not None and int(self.offsets[self.n].item()) > self.pair_cap:
            raise N.SPHError("neighbor pair buffer too small")

    # ------------------------------------------------------------------ export
    def export_fields(self) -> dict:
        """The arrays of the reference's per-step export group (src/simulationBase.py:742-772,
        solidBoundary.py:263) after the last step, as device tensors in the engine's row order
        with the UID of each row (int32); issued on the current stream, no host wait.
        fluidPosition / fluidVelocity are the new state, finalPosition / finalVelocity /
        fluidDensity the state the last right-hand side was evaluated at, as the reference
        writes its perennial and simulation states."""
        if "eval" not in self.last:
            raise N.SPHError("export_fields: no step has run yet")
        st = N.stream_ptr()
        n = self.n
        c = self.cfg
        ev = self.last["eval"]
        f = {"UID": self.arr["uid"], "fluidPosition": self.arr["x"], "fluidVelocity": self.arr["v"],
             "finalPosition": ev["x"], "finalVelocity": ev["v"], "fluidArea": self.arr["area"],
             "fluidDensity": ev["rho"], "fluidSupport": self.support_arr, "fluidAcceleration": self.last["acc_final"]}
        if isinstance(self.last.get("pressure"), torch.Tensor):
            f["fluidPressure"] = self.last["pressure"]
        else:
            p = torch.empty(n, dtype=torch.float32, device=self.device)
            N.call("sph_particle_op", 0, n, N.ptr(ev["rho"]), None, _ref(self.params), N.ptr(p), 0, st)
            f["fluidPressure"] = p
        if c.point_source:
            g = torch.zeros((n, 2), dtype=torch.float32, device=self.device)
            N.call("sph_particle_op", 3, n, N.ptr(ev["x"]), None, _ref(self.params), N.ptr(g), 1, st)
            f["fluidGravity"] = g
        if c.solver != "dfsph" and isinstance(self.last.get("dpdt"), torch.Tensor):
            f["fluidDpdt"] = self.last["dpdt"]
        if self.nb:
            src = self.dfsph_arrays["wall_rho"] if c.solver == "dfsph" else self.walls["rho"]
            wr = torch.empty(self.nb, dtype=torch.float32, device=self.device)
            N.call("sph_scatter_f32", N.ptr(self.walls["order"]), N.ptr(src), self.nb, N.ptr(wr), st)
            f["boundaryDensity"] = wr
        return f

    def export_attributes(self) -> dict:
        """Root attributes of the reference's export file (src/simulationBase.py:452-481) that
        this engine's configuration determines."""
        c = self.cfg
        a = {"simulationScheme": c.solver, "boundaryScheme": "solid",
             "densityScheme": "summation" if c.solver == "dfsph" else "continuum", "EOSgamma": c.gamma,
             "fluidPressureTerm": "TaitEOS", "boundaryPressureTerm": "PBSPH", "shiftingScheme": "deltaPlus",
             "shiftingEnabled": False, "defaultKernel": "wendland2", "device": str(self.device),
             "floatprecision": "single", "restDensity": c.rest_density, "c0": c.c0, "support": self.h,
             "velocityDiffusionScheme": "deltaSPH", "densityDiffusionScheme": c.density_diffusion,
             "alphaDiffusion": c.alpha, "deltaDiffusion": c.delta, "kinematicDiffusion": c.kinematic,
             "staticBoundary": True, "initialDt": c.dt, "integrationScheme": c.integration, "fixedDt": c.fixed_dt}
        if not c.point_source:
            a["fluidGravity"] = list(c.gravity)
        return a

    def boundary_information(self) -> dict:
        """The static wall arrays of the reference's boundaryInformation group
        (src/simulationBase.py:483-491) in the scene's wall order; boundaryNormals point from
        each wall particle to its mirrored ghost, into the fluid."""
        if not self.nb:
            return {}
        w = self.scene_walls
        d = w["ghost"].astype(np.float64) - w["pos"].astype(np.float64)
        nrm = d / np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-30)
        return {"boundaryPosition": w["pos"], "boundaryVelocity": np.zeros_like(w["pos"]),
                "boundarySupport": np.full(self.nb, np.float32(self.h), np.float32),
                "boundaryRestDensity": np.full(self.nb, np.float32(self.cfg.rest_density), np.float32),
                "boundaryArea": w["area"], "boundaryNormals": nrm.astype(np.float32),
                "boundaryBodyAssociation": np.zeros(self.nb, np.int64)}

    def export(self, exporter) -> bool:
        """Queue this step's export group on a pytorchsph_gb300.export.SnapshotExporter: the
        arrays of export_fields() and the attributes time, timestep and dt (the dt the step
        used), all copied from the device without a host wait."""
        f = self.export_fields()
        f["@time"] = self.time.clone()
        f["@dt"] = self.last.get("dt_used", self.dt).clone()
        return exporter.submit(f, timestep=self.steps)

    # ------------------------------------------------------------------ output
    def _orig(self, t):
        uid = self.arr["uid"].long()
        out = torch.empty_like(t)
        out[uid] = t
        return out

    def state(self):
        """Current fields in the original particle order (numpy)."""
        out = {"x": self._orig(self.arr["x"]), "v": self._orig(self.arr["v"]), "rho": self._orig(self.arr["rho"])}
        # fields of the last right-hand side share the sorted order of the current state
        names = {"acc_final": "acc", "dpdt": "dpdt", "pressure": "pressure", "alpha": "alpha", "source": "source"}
        for k, name in names.items():
            t = self.last.get(k)
            if isinstance(t, torch.Tensor) and t.shape[0] == self.n:
                out[name] = self._orig(t)
        out = {k: v.detach().cpu().numpy() for k, v in out.items()}
        out["dt"] = float(self.dt.item())
        for k in ("density_iters", "divergence_iters"):
            if k in self.last:
                out[k] = int(self.last[k].item())
        return out

    def wall_state(self):
        """Wall density / pressure in the scene's original wall order (numpy)."""
        if not self.nb:
            return {}
        o = self.walls["order"].long()
        res = {}
        src = self.dfsph_arrays if self.cfg.solver == "dfsph" else None
        for k, t in (("rho", src["wall_rho"] if src else self.walls["rho"]), ("pressure", self.walls["pressure"])):
            out = torch.empty(self.nb, dtype=t.dtype, device=t.device)
            out[o] = t[:self.nb]
            res[k] = out.cpu().numpy()
        return res
