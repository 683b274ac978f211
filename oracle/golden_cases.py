"""Test infrastructure only (oracle): load the golden step cases (tests/golden/step_golden.npz)
into the restated solver's inputs (sph_torch.Params / Walls / state dicts)."""
from __future__ import annotations

import json
import os

import numpy as np
import torch

import sph_torch as S

GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden",
                      "step_golden.npz")


def load():
    g = np.load(GOLDEN)
    return g, json.loads(str(g["meta"]))


def case(g, meta, name):
    m = meta[name]
    sc = lambda k: g[f"{name}/scene_{k}"]
    df = m.get("dfsph", {})
    p = S.Params(h=m["h"], rho0=m["rho0"], c0=m["c0"], alpha=m["alpha"], delta=m["delta"], kinematic=m["kinematic"],
                 diffusion=m["diffusion"], vmin=sc("vmin"), vmax=sc("vmax"),
                 min_density_iters=int(df.get("minDensitySolverIterations", 2)),
                 max_density_iters=int(df.get("maxDensitySolverIterations", 100)),
                 density_threshold=float(df.get("densityThreshold", 1e-4)),
                 divergence_solver=bool(df.get("divergenceSolver", True)),
                 min_divergence_iters=int(df.get("minDivergenceSolverIterations", 2)),
                 max_divergence_iters=int(df.get("maxDivergenceSolverIterations", 100)),
                 divergence_threshold=float(df.get("divergenceThreshold", 1e-3)),
                 omega_boundary=float(df.get("relaxedJacobiOmega", 0.5)),
                 point_source=bool(m.get("point_source", False)),
                 point_magnitude=float(m.get("gravity_magnitude", 9.81)),
                 point_center=tuple(m.get("point_center", (0.0, 0.0))),
                 boundary_pressure=m.get("boundary_pressure", "PBSPH"))
    walls = S.Walls(torch.from_numpy(sc("wall_pos")), torch.from_numpy(sc("ghost_pos")), torch.from_numpy(sc("wall_area")))
    state = {"x": torch.from_numpy(sc("pos")), "v": torch.from_numpy(sc("vel")), "rho": torch.from_numpy(sc("rho")),
             "area": torch.from_numpy(sc("area"))}
    return m, p, walls, state


def run(g, meta, name, dtype, steps=None):
    """Step the restated solver through the case; yields (k, new_state, extras, dt_used)."""
    m, p, walls, st = case(g, meta, name)
    solver = "dfsph" if m["scheme"] == "dfsph" else "deltaSPH"
    if solver == "dfsph":
        walls.density_term = S.wall_density_term(walls, m["h"], dtype)
    dt = m["dt"]
    for k in range(m["steps"] if steps is None else steps):
        new, ex = S.step(st, walls, p, dt, m["integration"], solver, dtype)
        yield k, new, ex, dt
        st = {"x": new["x"].float() if dtype == torch.float32 else new["x"], "v": new["v"], "rho": new["rho"],
              "area": st["area"]}
        if solver == "dfsph" and not m["fixed_dt"]:
            dt = S.update_dt(new, p, dt, m["dt_min"], m["dt_max"])
