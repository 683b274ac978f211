"""Golden time steps from the reference's own deltaSPH and DFSPH solvers.

Runs the reference's `integrate()` (src/simulationBase.py:632-782) on small dam-break
scenes through oracle/ref_step.py and stores, per case, the scene, the parameters and the
state after each step (positions, velocities, densities, dpdt, accelerations, pressures,
wall density, DFSPH iteration counts).  Needs the reference checkout; writes
tests/golden/step_golden.npz.
Usage:  python tests/golden/make_step_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import ref_step  # noqa: E402
from pytorchsph_gb300 import workloads  # noqa: E402

DFSPH = dict(minDensitySolverIterations=2, minDivergenceSolverIterations=2, maxDensitySolverIterations=100,
             maxDivergenceSolverIterations=100, densityThreshold=1e-4, divergenceThreshold=1e-3,
             divergenceSolver=True, relaxedJacobiOmega=0.5)


def perturbed_scene(seed, nx=16, ny=32, dx=0.01, tank=(0.5, 0.5)):
    """A dam-break block with small seeded position jitter, velocities and density noise so
    that every term of the step is non-zero from the first evaluation."""
    s = workloads.dam_break(nx, ny, dx, tank)
    rng = np.random.default_rng(seed)
    s["pos"] = (s["pos"] + rng.uniform(-0.05 * dx, 0.05 * dx, s["pos"].shape)).astype(np.float32)
    s["vel"] = rng.normal(0, 0.05, s["vel"].shape).astype(np.float32)
    s["rho"] = (1.0 + rng.uniform(-2e-3, 2e-3, s["rho"].shape)).astype(np.float32)
    return s


CASES = {
    "dsph_mog_sie": dict(seed=0, steps=3, kw=dict(scheme="deltaSPH", diffusion="MOG",
                                                  integration="semiImplicitEuler")),
    "dsph_delta_sie": dict(seed=1, steps=3, kw=dict(scheme="deltaSPH", diffusion="deltaSPH",
                                                    integration="semiImplicitEuler")),
    "dsph_mog_rk4": dict(seed=2, steps=2, kw=dict(scheme="deltaSPH", diffusion="MOG", integration="RK4")),
    # point-source body force (gravity.pointSource with potentialField, src/modules/gravity.py:46-57),
    # the force of the oscillating drops, centred off the origin
    "dsph_point_sie": dict(seed=4, steps=3, kw=dict(scheme="deltaSPH", diffusion="deltaSPH",
                                                    integration="semiImplicitEuler", point_source=True,
                                                    point_center=(0.08, 0.16))),
    # MLS wall pressures (solidBoundary.py:772-808, src/util.py:283-384); the harness patches
    # of oracle/ref_step.py make them run
    "dsph_ghostmls_sie": dict(seed=6, steps=2, kw=dict(scheme="deltaSPH", diffusion="deltaSPH",
                                                       integration="semiImplicitEuler", boundary_pressure="ghostMLS")),
    "dsph_deltamls_sie": dict(seed=7, steps=2, kw=dict(scheme="deltaSPH", diffusion="deltaSPH",
                                                       integration="semiImplicitEuler", boundary_pressure="deltaMLS")),
    "dsph_mlspressure_sie": dict(seed=8, steps=2, kw=dict(scheme="deltaSPH", diffusion="deltaSPH",
                                                          integration="semiImplicitEuler",
                                                          boundary_pressure="MLSPressure")),
    "dfsph_sie": dict(seed=3, steps=3, kw=dict(scheme="dfsph", integration="semiImplicitEuler", dt=0.0005,
                                               kinematic=0.01, dfsph=DFSPH, cfl_fixed=False)),
}


def main():
    torch.set_num_threads(4)
    out = {}
    meta = {}
    for name, c in CASES.items():
      for prec in ("single", "double"):
        scene = perturbed_scene(c["seed"])
        sim = ref_step.make_simulation(scene, precision=prec, **c["kw"])
        cfg = sim.config
        for k in ("pos", "vel", "rho", "area", "wall_pos", "ghost_pos", "wall_area", "vmin", "vmax"):
            out[f"{name}/scene_{k}"] = scene[k]
        meta[name] = {"h": float(scene["h"]), "dx": scene["dx"], "tank": scene["tank"],
                      "rho0": float(cfg["fluid"]["restDensity"]), "c0": float(cfg["fluid"]["c0"]),
                      "alpha": float(cfg["diffusion"]["alpha"]), "delta": float(cfg["diffusion"]["delta"]),
                      "kinematic": float(cfg["diffusion"]["kinematic"]), "dt": float(cfg["integration"]["dt"]),
                      "diffusion": cfg["diffusion"]["densityScheme"], "integration": cfg["integration"]["scheme"],
                      "scheme": cfg["simulation"]["scheme"], "steps": c["steps"],
                      "dt_min": float(cfg["timestep"]["min"]), "dt_max": float(cfg["timestep"]["max"]),
                      "fixed_dt": bool(cfg["timestep"]["fixed"]),
                      "point_source": bool(cfg["gravity"]["pointSource"]),
                      "gravity_magnitude": float(cfg["gravity"]["magnitude"]),
                      "point_center": [float(v) for v in cfg["gravity"]["center"]],
                      "boundary_pressure": cfg["pressure"]["boundaryPressureTerm"]}
        if "dfsph" in cfg:
            meta[name]["dfsph"] = {k: (float(v) if not isinstance(v, bool) else v) for k, v in cfg["dfsph"].items()}
        tag = "" if prec == "single" else "f64_"
        for k in range(c["steps"]):
            sim.integrate()
            snap = ref_step.snapshot(sim)
            for key, v in snap.items():
                out[f"{name}/{tag}step{k}_{key}"] = np.asarray(v)
        print(name, prec, "ok", flush=True)
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, "step_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()
