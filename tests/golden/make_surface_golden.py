"""Golden vectors of the reference's delta+ surface detection and shifting.

Runs the reference's deltaSPH solver with its delta+ module (src/modules/deltaPlus.py, enabled
by simulation.scheme = 'deltaPlus', src/deltaSPH.py:119-122) through oracle/ref_step.py on a
perturbed dam-break block and records, in float32 and float64:
  * surface: the inputs of the first detectSurface call (state, fluid / wall / wall-wall pair
    lists, wall arrays) and what it leaves behind (normalizationMatrix, fluidL, eigVals,
    fluidLambda, lambdaGrad, fluidNormal, angleMin/Max, fluidSurfaceMask and the walls' own
    normalization matrix and eigVals);
  * shift: with shifting.enabled the inputs of the first shift call (after the step's
    integration and the new search) and its outputs (shiftAmount before the adjustment,
    fluidUpdate and fluidSurfaceMask after it);
  * step: the acceleration, dpdt and wall pressure of the first right-hand side, whose
    pressure term is the delta+ one (computePressureAccelDeltaPlus, pressure.py:31-51).
The scene has more fluid particles than wall particles: computeFluidNormal indexes the fluid
arrays with wall indices (deltaPlus.py:150) and raises otherwise.
The reference's computeShiftAmount evaluates kernel(packing, support) on a Python float, which
its torch.pow rejects (deltaPlus.py:90); the harness hands that one argument over as a 0-d
tensor of the run's dtype and changes nothing else.
Needs the reference checkout; writes tests/golden/surface_golden.npz.
Usage:  python tests/golden/make_surface_golden.py
"""
from __future__ import annotations

import importlib
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import ref_step  # noqa: E402
from make_step_golden import perturbed_scene  # noqa: E402

SCENE = dict(seed=5, nx=32, ny=32, tank=(0.4, 0.4))
STATE_IN = ("fluidPosition", "fluidVelocity", "fluidDensity", "fluidArea", "fluidVolume", "fluidNeighbors",
            "fluidDistances", "fluidRadialDistances")
SURF_OUT = ("normalizationMatrix", "fluidL", "eigVals", "fluidLambda", "lambdaGrad", "fluidNormal", "angleMin",
            "angleMax", "fluidSurfaceMask")


def _np(v):
    return v.detach().clone().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)


def _walls(bm, out, tag):
    out[f"{tag}boundaryToFluidNeighbors"] = _np(bm.boundaryToFluidNeighbors)
    out[f"{tag}boundaryToFluidNeighborDistances"] = _np(bm.boundaryToFluidNeighborDistances)
    out[f"{tag}boundaryToFluidNeighborRadialDistances"] = _np(bm.boundaryToFluidNeighborRadialDistances)
    out[f"{tag}boundaryDensity"] = _np(bm.boundaryDensity)
    out[f"{tag}boundaryVolume"] = _np(bm.boundaryVolume)
    out[f"{tag}boundaryPositions"] = _np(bm.boundaryPositions)


def run(prec, shifting):
    sc = perturbed_scene(SCENE["seed"], nx=SCENE["nx"], ny=SCENE["ny"], tank=SCENE["tank"])
    sim = ref_step.make_simulation(sc, precision=prec, scheme="deltaPlus", diffusion="deltaSPH")
    dtype = sim.dtype
    dp = importlib.import_module("src.modules.deltaPlus")
    bm = sim.boundaryModule
    cap = {}
    sm = sim.shiftingModule
    orig_detect, orig_shift, orig_amount = sm.detectSurface, sm.shift, sm.computeShiftAmount
    kernel = dp.kernel

    def detect(state, s):
        if "surface" not in cap:
            d = {f"in_{k}": _np(state[k]) for k in STATE_IN}
            _walls(bm, d, "in_")
            orig_detect(state, s)
            for k in SURF_OUT:
                d[f"out_{k}"] = _np(state[k])
            d["out_boundaryNormalizationMatrix"] = _np(bm.normalizationMatrix)
            d["out_boundaryEigVals"] = _np(bm.eigVals)
            d["in_boundaryToBoundaryNeighbors"] = _np(bm.boundaryToBoundaryNeighbors)
            d["in_boundaryToBoundaryNeighborDistances"] = _np(bm.boundaryToBoundaryNeighborDistances)
            d["in_boundaryToBoundaryNeighborRadialDistances"] = _np(bm.boundaryToBoundaryNeighborRadialDistances)
            cap["surface"] = d
        else:
            orig_detect(state, s)

    def amount(state, s):
        orig_amount(state, s)
        cap.setdefault("shift", {})["out_shiftAmount"] = _np(state["shiftAmount"])

    def shift(state, s):
        d = cap.setdefault("shift", {})
        for k in STATE_IN + ("fluidNormal", "fluidSurfaceMask"):
            d[f"in_{k}"] = _np(state[k])
        _walls(bm, d, "in_")
        dp.kernel = lambda q, h: kernel(q if isinstance(q, torch.Tensor) else torch.tensor(q, dtype=dtype), h)
        try:
            orig_shift(state, s)
        finally:
            dp.kernel = kernel
        d["out_fluidUpdate"] = _np(state["fluidUpdate"])
        d["out_fluidSurfaceMask"] = _np(state["fluidSurfaceMask"])

    sm.detectSurface = detect
    sm.computeShiftAmount = amount
    sm.shift = shift
    sim.config["shifting"]["enabled"] = shifting
    orig_timestep = sim.timestep

    def timestep():
        res = orig_timestep()
        if "step" not in cap:   # the first right-hand side (deltaPlus pressure term, pressure.py:31-51)
            st = sim.simulationState
            cap["step"] = {"out_fluidAcceleration": _np(st["fluidAcceleration"]), "out_dpdt": _np(st["dpdt"]),
                           "out_boundaryPressure": _np(bm.pressure)}
        return res

    sim.timestep = timestep
    sim.integrate()
    cfg = sim.config
    meta = {"h": float(sc["h"]), "dx": sc["dx"], "tank": sc["tank"], "c0": float(cfg["fluid"]["c0"]),
            "rho0": float(cfg["fluid"]["restDensity"]), "packing": float(cfg["particle"]["packing"]),
            "alpha": float(cfg["diffusion"]["alpha"]), "delta": float(cfg["diffusion"]["delta"]),
            "n": len(sc["pos"]), "nb": int(bm.numPtcls)}
    return sc, cap, meta


def main():
    torch.set_num_threads(4)
    out = {}
    meta = {}
    for prec in ("single", "double"):
        tag = "" if prec == "single" else "f64_"
        sc, cap, m = run(prec, shifting=True)
        meta = m
        for k in ("pos", "vel", "rho", "area", "wall_pos", "ghost_pos", "wall_area", "vmin", "vmax"):
            out[f"scene_{k}"] = sc[k]
        for part in ("surface", "shift", "step"):
            for k, v in cap[part].items():
                if tag and part == "surface" and k.startswith("in_") and not k.startswith("in_boundary"):
                    continue          # the same values as the float32 run's (the first evaluation)
                if v.dtype == np.int64:
                    v = v.astype(np.int32)
                out[f"{tag}{part}/{k}"] = v
        print(prec, "ok", {p: len(cap[p]) for p in cap}, flush=True)
    out["meta"] = np.array(json.dumps(meta))
    path = os.path.join(HERE, "surface_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()
