"""Golden per-step iteration counts of the reference's DFSPH solver on settling dam breaks.

A block at rest dropped into a tank first settles under gravity: the reference's density
solve (src/modules/dfsph.py:195-260, relaxed Jacobi, omega 0.5, threshold 1e-4, 2-100
iterations) runs to its cap for the first steps and then converges in the minimum of two.
This records, for square blocks of 64 x 64 and 128 x 128 particles at dx = 0.002 in a tank
of four by two block widths, the reference's density and divergence iteration counts and
its adaptive dt for 20 steps of semi-implicit Euler (src/simulationBase.py:632-705,
src/modules/adaptiveDT.py:59-95), run through its own simulation class in float32.
Needs the reference checkout; writes tests/golden/dfsph_iters.json.
Usage:  python tests/golden/make_dfsph_iters_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import ref_step  # noqa: E402
from pytorchsph_gb300 import workloads  # noqa: E402

SOLVER = dict(minDensitySolverIterations=2, minDivergenceSolverIterations=2, maxDensitySolverIterations=100,
              maxDivergenceSolverIterations=100, densityThreshold=1e-4, divergenceThreshold=1e-3,
              divergenceSolver=True, relaxedJacobiOmega=0.5)
BLOCKS = (64, 128)
STEPS = 20
DX = 0.002
DT0 = 2e-4
KINEMATIC = 0.01


def main():
    torch.set_num_threads(8)
    out = {"dx": DX, "dt0": DT0, "kinematic": KINEMATIC, "steps": STEPS, "solver": SOLVER}
    for nb in BLOCKS:
        sc = workloads.dam_break(nb, nb, DX, (4 * nb * DX, 2 * nb * DX))
        sim = ref_step.make_simulation(sc, precision="single", scheme="dfsph", integration="semiImplicitEuler",
                                       dt=DT0, kinematic=KINEMATIC, dfsph=SOLVER, cfl_fixed=False)
        rec = {"density": [], "divergence": [], "dt": []}
        for _ in range(STEPS):
            sim.integrate()
            s = sim.simulationState
            rec["density"].append(len(s["densityIterations"]))
            rec["divergence"].append(len(s["divergenceIterations"]))
            rec["dt"].append(float(s["dt"]))
        print(nb, rec["density"], flush=True)
        out[f"{nb}x{nb}"] = rec
    with open(os.path.join(HERE, "dfsph_iters.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
