"""Golden gradients of the differentiable drop from the reference's own step.

The reference's time step does not run under torch autograd (its modules update tensors
in place, e.g. src/modules/gravity.py:51), so its gradient is taken by float64 central
finite differences of its own forward rollout instead.  The scene is the oscillating drop
(lattice disc of radius 0.5, v0 = A (x, -y)) moved into a 3 x 3 tank, centred at (1.5, 1.5):
the reference needs its solid walls, and at a metre from the fluid they take part in no
pair during the rollout, so the fluid sees the free drop.  Physics as the GPU rollout
(pytorchsph_gb300.adjoint.DropRollout): deltaSPH with MOG density diffusion, point source
of magnitude 1 at the centre (potential field), c0 = 10, dt = 0.1 h / c0, semi-implicit
Euler, the reference's summations in float64 (its search sees float32 positions).

Loss: mean over particles of |x_T - x*_T|^2 after STEPS steps, x* the rollout with A = 1.0,
alpha = 0.02 from the same start; gradients at A = 0.8, alpha = 0.01 with respect to 16
seeded initial velocity components and alpha, eps = 1e-4.
Needs the reference checkout; writes tests/golden/drop_fd_golden.npz.
Usage:  python tests/golden/make_drop_fd_golden.py
"""
from __future__ import annotations

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

N_TARGET = 600
STEPS = 40
CENTER = 1.5
TANK = 3.0
EPS = 1e-4
COMPONENTS = 16


def scene(amplitude):
    sc = dict(workloads.oscillating_drop(N_TARGET, 0.5, amplitude))
    sc["pos"] = (sc["pos"] + np.float32(CENTER)).astype(np.float32)
    sc["tank"] = (TANK, TANK)
    sc["column_height"] = 1.0
    w, g = workloads.tank_walls(TANK, TANK, sc["dx"], layers=3)
    sc["wall_pos"], sc["ghost_pos"] = w, g
    sc["wall_area"] = np.full(len(w), np.float32(sc["dx"] ** 2), np.float32)
    sc["vmin"] = np.array([0, 0], np.float32)
    sc["vmax"] = np.array([TANK, TANK], np.float32)
    return sc


def rollout(sc, v0, alpha, dt):
    sim = ref_step.make_simulation(sc, precision="double", scheme="deltaSPH", diffusion="MOG",
                                   integration="semiImplicitEuler", dt=dt, c0=10.0, alpha=alpha, gravity=1.0,
                                   point_source=True, point_center=(CENTER, CENTER))
    sim.perennialState["fluidVelocity"] = torch.as_tensor(v0, dtype=torch.float64).clone()
    sim.simulationState = sim.setupSimulationState(sim.perennialState)
    for _ in range(STEPS):
        sim.integrate()
    # integrateValues (src/simulationBase.py:563-568) writes the new state into
    # simulationState; perennialState keeps the state the step started from
    return sim.simulationState["fluidPosition"].detach().numpy().astype(np.float64)


def main():
    torch.set_num_threads(8)
    start, tgt = scene(0.8), scene(1.0)
    dt = 0.1 * start["h"] / 10.0
    v0 = start["vel"].astype(np.float64)
    target = rollout(tgt, tgt["vel"].astype(np.float64), 0.02, dt)
    loss = lambda x: float(((x - target) ** 2).sum() / len(x))
    x0 = rollout(start, v0, 0.01, dt)
    rng = np.random.default_rng(11)
    idx = rng.choice(v0.size, COMPONENTS, replace=False)
    fd = []
    for k in idx:
        e = np.zeros(v0.size)
        e[k] = EPS
        e = e.reshape(v0.shape)
        fd.append((loss(rollout(start, v0 + e, 0.01, dt)) - loss(rollout(start, v0 - e, 0.01, dt))) / (2 * EPS))
        print(k, fd[-1], flush=True)
    fa = (loss(rollout(start, v0, 0.01 + EPS, dt)) - loss(rollout(start, v0, 0.01 - EPS, dt))) / (2 * EPS)
    print("alpha", fa)
    np.savez_compressed(os.path.join(HERE, "drop_fd_golden.npz"), pos=start["pos"], vel=start["vel"],
                        rho=start["rho"], area=start["area"], support=start["support"], h=start["h"], dt=dt,
                        steps=STEPS, center=CENTER, tank=TANK, eps=EPS, target=target, x_final=x0, loss=loss(x0),
                        idx=idx.astype(np.int64), fd=np.array(fd), fd_alpha=fa)


if __name__ == "__main__":
    main()
