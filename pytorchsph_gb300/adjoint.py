"""Differentiable deltaSPH rollouts of a free fluid (the oscillating drop): forward steps and
their discrete adjoint on the GPU, with checkpointing.

The step is the reference's deltaSPH right-hand side (src/deltaSPH.py:146-200: point
source or gravity, continuity, MOG density diffusion, Tait pressure, artificial and laminar
viscosity) integrated by semi-implicit Euler (src/simulationBase.py:647-652).  Each step
searches neighbors on the GPU (the reference predicate, pairs in (i, j) order), then runs
`sph_drop_rhs` and `sph_drop_integrate`; the adjoint (`sph_drop_adjoint`) runs the steps
backwards, recomputing each checkpoint segment's states forward first.  Scalars are float64
(default) or float32; the search always sees float32 positions, as the reference's does.

Gradients are with respect to the initial velocity field and the artificial viscosity alpha.
`DropRolloutFunction` puts the rollout behind torch.autograd: its forward records every
step's neighbor list and a checkpoint every `checkpoint_every` steps, and its backward
recomputes each segment's states from its checkpoint with the recorded lists (no search)
and runs the adjoint kernels backwards.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from .search import GridSearch
from .sim import SphParamsC


class DropRollout:
    def __init__(self, scene: dict, c0: float, dt: float, kinematic: float = 0.001, delta: float = 0.1,
                 rest_density: float = 1000.0, gravity=(0.0, 0.0), point_source: bool = True,
                 point_magnitude: float = 1.0, fp64: bool = True, checkpoint_every: int = 20, device=None,
                 point_center=(0.0, 0.0)):
        self.dev = torch.device(device or torch.device("cuda", torch.cuda.current_device()))
        self.fp64 = bool(fp64)
        self.dtype = torch.float64 if fp64 else torch.float32
        t = lambda a: torch.as_tensor(np.asarray(a), dtype=self.dtype, device=self.dev).contiguous()
        self.n = len(scene["pos"])
        self.x0 = t(scene["pos"]).reshape(self.n, 2)
        self.rho0 = t(scene["rho"])
        self.area = t(scene["area"])
        self.support32 = torch.as_tensor(np.asarray(scene["support"], np.float32), device=self.dev).contiguous()
        self.h = float(np.float32(scene["support"][0]))
        self.vmin = np.asarray(scene["vmin"], np.float32)
        self.vmax = np.asarray(scene["vmax"], np.float32)
        self.dt = float(dt)
        self.every = int(checkpoint_every)
        self.P = SphParamsC()
        P = self.P
        P.support = self.h
        P.rest_density = rest_density
        P.c0 = c0
        P.gamma = 7.0
        P.delta = delta
        P.kinematic = kinematic
        P.gravity[0], P.gravity[1] = gravity
        P.point_source = int(point_source)
        P.point_magnitude = point_magnitude
        P.point_center[0], P.point_center[1] = point_center
        P.density_diffusion = 1            # MOG
        self.search = GridSearch(self.dev)
        self.acc = torch.empty((self.n, 2), dtype=self.dtype, device=self.dev)
        self.dpdt = torch.empty(self.n, dtype=self.dtype, device=self.dev)
        self.steps_run = 0

    # ------------------------------------------------------------------ forward
    def pairs(self, x):
        """(row offsets int32 [n+1], columns int64 [P]) of the reference pair list at x."""
        x32 = x.to(torch.float32).contiguous()
        res = self.search.run(x32, self.support32, kernel_support=self.h, density=False, min_coord=self.vmin,
                              max_coord=self.vmax)
        nb, _, _ = res.to_coo(distances=False)
        rows = nb[0].contiguous()
        cols = nb[1].contiguous()
        off = torch.empty(self.n + 1, dtype=torch.int32, device=self.dev)
        N.call("sph_row_offsets", N.ptr(rows), rows.shape[0], self.n, N.ptr(off), N.stream_ptr())
        return off, cols

    def step(self, x, v, rho, alpha, pairs=None):
        """Advance (x, v, rho) in place by one step; returns the pairs it used."""
        off, cols = pairs or self.pairs(x)
        self.P.alpha = float(alpha)
        st = N.stream_ptr()
        N.call("sph_drop_rhs", int(self.fp64), self.n, N.ptr(off), N.ptr(cols), N.ptr(x), N.ptr(v), N.ptr(rho),
               N.ptr(self.area), ctypes.byref(self.P), N.ptr(self.acc), N.ptr(self.dpdt), st)
        N.call("sph_drop_integrate", int(self.fp64), self.n, N.ptr(x), N.ptr(v), N.ptr(rho), N.ptr(self.acc),
               N.ptr(self.dpdt), self.dt, float(self.P.rest_density), st)
        self.steps_run += 1
        return off, cols

    def rollout(self, v0, alpha, steps, checkpoints=False, record_pairs=False):
        """Final positions after `steps` steps from (x0, v0, rho0) and the checkpoints (the states
        at every `checkpoint_every`-th step, when asked for); with record_pairs also the list of
        every step's (offsets, columns)."""
        x = self.x0.clone()
        v = v0.to(self.dtype).reshape(self.n, 2).clone()
        rho = self.rho0.clone()
        ck = {}
        pairs = []
        for k in range(steps):
            if checkpoints and k % self.every == 0:
                ck[k] = (x.clone(), v.clone(), rho.clone())
            pr = self.step(x, v, rho, alpha)
            if record_pairs:
                pairs.append(pr)
        return (x, ck, pairs) if record_pairs else (x, ck)

    # ------------------------------------------------------------------ adjoint
    def vjp(self, ck, alpha, steps, grad_x, pairs=None):
        """Vector-Jacobian product of the rollout: given d(objective)/d(x_T) = grad_x [n, 2],
        returns (d/d v0 [n, 2], d/d alpha).  Each checkpoint segment's states are recomputed
        forward from its checkpoint, with the recorded pair lists when given (else searched
        again), and the adjoint kernels run the segment's steps backwards."""
        lx = grad_x.to(self.dtype).reshape(self.n, 2).contiguous().clone()
        lv = torch.zeros_like(lx)
        lr = torch.zeros_like(self.rho0)
        nx, nv, nr = torch.empty_like(lx), torch.empty_like(lv), torch.empty_like(lr)
        dalpha = torch.zeros(self.n, dtype=self.dtype, device=self.dev)
        da = torch.empty_like(dalpha)
        self.P.alpha = float(alpha)
        for s0 in sorted(ck, reverse=True):
            s1 = min(s0 + self.every, steps)
            x, v, rho = (t.clone() for t in ck[s0])
            seg = []
            for k in range(s0, s1):          # recompute the segment's states
                state = (x.clone(), v.clone(), rho.clone())
                pr = self.step(x, v, rho, alpha, pairs[k] if pairs is not None else None)
                seg.append((state, pr))
            for (xs, vs, rs), (off, cols) in reversed(seg):
                N.call("sph_drop_adjoint", int(self.fp64), self.n, N.ptr(off), N.ptr(cols), N.ptr(xs), N.ptr(vs),
                       N.ptr(rs), N.ptr(self.area), ctypes.byref(self.P), self.dt, N.ptr(lx), N.ptr(lv), N.ptr(lr),
                       N.ptr(nx), N.ptr(nv), N.ptr(nr), N.ptr(da), N.stream_ptr())
                dalpha += da
                lx, nx = nx, lx
                lv, nv = nv, lv
                lr, nr = nr, lr
        return lv, dalpha.sum()

    def loss_and_grad(self, v0, alpha, target, steps):
        """Loss mean_i |x_T,i - target_i|^2 and its gradients with respect to v0 [n, 2] and alpha."""
        xT, ck, pairs = self.rollout(v0, alpha, steps, checkpoints=True, record_pairs=True)
        diff = xT - target.to(self.dtype)
        loss = float((diff * diff).sum().item()) / self.n
        lv, da = self.vjp(ck, alpha, steps, (2.0 / self.n) * diff, pairs)
        return loss, lv, float(da.item())

    def loss(self, v0, alpha, target, steps):
        xT, _ = self.rollout(v0, alpha, steps)
        d = xT - target.to(self.dtype)
        return float((d * d).sum().item()) / self.n


class DropRolloutFunction(torch.autograd.Function):
    """Final positions x_T [n, 2] of a `steps`-step DropRollout as a differentiable function of
    the initial velocities v0 [n, 2] and the artificial viscosity alpha (0-d tensor).

    Forward: the GPU rollout, recording each step's neighbor list and a checkpoint every
    `rollout.every` steps.  Backward: DropRollout.vjp with the recorded lists (the adjoint
    kernels of sph_drop_adjoint).  The rollout's precision (float32 or float64) is the
    rollout's; gradients come back in the inputs' dtypes."""

    @staticmethod
    def forward(ctx, v0, alpha, rollout, steps):
        a = float(alpha)
        xT, ck, pairs = rollout.rollout(v0.detach(), a, int(steps), checkpoints=True, record_pairs=True)
        ctx.rollout, ctx.ck, ctx.pairs, ctx.alpha, ctx.steps = rollout, ck, pairs, a, int(steps)
        ctx.v_dtype, ctx.a_dtype = v0.dtype, (alpha.dtype if isinstance(alpha, torch.Tensor) else torch.float64)
        ctx.a_device = alpha.device if isinstance(alpha, torch.Tensor) else v0.device
        return xT

    @staticmethod
    def backward(ctx, grad_x):
        gv, ga = ctx.rollout.vjp(ctx.ck, ctx.alpha, ctx.steps, grad_x, ctx.pairs)
        gv = gv.to(ctx.v_dtype) if ctx.needs_input_grad[0] else None
        ga = ga.to(device=ctx.a_device, dtype=ctx.a_dtype) if ctx.needs_input_grad[1] else None
        return gv, ga, None, None


def drop_rollout(rollout: DropRollout, v0: torch.Tensor, alpha, steps: int) -> torch.Tensor:
    """x_T = DropRolloutFunction.apply(v0, alpha, rollout, steps)."""
    if not isinstance(alpha, torch.Tensor):
        alpha = torch.tensor(float(alpha), dtype=torch.float64, device=v0.device)
    return DropRolloutFunction.apply(v0, alpha, rollout, steps)
