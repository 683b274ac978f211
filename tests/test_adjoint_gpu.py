"""Differentiable drop rollouts (pytorchsph_gb300.adjoint): the GPU forward against the
restated reference step (oracle/sph_torch.py, float64), the GPU adjoint against torch
autograd through that restatement, and against central finite differences of the GPU
forward (float64).

The oracle evaluates pair geometry from float32-rounded positions (as the reference's
float-only search does) while the GPU rollout uses float64 positions, so forward states
agree to ~1e-7 relative.  For the gradient the restated step is rerun with the same pair
sets but float64 geometry (the GPU's formulation; float32 geometry alone moves this
gradient by 1.2e-4), and the two gradients must agree to 1e-8.  Finite differences of the
GPU forward are held to 1e-3."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def drop(n, A):
    from pytorchsph_gb300 import workloads
    sc = workloads.oscillating_drop(n, 0.5, A)
    dt = 0.1 * sc["h"] / 10.0
    return sc, dt


def oracle_rollout(sc, v0, alpha, steps, dt):
    import sph_torch as S
    p = S.Params(h=sc["h"], c0=10.0, diffusion="MOG", vmin=sc["vmin"], vmax=sc["vmax"], gravity=(0.0, 0.0),
                 point_source=True, alpha=alpha, kinematic=0.001)
    st = {"x": torch.from_numpy(sc["pos"]).double(), "v": v0, "rho": torch.from_numpy(sc["rho"]).double(),
          "area": torch.from_numpy(sc["area"]).double()}
    for _ in range(steps):
        new, _ = S.step(st, None, p, dt, "semiImplicitEuler", "deltaSPH", torch.float64)
        st = {"x": new["x"], "v": new["v"], "rho": new["rho"], "area": st["area"]}
    return st["x"], st["rho"]


def test_forward_matches_reference_step(cuda):
    from pytorchsph_gb300.adjoint import DropRollout
    sc, dt = drop(1500, 1.2)
    r = DropRollout(sc, 10.0, dt, device=cuda)
    x = r.x0.clone()
    v = torch.as_tensor(sc["vel"], dtype=torch.float64, device=cuda).clone()
    rho = r.rho0.clone()
    for _ in range(10):
        r.step(x, v, rho, 0.02)
    xr, rr = oracle_rollout(sc, torch.from_numpy(sc["vel"]).double(), 0.02, 10, dt)
    disp = (xr - torch.from_numpy(sc["pos"]).double()).numpy()
    assert rel(x.cpu().numpy() - sc["pos"], disp) < 1e-5
    assert rel(rho.cpu() - 1.0, rr.numpy() - 1.0) < 1e-4


def exact_rollout(sc, v0, alpha, steps, dt):
    """The restated step with the pair set of the float32 search but pair geometry from the
    float64 positions (the GPU rollout's geometry), differentiable by torch autograd."""
    import sph_torch as S
    p = S.Params(h=sc["h"], c0=10.0, diffusion="MOG", vmin=sc["vmin"], vmax=sc["vmax"], gravity=(0.0, 0.0),
                 point_source=True, alpha=alpha, kinematic=0.001)
    x = torch.from_numpy(sc["pos"]).double()
    v, rho, A = v0, torch.from_numpy(sc["rho"]).double(), torch.from_numpy(sc["area"]).double()
    for _ in range(steps):
        nb = S.search(x.detach().to(torch.float32), None, p.h, p.vmin, p.vmax, torch.float64)
        nb = S.Neighbors(S.make_pairs(x, x, nb.ff.i.numpy(), nb.ff.j.numpy(), p.h, torch.float64), None, None)
        a, _, dp, _ = S.deltasph_rhs({"x": x, "v": v, "rho": rho, "area": A}, None, nb, p, torch.float64)
        v, x, rho = v + dt * a, x + dt * (v + dt * a), rho + dt * dp / p.rho0
    return x


def test_adjoint_matches_autograd(cuda):
    from pytorchsph_gb300.adjoint import DropRollout
    sc, dt = drop(800, 1.0)
    steps = 8
    rng = np.random.default_rng(1)
    target = torch.as_tensor(sc["pos"] + 1e-3 * rng.standard_normal(sc["pos"].shape), dtype=torch.float64)
    v0 = torch.from_numpy(sc["vel"]).double().requires_grad_(True)
    alpha = torch.tensor(0.015, dtype=torch.float64, requires_grad=True)
    xT = exact_rollout(sc, v0, alpha, steps, dt)
    loss = ((xT - target) ** 2).sum() / len(sc["pos"])
    loss.backward()
    r = DropRollout(sc, 10.0, dt, checkpoint_every=3, device=cuda)
    L, gv, ga = r.loss_and_grad(torch.as_tensor(sc["vel"], dtype=torch.float64, device=cuda), 0.015,
                                target.to(cuda), steps)
    ref_loss = float(loss.detach())
    assert abs(L - ref_loss) <= 1e-9 * abs(ref_loss)
    assert rel(gv.cpu(), v0.grad) < 1e-8
    assert abs(ga - float(alpha.grad)) <= 1e-8 * abs(float(alpha.grad))


def test_adjoint_matches_finite_differences(cuda):
    from pytorchsph_gb300.adjoint import DropRollout
    sc, dt = drop(1200, 0.8)
    steps = 20
    tgt_sc, _ = drop(1200, 1.0)
    r = DropRollout(sc, 10.0, dt, checkpoint_every=7, device=cuda)
    v_t = torch.as_tensor(tgt_sc["vel"], dtype=torch.float64, device=cuda)
    target, _ = r.rollout(v_t, 0.02, steps)
    v0 = torch.as_tensor(sc["vel"], dtype=torch.float64, device=cuda)
    L, gv, ga = r.loss_and_grad(v0, 0.01, target, steps)
    rng = np.random.default_rng(0)
    idx = rng.choice(v0.numel(), 8, replace=False)
    eps = 1e-4
    fd, ad = [], []
    for k in idx:
        e = torch.zeros(v0.numel(), dtype=torch.float64, device=cuda)
        e[k] = eps
        e = e.reshape(v0.shape)
        fd.append((r.loss(v0 + e, 0.01, target, steps) - r.loss(v0 - e, 0.01, target, steps)) / (2 * eps))
        ad.append(float(gv.reshape(-1)[k]))
    assert rel(ad, fd) < 1e-3
    fa = (r.loss(v0, 0.01 + 1e-4, target, steps) - r.loss(v0, 0.01 - 1e-4, target, steps)) / 2e-4
    assert abs(ga - fa) <= 1e-3 * abs(fa)


def test_autograd_function_matches_adjoint_and_gradcheck(cuda):
    """DropRolloutFunction (torch.autograd) gives the adjoint's gradients bit for bit, and
    torch.autograd.gradcheck accepts it on a small float64 case."""
    from pytorchsph_gb300.adjoint import DropRollout, drop_rollout
    sc, dt = drop(600, 1.0)
    steps = 6
    r = DropRollout(sc, 10.0, dt, checkpoint_every=4, device=cuda)
    rng = np.random.default_rng(3)
    target = torch.as_tensor(sc["pos"] + 1e-3 * rng.standard_normal(sc["pos"].shape), dtype=torch.float64,
                             device=cuda)
    v0 = torch.as_tensor(sc["vel"], dtype=torch.float64, device=cuda).requires_grad_(True)
    alpha = torch.tensor(0.015, dtype=torch.float64, device=cuda, requires_grad=True)
    xT = drop_rollout(r, v0, alpha, steps)
    loss = ((xT - target) ** 2).sum() / r.n
    loss.backward()
    L, gv, ga = r.loss_and_grad(v0.detach(), 0.015, target, steps)
    assert float(loss.detach()) == L
    assert torch.equal(v0.grad, gv) and float(alpha.grad) == ga
    # gradcheck on a smaller drop (pair sets do not change under its perturbations)
    sc2, dt2 = drop(120, 1.0)
    r2 = DropRollout(sc2, 10.0, dt2, checkpoint_every=2, device=cuda)
    v2 = torch.as_tensor(sc2["vel"], dtype=torch.float64, device=cuda).requires_grad_(True)
    a2 = torch.tensor(0.02, dtype=torch.float64, device=cuda, requires_grad=True)
    assert torch.autograd.gradcheck(lambda v, a: drop_rollout(r2, v, a, 3), (v2, a2), eps=1e-6, atol=1e-7,
                                    rtol=1e-4, fast_mode=True)


def test_float32_adjoint_at_drop_scale_matches_float64_differences(cuda):
    """The differentiable drop at full size: about 16,384 particles, 200 steps, checkpoints
    every 20 steps, float32 forward and adjoint through DropRolloutFunction; target rollout
    with A = 1.0, alpha = 0.02, start A = 0.8, alpha = 0.01; loss mean |x_T - x*_T|^2.
    Checked against float64 central differences (eps = 1e-4) of the loss on 64 seeded velocity
    components and on alpha: relative error (to the largest component) at most 1e-3."""
    from pytorchsph_gb300.adjoint import DropRollout, drop_rollout
    sc, dt = drop(16384, 0.8)
    tgt, _ = drop(16384, 1.0)
    steps = 200
    r64 = DropRollout(sc, 10.0, dt, fp64=True, checkpoint_every=20, device=cuda)
    r32 = DropRollout(sc, 10.0, dt, fp64=False, checkpoint_every=20, device=cuda)
    target, _ = r64.rollout(torch.as_tensor(tgt["vel"], dtype=torch.float64, device=cuda), 0.02, steps)
    v0 = torch.as_tensor(sc["vel"], dtype=torch.float32, device=cuda).requires_grad_(True)
    alpha = torch.tensor(0.01, dtype=torch.float32, device=cuda, requires_grad=True)
    xT = drop_rollout(r32, v0, alpha, steps)
    loss = ((xT - target.float()) ** 2).sum() / r32.n
    loss.backward()
    v64 = v0.detach().double()
    rng = np.random.default_rng(5)
    idx = rng.choice(v64.numel(), 64, replace=False)
    eps = 1e-4
    fd, ad = [], []
    for k in idx:
        e = torch.zeros(v64.numel(), dtype=torch.float64, device=cuda)
        e[k] = eps
        e = e.reshape(v64.shape)
        fd.append((r64.loss(v64 + e, 0.01, target, steps) - r64.loss(v64 - e, 0.01, target, steps)) / (2 * eps))
        ad.append(float(v0.grad.reshape(-1)[k]))
    assert rel(ad, fd) < 1e-3, rel(ad, fd)
    fa = (r64.loss(v64, 0.01 + eps, target, steps) - r64.loss(v64, 0.01 - eps, target, steps)) / (2 * eps)
    assert abs(float(alpha.grad) - fa) <= 1e-3 * abs(fa), (float(alpha.grad), fa)


def test_adjoint_matches_reference_finite_differences(cuda):
    """The GPU adjoint (float64) against the reference's own gradient: central finite
    differences (eps 1e-4) of the reference's forward rollout, 40 steps of a ~550-particle
    drop moved into a 3 x 3 tank whose walls stay out of reach
    (tests/golden/drop_fd_golden.npz, made by make_drop_fd_golden.py; the reference's step
    does not run under torch autograd).  The GPU forward reproduces the reference's final
    positions (1e-8; the restated step gets 7e-10) and loss, and its gradient the 16
    velocity components and alpha to 1e-4."""
    import os
    from pytorchsph_gb300.adjoint import DropRollout
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "drop_fd_golden.npz"))
    c, tank = float(g["center"]), float(g["tank"])
    sc = {"pos": g["pos"], "rho": g["rho"], "area": g["area"], "support": g["support"],
          "vmin": np.zeros(2, np.float32), "vmax": np.full(2, tank, np.float32)}
    r = DropRollout(sc, 10.0, float(g["dt"]), fp64=True, checkpoint_every=10, device=cuda, point_center=(c, c))
    steps = int(g["steps"])
    v0 = torch.as_tensor(g["vel"], dtype=torch.float64, device=cuda)
    target = torch.as_tensor(g["target"], dtype=torch.float64, device=cuda)
    xT, _ = r.rollout(v0, 0.01, steps)
    assert np.abs(xT.cpu().numpy() - g["x_final"]).max() < 1e-8
    loss, gv, ga = r.loss_and_grad(v0, 0.01, target, steps)
    assert abs(loss - float(g["loss"])) <= 1e-4 * float(g["loss"])
    ad = gv.reshape(-1).cpu().numpy()[g["idx"]]
    assert rel(ad, g["fd"]) < 1e-4, rel(ad, g["fd"])
    assert abs(ga - float(g["fd_alpha"])) <= 1e-4 * abs(float(g["fd_alpha"])), (ga, float(g["fd_alpha"]))
