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
