"""ORACLE — test infrastructure only.  Plain-torch restatement of the reference's SPH
summations, wall terms, solvers and integrators (wi-re/pytorchSPH), in any float dtype.

It follows the reference formula by formula on COO pair lists (pairs ordered (i, j), sums
by index_add_ in pair order, like `util.scatter_sum`, src/util.py:35-51) and keeps the
reference's quirks.  It is pinned against the reference itself (tests/golden/, generated by
tests/golden/make_step_golden.py through oracle/ref_step.py) and is what the GPU kernels are
compared with at sizes and step counts the reference harness cannot reach.  Nothing in the
product imports it.

Conventions (as in the reference): pairs (i, j) include i == j; e_ij = (x_i - x_j)/r, or 0
when r < 1e-7 (src/modules/neighborSearch.py:218-222); q = r / h with the scalar support h
(:223); rho is the relative density (rho_tilde), absolute density = rho * rho0.
Wall pairs come from the wall side (query = wall b, src/modules/solidBoundary.py:618-642):
the fluid-side sums use e = (x_f - x_b)/r, the wall-side DFSPH sums e = (x_b - x_f)/r.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

import nsearch as ns

PI = math.pi


# ----------------------------------------------------------------- kernels (src/kernels.py:20-33)
def W(q, h):
    return torch.pow(1.0 - q, 4) * (1.0 + 4.0 * q) * (7.0 / PI) / h ** 2


def gradW(q, e, h):
    return -e * (7.0 / PI) / h ** 3 * (20.0 * q * (1.0 - q) ** 3)[:, None]


def spiky(q, e, h):
    return -e * 30.0 / PI / h ** 3 * ((1.0 - q) ** 2)[:, None]


def ssum(vals, idx, n):
    out = torch.zeros((n,) + tuple(vals.shape[1:]), dtype=vals.dtype)
    return out.index_add_(0, idx, vals)


# ----------------------------------------------------------------- pinv2x2 (src/util.py:386-433)
def pinv2x2(M):
    a, b, c, d = M[:, 0, 0], M[:, 0, 1], M[:, 1, 0], M[:, 1, 1]
    theta = 0.5 * torch.atan2(2 * a * c + 2 * b * d, a ** 2 + b ** 2 - c ** 2 - d ** 2)
    ct, st = torch.cos(theta), torch.sin(theta)
    U = torch.zeros_like(M)
    U[:, 0, 0], U[:, 0, 1], U[:, 1, 0], U[:, 1, 1] = ct, -st, st, ct
    S1 = a ** 2 + b ** 2 + c ** 2 + d ** 2
    S2 = torch.sqrt((a ** 2 + b ** 2 - c ** 2 - d ** 2) ** 2 + 4 * (a * c + b * d) ** 2)
    o1 = torch.sqrt((S1 + S2) / 2)
    o2 = torch.sqrt((S1 - S2) / 2)
    phi = 0.5 * torch.atan2(2 * a * b + 2 * c * d, a ** 2 - b ** 2 + c ** 2 - d ** 2)
    cp, sp = torch.cos(phi), torch.sin(phi)
    s11 = torch.sign((a * ct + c * st) * cp + (b * ct + d * st) * sp)
    s22 = torch.sign((a * st - c * ct) * sp + (-b * st + d * ct) * cp)
    V = torch.zeros_like(M)
    V[:, 0, 0], V[:, 0, 1], V[:, 1, 0], V[:, 1, 1] = cp * s11, -sp * s22, sp * s11, cp * s22
    o1i = torch.where(torch.abs(o1) > 1e-5, 1 / o1, torch.zeros_like(o1))
    o2i = torch.where(torch.abs(o2) > 1e-5, 1 / o2, torch.zeros_like(o2))
    S_1 = torch.diag_embed(torch.stack([o1i, o2i], 1))
    return torch.matmul(torch.matmul(V, S_1), U.mT)


# ----------------------------------------------------------------- pairs
@dataclass
class Pairs:
    i: torch.Tensor          # row (query)
    j: torch.Tensor          # column
    e: torch.Tensor          # unit vector (x_row - x_col)/r (0 when r < 1e-7)
    q: torch.Tensor          # r / h


def make_pairs(xi, xj, rows, cols, h, dtype):
    """Distances of src/modules/neighborSearch.py:218-223 for pairs (rows into xi, cols into xj)."""
    i = torch.as_tensor(np.asarray(rows, np.int64))
    j = torch.as_tensor(np.asarray(cols, np.int64))
    d = (xi[i] - xj[j]).to(dtype)
    r = torch.linalg.norm(d, axis=1)
    e = torch.where((r >= 1e-7)[:, None], d / torch.where(r >= 1e-7, r, torch.ones_like(r))[:, None],
                    torch.zeros_like(d))
    return Pairs(i, j, e, r / h)


def canonical(rows, cols):
    key = np.sort(np.asarray(rows, np.int64) * (1 << 32) + np.asarray(cols, np.int64))
    return key >> 32, key & 0xFFFFFFFF


@dataclass
class Neighbors:
    ff: Pairs                 # fluid-fluid
    bf: Pairs | None          # wall b -> fluid f (rows = b)
    gf: Pairs | None          # ghost g -> fluid f (rows = g)


def search(x32, walls, h, vmin, vmax, dtype, ghost_from_walls=False):
    """Pairs with the reference's exact search (the C oracle, pinned to cppSrc/neighSearch.cpp).
    ghost_from_walls: the ghost pair list is queried from the wall positions, as
    boundaryNeighborhoodSearch does for the deltaMLS and MLSPressure wall pressures
    (solidBoundary.py:639-640)."""
    xs = x32.detach().to(torch.float32).numpy()
    hs = np.full(len(xs), np.float32(h), np.float32)
    si = ns.SortInfo(xs, hs, vmin, vmax)
    r, c = ns.nl_cells(si)
    r, c = canonical(r, c)
    X = x32.to(dtype)
    ff = make_pairs(X, X, r, c, h, dtype)
    bf = gf = None
    if walls is not None and walls.n > 0:
        hb = np.full(walls.n, np.float32(h), np.float32)
        rb, cb = ns.nl_query(si, walls.x.numpy(), hb)
        rb, cb = canonical(rb, cb)
        bf = make_pairs(walls.x.to(dtype), X, rb, cb, h, dtype)
        xq = walls.x if ghost_from_walls else walls.xg
        rg, cg = ns.nl_query(si, xq.numpy(), hb)
        rg, cg = canonical(rg, cg)
        gf = make_pairs(xq.to(dtype), X, rg, cg, h, dtype)
    return Neighbors(ff, bf, gf)


@dataclass
class Walls:
    x: torch.Tensor          # wall positions float32 [Nb, 2]
    xg: torch.Tensor         # ghost positions
    area: torch.Tensor       # boundaryVolume = pi r^2
    density_term: torch.Tensor | None = None   # static wall-wall kernel sum (summation density)

    @property
    def n(self):
        return self.x.shape[0]


def wall_density_term(walls, h, dtype):
    """boundaryDensityTerm = sum over wall neighbors (|x_b - x_b'| <= h) of W * A_b'
    (src/modules/solidBoundary.py:180-200); W vanishes at q = 1, so <= vs < does not matter."""
    xb = walls.x.to(torch.float64)
    d = torch.cdist(xb, xb)
    bi, bj = torch.nonzero(d <= h, as_tuple=True)
    dd = walls.x.to(dtype)[bi] - walls.x.to(dtype)[bj]
    q = torch.linalg.norm(dd, axis=1) / h
    return ssum(W(q, h) * walls.area.to(dtype)[bj], bi, walls.n)


# ----------------------------------------------------------------- parameters
@dataclass
class Params:
    h: float
    rho0: float = 1000.0
    c0: float = 50.0
    gamma: float = 7.0
    alpha: float = 0.01
    delta: float = 0.1
    kinematic: float = 0.001
    gravity: tuple = (0.0, -9.81)
    point_source: bool = False          # gravity as -g (x - c) (potential field)
    point_magnitude: float = 1.0
    point_center: tuple = (0.0, 0.0)   # gravity.center
    boundary_pressure: str = "PBSPH"    # pressure.boundaryPressureTerm: PBSPH | ghostMLS | deltaMLS | MLSPressure
    diffusion: str = "MOG"              # "MOG" | "deltaSPH"
    boundary_diffusion: bool = True
    vmin: np.ndarray = field(default_factory=lambda: np.zeros(2, np.float32))
    vmax: np.ndarray = field(default_factory=lambda: np.ones(2, np.float32))
    # DFSPH
    min_density_iters: int = 2
    max_density_iters: int = 100
    density_threshold: float = 1e-4
    divergence_solver: bool = True
    min_divergence_iters: int = 2
    max_divergence_iters: int = 100
    divergence_threshold: float = 1e-3
    omega_boundary: float = 0.5

    @property
    def eps(self):
        return self.h ** 2 * 0.1


# ----------------------------------------------------------------- deltaSPH pieces
def tait(rho, p: Params):
    """TaitEOS, src/modules/pressure.py:82-83 (and the wall's, solidBoundary.py:803-804)."""
    return p.rho0 * p.c0 ** 2 / p.gamma * (torch.pow(rho, p.gamma) - 1)


def mdbc_density(walls, st, nb: Neighbors, p: Params, dtype):
    """computeBoundaryDensitymDBC, src/modules/solidBoundary.py:561-617."""
    P = nb.gf
    bb, bf = P.i, P.j
    h = p.h
    k = W(P.q, h)
    g = gradW(P.q, P.e, h)
    mass = st["area"][bf] * p.rho0
    V = st["volume"]
    nom = ssum(mass * k, bb, walls.n)
    den = ssum(V[bf] * k, bb, walls.n)
    shep = nom / den
    gsum = ssum(mass[:, None] * g, bb, walls.n)
    b = torch.cat([nom[:, None], gsum], 1)
    vsum = ssum(V[bf] * k, bb, walls.n)
    vgs = ssum(V[bf][:, None] * g, bb, walls.n)
    xg = walls.xg.to(dtype)
    xij = st["x"][bf] - xg[bb]
    psum = ssum((V[bf] * k)[:, None] * xij, bb, walls.n)
    pm = ssum(V[bf][:, None, None] * torch.einsum("nu,nv->nuv", xij, g), bb, walls.n)
    A = torch.zeros((walls.n, 3, 3), dtype=dtype)
    A[:, 0, 0] = vsum
    A[:, 1, 0] = vgs[:, 0]
    A[:, 2, 0] = vgs[:, 1]
    A[:, 0, 1] = psum[:, 0]
    A[:, 0, 2] = psum[:, 1]
    A[:, 1, 1] = pm[:, 0, 0]
    A[:, 1, 2] = pm[:, 0, 1]
    A[:, 2, 1] = pm[:, 1, 0]
    A[:, 2, 2] = pm[:, 1, 1]
    res = torch.matmul(torch.linalg.pinv(A), b.unsqueeze(2))[:, :, 0]
    cnt = torch.bincount(bb, minlength=walls.n)
    rho_b = torch.ones(walls.n, dtype=dtype)
    rho_b = torch.where(cnt > 0, shep / p.rho0, rho_b)
    lin = (res[:, 0] + torch.einsum("nu,nu->n", walls.x.to(dtype) - xg, res[:, 1:])) / p.rho0
    rho_b = torch.where(cnt > 10, lin, rho_b)
    return torch.clamp(rho_b, min=1)


def mls_pressure(xq, st, P: Pairs, pf, p: Params, nb: int):
    """precomputeMLS (src/util.py:332-384) and the wall pressure sum of solidBoundary.py:787-790:
    M_b = sum_j 2 b_j b_j^T V_j W_j with b_j = (1, x_j - x_q), V_j = A_j / (rho~_j rho0);
    p_b = sum_j (pinv(M_b) e1 . b_j) W_j V_j p_j."""
    i, j = P.i, P.j
    x, A, rt = st["x"], st["area"], st["rho"]
    k = W(P.q, p.h)
    bij = torch.cat([torch.ones((i.shape[0], 1), dtype=x.dtype), x[j] - xq[i]], 1)
    V = (A / (rt * p.rho0))[j]
    M = ssum(2 * torch.einsum("nu,nv->nuv", bij, bij) * (V * k)[:, None, None], i, nb)
    Me1 = torch.linalg.pinv(M)[:, :, 0]
    pg = torch.einsum("nd,nd->n", Me1[i], bij) * k * V
    return ssum(pg * pf[j], i, nb)


def mls_boundary_pressure(xb, st, P: Pairs, pf, p: Params, nb: int):
    """prepareMLSBoundaries + evalMLSBoundaries (src/util.py:283-330), clamped at 0
    (solidBoundary.py:802-803), with fluidVolume as the fluid's area."""
    i, j = P.i, P.j
    x, V = st["x"], st["volume"]
    k = W(P.q, p.h) * V[j]
    nom = ssum(k[:, None] * x[j], i, nb)
    den = ssum(k, i, nb)
    d = xb.clone()
    m = den > 1e-9
    d[m] = nom[m] / den[m, None]
    xbar = x[j] - d[i]
    M1 = torch.linalg.pinv(ssum(torch.einsum("nu,nv->nuv", xbar, xbar) * k[:, None, None], i, nb))
    vec = xbar * k[:, None]
    bbar = torch.cat([torch.ones((nb, 1), dtype=x.dtype), xb - d], 1)
    vsum = ssum(vec * pf[j, None], i, nb)
    alpha = ssum(pf[j] * k, i, nb)
    s = ssum(k, i, nb)
    ms = s > 1e-6
    alpha[ms] = alpha[ms] / s[ms]
    c = torch.cat([alpha[:, None], torch.matmul(M1, vsum.unsqueeze(2))[:, :, 0]], 1)
    return torch.clamp(torch.einsum("nu,nu->n", bbar, c), min=0)


def wall_pressure(walls, st, nb: Neighbors, rho_b, p: Params, dtype):
    """solidBoundaryModule.computePressure (solidBoundary.py:772-808): PBSPH = Tait of the mDBC
    density; ghostMLS / deltaMLS = MLS interpolation of the fluid pressure at the ghost / wall
    positions; MLSPressure = the Shepard-centred linear MLS fit."""
    scheme = p.boundary_pressure
    if scheme == "PBSPH":
        return tait(rho_b, p)
    pf = tait(st["rho"], p)
    if scheme in ("ghostMLS", "deltaMLS"):
        xq = (walls.xg if scheme == "ghostMLS" else walls.x).to(dtype)
        return mls_pressure(xq, st, nb.gf, pf, p, walls.n)
    if scheme == "MLSPressure":
        return mls_boundary_pressure(walls.x.to(dtype), st, nb.gf, pf, p, walls.n)
    raise ValueError(scheme)


def deltasph_rhs(st, walls, nb: Neighbors, p: Params, dtype):
    """deltaSPHSimulation.timestep, src/deltaSPH.py:146-200, solid walls, continuum density.
    Returns (acceleration, velocity, dpdt, extras)."""
    h = p.h
    n = st["x"].shape[0]
    x, u, rt, A = st["x"], st["v"], st["rho"], st["area"]
    rho = rt * p.rho0
    st["volume"] = V = A / rt                                              # density.py:34
    F = nb.ff
    i, j = F.i, F.j
    g = gradW(F.q, F.e, h)
    extras = {}
    # walls: mDBC density, wall volume / pressure
    have_walls = walls is not None and walls.n > 0 and nb.bf is not None
    if have_walls:
        rho_b = mdbc_density(walls, st, nb, p, dtype)
        Vb = walls.area.to(dtype) / rho_b
        pb = wall_pressure(walls, st, nb, rho_b, p, dtype)                 # solidBoundary.py:772-808
        B = nb.bf
        bb, bf = B.i, B.j
        gb = gradW(B.q, -B.e, h)                                            # fluid side: e = (x_f - x_b)/r
        extras["rho_b"] = rho_b
        extras["p_b"] = pb
    acc = torch.zeros((n, 2), dtype=dtype)
    # 7 gravity (gravity.py:46-57)
    if p.point_source:
        xc = x - torch.tensor(p.point_center, dtype=dtype)
        dist = torch.linalg.norm(xc, axis=1)
        m = dist > 1e-7
        # the reference normalises in place where dist > 1e-7; torch.where keeps it
        # differentiable (same values)
        diff = torch.where(m[:, None], xc / torch.where(m, dist, torch.ones_like(dist))[:, None], xc)
        acc = acc - p.point_magnitude * diff * dist[:, None]
    else:
        acc = acc + torch.tensor(p.gravity, dtype=dtype)
    # 8 continuity (momentum.py:13-19, solidBoundary.py:746-770)
    dpdt = -ssum(torch.einsum("nu,nu->n", u[j] - u[i], g) * V[j] * rho[j], i, n)
    if have_walls:
        ub = torch.zeros((walls.n, 2), dtype=dtype)
        dpdt = dpdt - ssum(torch.einsum("nu,nu->n", ub[bb] - u[bf], gb) * Vb[bb] * (rho_b * p.rho0)[bb], bf, n)
    # 9 density diffusion (densityDiffusion.py:12-82)
    rji = x[j] - x[i]
    rji2 = torch.linalg.norm(rji, dim=1) ** 2 + p.eps
    if p.diffusion == "MOG":
        psi = (2 * (rho[j] - rho[i]) / rji2)[:, None] * rji
        dpdt = dpdt + h * p.delta * p.c0 * ssum(torch.einsum("nu,nu->n", psi, g) * V[j], i, n)
    elif p.diffusion == "deltaSPH":
        L = ssum(V[j][:, None, None] * torch.einsum("nu,nv->nuv", x[j] - x[i], g), i, n)
        if have_walls:
            L = L + ssum(Vb[bb][:, None, None] * torch.einsum("nu,nv->nuv", walls.x.to(dtype)[bb] - x[bf], gb), bf, n)
        Linv = pinv2x2(L)
        grad = torch.matmul(Linv[i], g.unsqueeze(2))[:, :, 0]
        gr = -ssum((2 * (rho[j] - rho[i]) * V[j])[:, None] * grad, i, n)
        if have_walls:
            gradb = torch.matmul(Linv[bf], gb.unsqueeze(2))[:, :, 0]
            gr = gr - ssum((2 * (rho_b[bb] * p.rho0 - rho[bf]) * Vb[bb])[:, None] * gradb, bf, n)
        psi = (2 * (rho[j] - rho[i]) / rji2)[:, None] * rji - (gr[i] + gr[j])
        dpdt = dpdt + h * p.delta * p.c0 * ssum(torch.einsum("nu,nu->n", psi, g) * V[j], i, n)
        extras["L"], extras["grad_rho"] = L, gr
    # 10 pressure (pressure.py:80-116)
    pr = tait(rt, p)
    acc = acc + (-1 / rho[:, None]) * ssum(((pr[i] + pr[j]) * V[j])[:, None] * g, i, n)
    if have_walls:
        acc = acc + (-1 / rho[:, None]) * ssum(((pr[bf] + pb[bb]) * Vb[bb])[:, None] * gb, bf, n)
    # 11 artificial viscosity (diffusion.py:12-25, solidBoundary.py:820-844)
    pij = torch.einsum("nu,nu->n", u[j] - u[i], rji)
    pij = torch.clamp(pij, max=0) / rji2
    acc = acc + h * p.alpha * p.c0 * ssum((pij * V[j] * rho[j] / (rho[i] + rho[j]))[:, None] * g, i, n)
    if have_walls and p.boundary_diffusion:
        rjb = walls.x.to(dtype)[bb] - x[bf]
        rjb2 = torch.linalg.norm(rjb, dim=1) ** 2 + p.eps
        pib = torch.clamp(torch.einsum("nu,nu->n", ub[bb] - u[bf], rjb), max=0) / rjb2
        rb = rho_b[bb] * p.rho0
        acc = acc + h * p.alpha * p.c0 * ssum((pib * Vb[bb] * rb / (rho[bf] + rb))[:, None] * gb, bf, n)
    # 12 laminar viscosity (laminar.py:12-27; index choices as in the reference)
    rij = x[j] - x[i]
    rij2 = torch.linalg.norm(rij, dim=1) ** 2 + p.eps
    mui = rho[i] * p.kinematic
    muj = rho[i] * p.kinematic
    mj = rho[j] * V[j]
    term = 4 * mj * (mui + muj) * torch.einsum("nu,nu->n", rij, g) / ((rho[i] + rho[j]) ** 2 * rij2)
    acc = acc - ssum(term[:, None] * (u[i] - u[j]), i, n)
    extras["pressure"] = pr
    return acc, u, dpdt, extras


# ----------------------------------------------------------------- DFSPH (src/modules/dfsph.py)
def dfsph_rhs(st, walls, nb: Neighbors, p: Params, dt, dtype):
    """dfsphSimulation.timestep, src/dfsph.py:134-202, summation density, solid walls (PBSPH)."""
    h = p.h
    n = st["x"].shape[0]
    x, u, A = st["x"], st["v"], st["area"]
    F = nb.ff
    i, j = F.i, F.j
    rho0 = p.rho0
    rho0v = torch.full((n,), rho0, dtype=dtype)
    # 4 density (density.py:26-34); V uses the fluid-only density
    rt = ssum(W(F.q, h) * A[j], i, n)
    st["volume"] = V = A / rt
    have_walls = walls is not None and walls.n > 0 and nb.bf is not None
    extras = {}
    if have_walls:                                                          # solidBoundary.py:522-549
        B = nb.bf
        bb, bf = B.i, B.j
        kb = W(B.q, h)
        Ab = walls.area.to(dtype)
        rt = rt + ssum(kb * Ab[bb], bf, n)
        rho_b = torch.clamp(walls.density_term.to(dtype) + ssum(kb * A[bf], bb, walls.n), max=1)
        extras["rho_b"] = rho_b
    st["rho"] = rt
    # 6-7 acceleration: gravity
    acc = torch.zeros((n, 2), dtype=dtype) + torch.tensor(p.gravity, dtype=dtype)
    gS = spiky(F.q, F.e, h)

    def solve(density, acc_in):
        vstar = u + dt * acc_in
        Aact = A / rt
        # alpha (dfsph.py:58-83, solidBoundary.py:443-479)
        k1 = ssum(Aact[j][:, None] * gS, i, n)
        k2 = ssum((Aact ** 2 / (A * rho0v))[j] * torch.einsum("nd,nd->n", gS, gS), i, n)
        wb = density and have_walls
        if wb:
            gSb = spiky(B.q, B.e, h)                                        # e = (x_b - x_f)/r
            g2b = torch.einsum("nd,nd->n", gSb, gSb)
            Aact_b = Ab / rho_b
            k1 = k1 + ssum(Aact_b[bb][:, None] * gSb, bf, n)
            k2 = k2 + ssum((Aact_b ** 2 / (Ab * rho0))[bb] * g2b, bf, n)
            alpha_b = torch.clamp(-dt ** 2 * Aact_b * ssum((Aact ** 2 / (A * rho0v))[bf] * g2b, bb, walls.n),
                                  max=-0.01 ** 2 * h ** 2)
        fac = -dt ** 2 * Aact
        alpha = fac / (A * rho0v) * torch.einsum("nd,nd->n", k1, k1) + fac * k2
        alpha = torch.clamp(alpha, -1, -1e-7)
        # source (dfsph.py:85-100, solidBoundary.py:481-520)
        src = ssum(-dt * Aact[j] * torch.einsum("nd,nd->n", vstar[i] - vstar[j], gS), i, n)
        if wb:
            vb = torch.zeros((walls.n, 2), dtype=dtype)
            prod = torch.einsum("nd,nd->n", vb[bb] - vstar[bf], gSb)
            src = src - dt * ssum(Aact_b[bb] * prod, bf, n)
            src_b = 1.0 - rho_b + (-dt) * ssum(Aact[bf] * prod, bb, walls.n)
        source = 1.0 - rt + src if density else src
        p2 = torch.zeros(n, dtype=dtype)
        pw = torch.zeros(walls.n, dtype=dtype) if wb else None

        def accel(pf):
            pp = pf / (rt * rho0v) ** 2
            a = ssum((-(A * rho0v)[j] * (pp[i] + pp[j]))[:, None] * gS, i, n)
            if wb:                                                          # solidBoundary.py:310-403 (PBSPH)
                pbn = pw[bb] / ((rho_b[bb] * rho0) ** 2)
                a = a + ssum((-(Ab * rho0)[bb] * (pp[bf] + pbn))[:, None] * (-gSb), bf, n)
            return a

        errors = []
        it = 0
        err = 0.0
        thr = p.density_threshold if density else p.divergence_threshold
        mn = p.min_density_iters if density else p.min_divergence_iters
        mx = p.max_density_iters if density else p.max_divergence_iters
        res = None
        while (it < mn or err > thr) and it <= mx:                         # dfsph.py:205-231
            pa = accel(p2)
            pcur = p2
            ks = ssum(torch.einsum("nd,nd->n", (dt ** 2 * Aact[j])[:, None] * (pa[i] - pa[j]), gS), i, n)
            if wb:                                                          # solidBoundary.py:405-431
                bks = ssum(torch.einsum("nd,nd->n", (dt ** 2 * Aact[bf])[:, None] * pa[bf], -gSb), bb, walls.n)
                rb = bks - src_b
                pw = torch.clamp(pw - p.omega_boundary * rb / alpha_b, min=0.0)
                ks = ks + ssum(torch.einsum("nd,nd->n", (dt ** 2 * Aact_b[bb])[:, None] * pa[bf], -gSb), bf, n)
            res = ks - source
            p2 = pcur - 0.3 * res / alpha
            if density:
                p2 = torch.clamp(p2, min=0.0)
            if wb:
                err = float((torch.sum(torch.clamp(res, min=-thr)) + torch.sum(torch.clamp(rb, min=-thr)))
                            / (walls.n + n))
            else:
                err = float(torch.mean(torch.clamp(res, min=-thr)))
            errors.append(err)
            it += 1
        pa = accel(p2)
        return pa, errors, {"alpha": alpha, "source": source, "pressure": p2}

    if p.divergence_solver:
        pa, derr, _ = solve(False, acc)
        acc = acc + pa
        extras["divergence_errors"] = derr
    pa, err, info = solve(True, acc)
    acc = acc + pa
    extras["density_errors"] = err
    extras.update(info)
    # 11 velocity diffusion + 12 laminar with V = A / (fluid-only density), rho = density*rho0
    rho = rt * rho0
    g = gradW(F.q, F.e, h)
    rji = x[j] - x[i]
    rji2 = torch.linalg.norm(rji, dim=1) ** 2 + p.eps
    pij = torch.clamp(torch.einsum("nu,nu->n", u[j] - u[i], rji), max=0) / rji2
    acc = acc + h * p.alpha * p.c0 * ssum((pij * V[j] * rho[j] / (rho[i] + rho[j]))[:, None] * g, i, n)
    if have_walls and p.boundary_diffusion:
        gb = gradW(B.q, -B.e, h)
        Vb = Ab / rho_b
        rjb = walls.x.to(dtype)[bb] - x[bf]
        rjb2 = torch.linalg.norm(rjb, dim=1) ** 2 + p.eps
        pib = torch.clamp(torch.einsum("nu,nu->n", -u[bf], rjb), max=0) / rjb2
        rb = rho_b[bb] * rho0
        acc = acc + h * p.alpha * p.c0 * ssum((pib * Vb[bb] * rb / (rho[bf] + rb))[:, None] * gb, bf, n)
    mui = rho[i] * p.kinematic
    mj = rho[j] * V[j]
    term = 4 * mj * (2 * mui) * torch.einsum("nu,nu->n", rji, g) / ((rho[i] + rho[j]) ** 2 * rji2)
    acc = acc - ssum(term[:, None] * (u[i] - u[j]), i, n)
    return acc, u, None, extras


# ----------------------------------------------------------------- integration (simulationBase.py:564-705)
def step(state, walls, p: Params, dt, scheme="semiImplicitEuler", solver="deltaSPH", dtype=torch.float64):
    """One integrate() of the reference; returns (new_state, info of the last RHS evaluation)."""
    x0 = state["x"].to(dtype)
    v0 = state["v"].to(dtype)
    r0 = state["rho"].to(dtype)
    A = state["area"].to(dtype)

    def rhs(x, v, r):
        nb = search(x.to(torch.float32), walls, p.h, p.vmin, p.vmax, dtype,
                    ghost_from_walls=p.boundary_pressure in ("deltaMLS", "MLSPressure"))
        st = {"x": x, "v": v, "rho": r, "area": A}
        if solver == "dfsph":
            a, vel, dp, ex = dfsph_rhs(st, walls, nb, p, dt, dtype)
            ex["rho"] = st["rho"]
        else:
            a, vel, dp, ex = deltasph_rhs(st, walls, nb, p, dtype)
        return a, vel, dp, ex

    cont = solver != "dfsph"
    if scheme == "semiImplicitEuler":
        a, vel, dp, ex = rhs(x0, v0, r0)
        v1 = v0 + dt * a
        x1 = x0 + dt * (vel + dt * a)
        r1 = r0 + dt * dp / p.rho0 if cont else ex["rho"]
        return {"x": x1, "v": v1, "rho": r1, "area": A, "acc": a, "dpdt": dp}, ex
    if scheme == "RK4":
        a1, u1, d1, _ = rhs(x0, v0, r0)
        a2, u2, d2, _ = rhs(x0 + 0.5 * dt * u1, v0 + 0.5 * dt * a1, r0 + 0.5 * dt * d1 / p.rho0)
        a3, u3, d3, _ = rhs(x0 + 0.5 * dt * u2, v0 + 0.5 * dt * a2, r0 + 0.5 * dt * d2 / p.rho0)
        a4, u4, d4, ex = rhs(x0 + dt * u3, v0 + dt * a3, r0 + dt * d3 / p.rho0)
        sa = a1 + 2 * a2 + 2 * a3 + a4
        su = u1 + 2 * u2 + 2 * u3 + u4
        sd = d1 + 2 * d2 + 2 * d3 + d4
        return {"x": x0 + dt / 6 * su, "v": v0 + dt / 6 * sa, "rho": r0 + dt / 6 * sd / p.rho0, "area": A,
                "acc": sa, "dpdt": d4}, ex
    raise ValueError(scheme)


def update_dt(state, p: Params, dt, dt_min, dt_max, cfl=0.4, scheme="dfsph"):
    """adaptiveTimeSteppingModule.updateTimestep, src/modules/adaptiveDT.py:59-95 (fixed = false).
    The viscosity / acceleration / acoustic switches are the configured minimum dt (:50-52)."""
    h = p.h
    visc = 0.125 * h ** 2 / p.kinematic
    acc = float(0.25 * torch.min(torch.sqrt(h / torch.linalg.norm(state["acc"], axis=-1))))
    if scheme in ("deltaSPH", "deltaPlus"):
        vdt = cfl * h / p.c0
    else:
        vdt = float(0.4 * h / torch.max(torch.linalg.norm(state["v"], axis=-1)))
    m = dt_max
    if dt_min:
        m = min(m, visc)
        m = min(m, acc)
        if not math.isnan(vdt):
            m = min(m, vdt)
    target = m if m > dt_min else dt_min
    return min(max(target, dt * 0.5), dt * 1.05)


# ----------------------------------------------------------------- delta+ (src/modules/deltaPlus.py)
def eigvals2x2(M):
    """The eigVals pinv2x2 returns (src/util.py:408-431): singular values (o1, o2), swapped
    where |o2| > |o1|."""
    a, b, c, d = M[:, 0, 0], M[:, 0, 1], M[:, 1, 0], M[:, 1, 1]
    S1 = a ** 2 + b ** 2 + c ** 2 + d ** 2
    S2 = torch.sqrt((a ** 2 + b ** 2 - c ** 2 - d ** 2) ** 2 + 4 * (a * c + b * d) ** 2)
    e = torch.stack([torch.sqrt((S1 + S2) / 2), torch.sqrt((S1 - S2) / 2)], 1)
    swap = torch.abs(e[:, 1]) > torch.abs(e[:, 0])
    e[swap] = torch.flip(e[swap], [1])
    return e


def _scatter_fill0(vals, idx, n, reduce):
    """torch_scatter max / min: the reduction over each index, 0 where an index has none."""
    out = torch.zeros(n, dtype=vals.dtype)
    return out.scatter_reduce(0, idx, vals, reduce=reduce, include_self=False)


def surface_detect(fl, wl, ww, h, dtype):
    """detectSurface (deltaPlus.py:242-245): the normalization matrix (fluid pairs plus the
    wall part, densityDiffusion.py:30-44, solidBoundary.py:676-694) with pinv2x2, the walls'
    own matrices, the lambda gradient and normal (:132-163) and the surface mask (:165-205).
    fl: fluid state and pairs {x, rho, area, volume, i, j, e, q}; wl: wall pairs and arrays
    {bb, bf, e (x_b - x_f)/r, q, x, area, rho}; ww: wall-wall pairs {i, j, e (x_j - x_i)/r, q}
    in the reference's sign.  Returns a dict with the reference's state names."""
    T = lambda a: a.to(dtype)
    x, rho, area, vol = T(fl["x"]), T(fl["rho"]), T(fl["area"]), T(fl["volume"])
    i, j, e, q = fl["i"], fl["j"], T(fl["e"]), T(fl["q"])
    n = x.shape[0]
    bb, bf, be, bq = wl["bb"], wl["bf"], T(wl["e"]), T(wl["q"])
    xb, Ab, rhob = T(wl["x"]), T(wl["area"]), T(wl["rho"])
    nb = xb.shape[0]
    rho0 = wl.get("rho0", 1000.0)
    Vb = Ab * rho0 / rhob / rho0              # self.fluidVolume of solidBoundary.py:678

    def norm_matrix(ii, jj, ri, rj, Vj, dist, qq, num):   # computeNormalizationMatrix
        g = gradW(qq, dist, h)
        term = torch.einsum('nu,nv->nuv', rj[jj] - ri[ii], g) * Vj[jj][:, None, None]
        return ssum(term, ii, num)

    M = norm_matrix(i, j, x, x, vol, e, q, n)
    # walls' own matrices: wall -> fluid pairs, then the wall-wall pairs (solidBoundary.py:679-692)
    Mb = norm_matrix(bb, bf, xb, x, vol, be, bq, nb)
    Mb = Mb + norm_matrix(ww["i"], ww["j"], xb, xb, Vb, T(ww["e"]), T(ww["q"]), nb)
    eig_b = eigvals2x2(Mb)
    # fluid side of the wall part: fluid i = bf, j = bb, distances -e
    M = M + norm_matrix(bf, bb, x, xb, Vb, -be, bq, n)
    L = pinv2x2(M)
    eig = eigvals2x2(M)
    lam = eig[:, 1]
    # lambda gradient and normal (deltaPlus.py:132-163)
    g = gradW(q, e, h)
    corr = torch.bmm(L[i], g[:, :, None])[:, :, 0]
    term = -((area[j] / rho[j]) * (lam[j] - lam[i]))[:, None] * corr
    lg = ssum(term, i, n)
    gb = gradW(bq, -be, h)
    corr = torch.bmm(L[bf], gb[:, :, None])[:, :, 0]
    term = -((area[bb] / rho[bb]) * (eig_b[:, 1][bb] - lam[bf]))[:, None] * corr   # the reference's fluidArea[bb]
    lg = lg + ssum(term, bf, n)
    eps = h ** 2 * 0.1
    normal = lg / (torch.linalg.norm(lg, dim=1) + eps)[:, None]
    # surface mask (deltaPlus.py:165-205)
    m = i != j
    ii, jj = i[m], j[m]
    dots = torch.einsum('nd,nd->n', -e[m], normal[ii])
    sc = _scatter_fill0(dots, ii, n, "amax")
    angle_min = torch.arccos(_scatter_fill0(dots, ii, n, "amin"))
    angle_max = torch.arccos(sc)
    dots = torch.einsum('nd,nd->n', be, normal[bf])
    sc = torch.arccos(torch.max(sc, _scatter_fill0(dots, bf, n, "amax")))
    mask = torch.zeros_like(sc)
    mask[torch.logical_and(sc > math.pi / 6, lam < 0.6)] = 1
    mask2 = _scatter_fill0(mask[jj], ii, n, "amax")
    final = torch.zeros_like(sc)
    final[mask2 > 0] = 2 / 3
    final[mask > 0] = 1
    zero, surf, bulk = final > 0.7, torch.logical_and(lam >= 0.5, final > 0.), final < 0.1
    surface = final.clone()
    surface[surf] = 1
    surface[zero] = 0
    surface[bulk] = 2
    return {"normalizationMatrix": M, "fluidL": L, "eigVals": eig, "fluidLambda": lam, "lambdaGrad": lg,
            "fluidNormal": normal, "angleMin": angle_min, "angleMax": angle_max, "fluidSurfaceMask": surface,
            "boundaryNormalizationMatrix": Mb, "boundaryEigVals": eig_b}


def shift(fl, wl, normal, surface, h, c0, packing, dtype, cfl=1.5):
    """shift (deltaPlus.py:247-251): computeShiftAmount (:81-115) and adjustShiftingAmount
    (:207-240).  Returns (shiftAmount before the adjustment, fluidUpdate, fluidSurfaceMask)."""
    T = lambda a: a.to(dtype)
    v, rho, area = T(fl["v"]), T(fl["rho"]), T(fl["area"])
    i, j, e, q = fl["i"], fl["j"], T(fl["e"]), T(fl["q"])
    n = v.shape[0]
    bb, bf, be, bq = wl["bb"], wl["bf"], T(wl["e"]), T(wl["q"])
    Ab, rhob = T(wl["area"]), T(wl["rho"])
    Ma = torch.max(torch.linalg.norm(v, dim=1)) / c0
    k0 = W(torch.tensor(packing, dtype=dtype), h)
    R, npow = 0.2, 4
    coef = -cfl * Ma * (4 * h ** 2)
    kt = 1 + R * torch.pow(W(q, h) / k0, npow)
    term = (kt * area[j] / (rho[i] + rho[j]))[:, None] * gradW(q, e, h)
    s = coef * ssum(term, i, n)
    kt = 1 + R * torch.pow(W(bq, h) / k0, npow)
    term = (kt * Ab[bb] / (rho[bf] + rhob[bb]))[:, None] * gradW(bq, -be, h)
    s = s + coef * ssum(term, bf, n)
    raw = s.clone()
    ln = torch.linalg.norm(s, axis=1)
    big = ln > h * 0.05
    s[big] = s[big] / ln[big, None] * h * 0.05
    nrm, surf = T(normal), T(surface)
    outer = torch.einsum('nu,nv->nuv', nrm, nrm)
    eye = torch.eye(2, dtype=dtype)
    ns = torch.matmul(eye - outer, s.unsqueeze(2))[:, :, 0]
    zero, sr, bulk = surf < 0.5, surf < 1.5, surf > 1.5
    s[sr] = ns[sr]
    s[zero] = 0
    mask = surf.clone()
    mask[sr] = 1
    mask[zero] = 0
    mask[bulk] = 2
    return raw, s, mask
