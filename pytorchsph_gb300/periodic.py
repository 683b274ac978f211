"""Periodic boundaries (src/modules/periodicBC.py) on the GPU.

* `createGhostParticlesKernel` — the reference's function (periodicBC.py:23-103), same
  arguments and return value (lists of index tensors and offset tensors per category), built
  on `sph_periodic_ghosts`.
* `periodicBCModule` — the reference's module with its interface (initialize, resetState,
  filterVirtualParticles, createGhostParticles, enforcePeriodicBC, syncToGhost): ghost copies
  appended to every per-particle array of the state, as the reference does, so the other
  modules run over real + ghost particles unchanged.  Its condition `periodicX or periodicX`
  (:272, :316) is kept: a box periodic only along y makes no copies, as in the reference.
* `periodic_neighbors` — the same pair set without copies: the periodic cell grid of
  `sph_nl_periodic_*` wraps neighbor cells and tests image positions, returning (rows, cols,
  codes) over the real particles with the image shift of each pair.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from .modules import Module, Parameter

CATEGORIES = ("xp", "xn", "yp", "yn", "xp_yp", "xp_yn", "xn_yp", "xn_yn")


def _host2(v):
    a = (ctypes.c_float * 2)(float(v[0]), float(v[1]))
    return ctypes.cast(a, ctypes.c_void_p), a


def _f2(t):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.dim() == 2 and
            t.shape[1] == 2):
        raise RuntimeError("positions must be a float32 CUDA tensor of shape [N, 2]")
    return t.contiguous()


def createGhostParticlesKernel(positions, domainMin, domainMax, buffer, support, periodicX, periodicY):
    """periodicBC.py:23-103: (filters, offsets), one index tensor (int64) and one offset
    tensor ([k, 2]) per enabled category in the reference's order."""
    pos = _f2(positions)
    n = pos.shape[0]
    dev = pos.device
    lib = N.load()
    dmin, _a = _host2(domainMin)
    dmax, _b = _host2(domainMax)
    cap = 3 * n + 8
    idx = torch.empty(cap, dtype=torch.int64, device=dev)
    off = torch.empty((cap, 2), dtype=torch.float32, device=dev)
    counts = torch.empty(8, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    sc = torch.empty((lib.sph_periodic_ghosts_scratch_bytes(n) + 7) // 8, dtype=torch.int64, device=dev)
    N.call("sph_periodic_ghosts", N.ptr(pos), n, dmin, dmax, float(buffer) * float(support), int(bool(periodicX)),
           int(bool(periodicY)), cap, N.ptr(idx), N.ptr(off), N.ptr(counts), N.ptr(status), N.ptr(sc), sc.numel() * 8,
           N.stream_ptr())
    c = counts.cpu().tolist()
    if int(status.item()):
        raise RuntimeError("createGhostParticlesKernel: more ghost copies than 3 per particle")
    enabled = []
    if periodicX:
        enabled += [0, 1]
    if periodicY:
        enabled += [2, 3]
    if periodicX and periodicY:
        enabled += [4, 5, 6, 7]
    filters, offsets = [], []
    base = 0
    for k in range(8):
        if k in enabled:
            filters.append(idx[base:base + c[k]])
            offsets.append(off[base:base + c[k]])
        base += c[k]
    return filters, offsets


def periodic_neighbors(positions, supports, domainMin, domainMax, periodicX=True, periodicY=False,
                       cell_size=None):
    """Pairs of the real particles in the periodic box without ghost copies: (rows, cols) int64
    in (i, j) order and codes int8 = (sx + 1) | (sy + 1) << 2, s the image shift of column j
    (x_j + sx L_x, y_j + sy L_y).  cell_size defaults to the largest support."""
    pos = _f2(positions)
    sup = supports.contiguous()
    n = pos.shape[0]
    dev = pos.device
    lib = N.load()
    dmin, _a = _host2(domainMin)
    dmax, _b = _host2(domainMax)
    cs = float(cell_size) if cell_size is not None else float(sup.max().item())
    st = N.stream_ptr()
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    sc = torch.empty((lib.sph_nl_periodic_scratch_bytes(n, dmin, dmax, cs) + 7) // 8, dtype=torch.int64, device=dev)
    offsets = torch.empty(n + 1, dtype=torch.int64, device=dev)
    args = (N.ptr(pos), N.ptr(sup), n, dmin, dmax, cs, int(bool(periodicX)), int(bool(periodicY)))
    N.call("sph_nl_periodic_count", *args, N.ptr(offsets), N.ptr(status), N.ptr(sc), sc.numel() * 8, st)
    P = int(offsets[n].item())
    rows = torch.empty(P, dtype=torch.int64, device=dev)
    cols = torch.empty(P, dtype=torch.int64, device=dev)
    codes = torch.empty(P, dtype=torch.int8, device=dev)
    N.call("sph_nl_periodic_fill", *args, N.ptr(offsets), P, N.ptr(rows), N.ptr(cols), N.ptr(codes), N.ptr(status),
           N.ptr(sc), sc.numel() * 8, st)
    f = int(status.item())
    if f:
        raise N.SPHError(f"periodic search: {N.decode_flags(f)}")
    return rows, cols, codes


class periodicBCModule(Module):
    """src/modules/periodicBC.py:106-327 with GPU ghost creation."""

    def __init__(self):
        super().__init__('densityInterpolation', 'Evaluates density at the current timestep')

    def getParameters(self):
        return [
            Parameter('periodicBC', 'periodicX', 'bool', False, required=False, export=True, hint=''),
            Parameter('periodicBC', 'periodicY', 'bool', False, required=False, export=True, hint=''),
            Parameter('periodicBC', 'buffer', 'float', 2, required=False, export=True, hint=''),
        ]

    def initialize(self, simulationConfig, simulationState):
        self.support = simulationConfig['particle']['support']
        self.periodicX = simulationConfig['periodicBC']['periodicX']
        self.periodicY = simulationConfig['periodicBC']['periodicY']
        self.buffer = simulationConfig['periodicBC']['buffer']
        self.domainMin = simulationConfig['domain']['min']
        self.domainMax = simulationConfig['domain']['max']
        self.virtualMin = simulationConfig['domain']['virtualMin']
        self.virtualMax = simulationConfig['domain']['virtualMax']
        self.dtype = simulationConfig['compute']['precision']

    def _prune(self, simulationState):
        realParticles = self.filterVirtualParticles(simulationState['fluidPosition'], simulationState)
        for arr in list(simulationState):
            t = simulationState[arr]
            if torch.is_tensor(t) and t.dim() > 0 and t.shape[0] == simulationState['numParticles']:
                simulationState[arr] = t[realParticles]
        simulationState['numParticles'] = simulationState['fluidPosition'].shape[0]
        simulationState['realParticles'] = simulationState['fluidPosition'].shape[0]

    def resetState(self, simulationState):
        if 'realParticles' not in simulationState:
            simulationState['realParticles'] = simulationState['numParticles']
        self._prune(simulationState)
        simulationState.pop('ghostIndices', None)
        simulationState.pop('ghosts', None)
        simulationState['numParticles'] = simulationState['realParticles']

    def filterVirtualParticles(self, positions, state):
        """periodicBC.py:146-180: the rows to keep, one per UID, sorted by UID: rows inside the
        domain along the periodic directions; a UID left with no such row (or with several)
        keeps its row closest to the domain, clamped into it."""
        n = state['numParticles']
        real = state['realParticles']
        uid = state['UID']
        dev = positions.device
        keep = torch.ones(n, dtype=torch.bool, device=dev)
        if self.periodicX:
            keep &= (positions[:, 0] >= self.domainMin[0]) & (positions[:, 0] < self.domainMax[0])
        if self.periodicY:
            keep &= (positions[:, 1] >= self.domainMin[1]) & (positions[:, 1] < self.domainMax[1])
        kept = torch.zeros(real, dtype=torch.int64, device=dev).index_add_(0, uid, keep.to(torch.int64))
        bad = torch.nonzero(kept != 1).flatten()
        if bad.numel():               # rare: resolved on the host, as the reference loops over them
            rows = torch.arange(n, device=dev)
            for u in bad.tolist():
                cand = rows[uid == u]
                p = positions[cand]
                clip = p.clone()
                clip[:, 0] = torch.clamp(clip[:, 0], min=self.domainMin[0], max=self.domainMax[0])
                clip[:, 1] = torch.clamp(clip[:, 1], min=self.domainMin[1], max=self.domainMax[1])
                best = int(torch.argmin(torch.linalg.norm(clip - p, axis=1)))
                keep[cand] = False
                keep[cand[best]] = True
                positions[cand[best]] = clip[best]
        idx = torch.nonzero(keep).flatten()
        return idx[torch.argsort(uid[idx], stable=True)]

    def createGhostParticles(self, positions):
        return createGhostParticlesKernel(positions, self.domainMin, self.domainMax, self.buffer, self.support,
                                          self.periodicX, self.periodicY)

    def enforcePeriodicBC(self, simulationState, simulation):
        st = simulationState
        if self.periodicX or self.periodicX:   # the reference's own condition (periodicBC.py:272)
            if 'realParticles' not in st:
                st['realParticles'] = st['numParticles']
            self._prune(st)
            filters, offsets = self.createGhostParticles(st['fluidPosition'])
            ghostIndices = torch.cat(filters)
            ghostOffsets = torch.vstack(offsets)
            realParticles = self.filterVirtualParticles(st['fluidPosition'], st)
            for arr in list(st):
                t = st[arr]
                if torch.is_tensor(t) and t.dim() > 0 and t.shape[0] == st['numParticles']:
                    if arr == 'fluidPosition':
                        st[arr] = torch.cat((t, t[ghostIndices] + ghostOffsets))
                    else:
                        st[arr] = torch.cat((t, t[ghostIndices]))
            del realParticles
            st['numParticles'] = st['fluidPosition'].shape[0]
            ones = torch.full((st['realParticles'],), -1, dtype=torch.int64, device=ghostIndices.device)
            st['ghostIndices'] = torch.cat((ones, ghostIndices))
            st['ghosts'] = ghostIndices

    def syncToGhost(self, qty, simulationState, simulation):
        if self.periodicX or self.periodicX:
            ghosts = simulationState['ghosts']
            qty[simulationState['numParticles'] - ghosts.shape[0]:] = qty[ghosts]
