"""Batched serving of many deltaSPH scenes on one GB300.

`SceneBatch` holds any number of independent scenes in one concatenated particle array
(per-particle scene index, per-scene grid / parameters / dt in a device scene table,
(scene, cell) sort keys) and advances all of them with one fixed sequence of kernels:
keys -> counting sort -> permute -> mDBC beside neighbor records + segment lists -> pass 1
-> diffusion + update (with pairs = "csr": a CSR count / scan / fill after the permute).
Buffers are static, so one batch step can be captured once in a CUDA graph and replayed.
Scenes never interact: each scene's particles sort into their own cell range and every
kernel reads only its own scene's cells, so a scene gives the same bits alone and in any
mix.

`Server` is the request loop: requests arrive (a trace with arrival times), are admitted
while the device memory budget allows, step together with every other live scene, and
retire after their step count.  Admission / retirement rebuild the batch between steps;
steps in between replay the captured graph.  It records per-scene step latency and
time-to-completion.
"""
from __future__ import annotations

import bisect
import ctypes
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as N
from .search import MAX_CELLS, Workspace
from .sim import SimConfig, SphParamsC, FluidViewC, WallViewC, DIFFUSION


def _params_for(cfg: SimConfig, h: float, cells: int, cell_ratio: int = 1) -> SphParamsC:
    P = SphParamsC()
    P.support = h
    P.rest_density = cfg.rest_density
    P.c0 = cfg.c0
    P.gamma = cfg.gamma
    P.alpha = cfg.alpha
    P.delta = cfg.delta
    P.kinematic = cfg.kinematic
    P.gravity[0], P.gravity[1] = cfg.gravity
    P.point_source = int(cfg.point_source)
    P.point_magnitude = cfg.point_magnitude
    P.point_center[0], P.point_center[1] = cfg.point_center
    P.density_diffusion = DIFFUSION[cfg.density_diffusion]
    P.boundary_diffusion = int(bool(cfg.boundary_diffusion))
    P.search_radius = cfg.search_radius * cell_ratio     # cells of h / cell_ratio
    P.cell_capacity = cells
    return P


class ForceGroupC(ctypes.Structure):
    """sph_force_group: sorted particles [begin, end), lanes per particle, diffusion scheme."""
    _fields_ = [("begin", ctypes.c_int64), ("end", ctypes.c_int64), ("tpp", ctypes.c_int32),
                ("scheme", ctypes.c_int32)]


class _Grid(ctypes.Structure):
    _fields_ = [("qmin", ctypes.c_float * 2), ("hmax", ctypes.c_float), ("hmax_threshold", ctypes.c_float),
                ("cells_x", ctypes.c_int32), ("cells_y", ctypes.c_int32), ("num_cells", ctypes.c_int32),
                ("threshold_support", ctypes.c_float)]


@dataclass
class SceneSpec:
    scene: dict
    cfg: SimConfig
    steps: int = 1000
    name: str = ""
    cell_ratio: int = 1      # grid cells of support / cell_ratio, searched cell_ratio cells out
    tpp: int = 1             # lanes per particle in the force passes (1, 2, 4; pairs from cell rows)
    dev: dict | None = field(default=None, repr=False)   # device copies + grid, made once

    def on_device(self, device):
        """The scene's arrays on `device` and its grid (host copies of the sph_grid), cached."""
        upload_scenes([self], device)
        return self.dev


_FIELDS = (("pos", "pos", 2, "n"), ("vel", "vel", 2, "n"), ("rho", "rho", 1, "n"), ("area", "area", 1, "n"),
           ("sup", "support", 1, "n"), ("wall_pos", "wall_pos", 2, "nb"), ("ghost_pos", "ghost_pos", 2, "nb"),
           ("wall_area", "wall_area", 1, "nb"))


def _pinned(a, dtype):
    t = torch.empty(a.shape, dtype=dtype, pin_memory=True)
    t.numpy()[...] = a
    return t


class PendingUpload:
    """Scenes whose arrays and grid launch are queued on the device (upload_scenes with
    wait=False).  finish() waits for the event behind the grids' copy back to pinned host
    memory (long done when called a step later), checks the status and gives each spec its
    `dev` entry."""

    def __init__(self, todo, device, counts, dev_fields, grids_host, status_host, event, keep):
        self.todo, self.device, self.counts, self.dev_fields = todo, device, counts, dev_fields
        self.grids_host, self.status_host, self.event, self._keep = grids_host, status_host, event, keep

    def ready(self) -> bool:
        return self.event is None or self.event.query()

    def finish(self):
        if self.event is not None:
            self.event.synchronize()
        self._keep = None
        flags = int(self.status_host[0])
        if flags:
            raise N.SPHError(f"scene grids: {N.decode_flags(flags)}")
        raw = self.grids_host.numpy().tobytes()
        offs = {name: np.concatenate([[0], np.cumsum(c)]) for name, (_, c) in self.dev_fields.items()}
        for s, sp in enumerate(self.todo):
            d = {"device": self.device, "n": self.counts["n"][s], "nb": self.counts["nb"][s],
                 "cell_ratio": sp.cell_ratio, "grid": _Grid.from_buffer_copy(raw[32 * s:32 * (s + 1)])}
            d["src"] = {}
            for name, (t, _) in self.dev_fields.items():
                lo, hi = offs[name][s], offs[name][s + 1]
                if hi > lo:
                    d[name] = t[lo:hi]
                    d["src"][name] = (t, int(lo), int(hi))   # rows of one upload buffer
            sp.dev = d


def upload_scenes(specs, device, wait: bool = True):
    """Device copies and grids of every spec not yet on `device`: one copy per field for all
    of them (from pinned host memory) and one grid launch (sph_grid_build_segments).  Every
    host-to-device copy comes from pinned memory and the grids come back through pinned
    memory behind an event, so with wait=False nothing here waits for the device: the
    returned PendingUpload is finished later (None when every spec was on the device)."""
    device = torch.device(device)
    todo = [sp for sp in specs if sp.dev is None or sp.dev["device"] != device or
            sp.dev["cell_ratio"] != sp.cell_ratio]
    if not todo:
        return None
    counts = {"n": [len(sp.scene["pos"]) for sp in todo],
              "nb": [len(sp.scene.get("wall_pos", ())) for sp in todo]}
    dev_fields = {}
    keep = []                     # pinned sources, alive until the copies have run
    # a large upload (a burst of arrivals) goes from pageable memory: on this host a copy
    # from pageable memory runs about as fast as from pinned memory, and page-locking a
    # fresh buffer of hundreds of MB costs far more than the copy; small uploads use torch's
    # cached pinned blocks and stay asynchronous
    big = sum(counts["n"]) * 24 + sum(counts["nb"]) * 20 > (64 << 20)
    for name, key, width, cnt in _FIELDS:
        c = counts[cnt]
        total = sum(c)
        if total == 0:
            continue
        shape = (total, width) if width > 1 else (total,)
        host = torch.from_numpy(np.empty(shape, np.float32)) if big else torch.empty(shape, dtype=torch.float32,
                                                                                       pin_memory=True)
        hv = host.numpy()
        o = 0
        for sp, k in zip(todo, c):
            if k:
                hv[o:o + k] = np.asarray(sp.scene[key], np.float32).reshape(hv[o:o + k].shape)
                o += k
        dev_fields[name] = (host.to(device, non_blocking=True), c)
        keep.append(host)
    S = len(todo)
    # the grid's cell size is the largest support of the scene over its cell_ratio; the grid
    # pads the domain by one cell below and two above, so the domain given to it grows by
    # the difference to keep that padding one and two supports (walls lie in it)
    grow = np.array([float(np.max(sp.scene["support"])) * (1.0 - 1.0 / sp.cell_ratio) for sp in todo],
                    np.float32)[:, None]
    small = [_pinned(np.concatenate([[0], np.cumsum(counts["n"])]).astype(np.int64), torch.int64),
             _pinned(np.array([sp.scene["vmin"] for sp in todo], np.float32) - grow, torch.float32),
             _pinned(np.array([sp.scene["vmax"] for sp in todo], np.float32) + 2.0 * grow, torch.float32)]
    keep += small
    seg, vmin, vmax = (t.to(device, non_blocking=True) for t in small)
    grids = torch.empty(S * 8, dtype=torch.int32, device=device)
    status = torch.zeros(1, dtype=torch.int32, device=device)
    cell_h = dev_fields["sup"][0]
    if any(sp.cell_ratio != 1 for sp in todo):
        per = _pinned(np.repeat(np.array([1.0 / sp.cell_ratio for sp in todo], np.float32), counts["n"]),
                      torch.float32)
        keep.append(per)
        cell_h = cell_h * per.to(device, non_blocking=True)
    N.call("sph_grid_build_segments", N.ptr(dev_fields["pos"][0]), N.ptr(cell_h), N.ptr(seg), S,
           N.ptr(vmin), N.ptr(vmax), MAX_CELLS, N.ptr(grids), N.ptr(status), N.stream_ptr())
    grids_host = torch.empty(S * 8, dtype=torch.int32, pin_memory=True)
    status_host = torch.empty(1, dtype=torch.int32, pin_memory=True)
    grids_host.copy_(grids, non_blocking=True)
    status_host.copy_(status, non_blocking=True)
    ev = torch.cuda.Event()
    ev.record()
    pending = PendingUpload(todo, device, counts, dev_fields, grids_host, status_host, ev,
                            keep + [seg, vmin, vmax, grids, status, cell_h])
    if wait:
        pending.finish()
    return pending


def scene_order(lanes, schemes):
    """Batch order of the scenes: grouped by (lanes per particle, diffusion scheme), each
    group in the given order.  Returns order[k] = the input index of batch scene k."""
    return sorted(range(len(lanes)), key=lambda k: (lanes[k], schemes[k]))


def force_groups(p_off, kinds):
    """Force-pass groups of a batch whose scene k (in batch order) holds the particles
    [p_off[k], p_off[k+1]) and has kind (lanes per particle, scheme): one [begin, end, tpp,
    scheme] per run of equal kinds, tiling [0, p_off[-1]); one default group for no scenes."""
    groups = []
    for k, kind in enumerate(kinds):
        if k == 0 or kind != kinds[k - 1]:
            groups.append([p_off[k], p_off[k + 1], *kind])
        else:
            groups[-1][1] = p_off[k + 1]
    return groups or [[0, p_off[-1] if p_off else 0, 1, -1]]


class SceneBatch:
    """A fixed set of scenes stepped together (deltaSPH, semi-implicit Euler).

    pairs = "cells": the force passes take each particle's pairs straight from its cell rows
    (no neighbor list; the records launch keeps each particle's accepted candidates as
    segment bit masks for both force passes).  pairs =
    "csr": a CSR neighbor list is counted and filled every step first.  Both visit the
    pairs in the same order and give the same sums.

    Each scene runs with its spec's cell_ratio and tpp (set from `tuning`, a
    `tune.Tuning`, when given): the batch keeps its scenes grouped by (tpp, density-diffusion
    scheme), and each group is one particle range of the force passes with a kernel compiled
    for its lanes and scheme.  Per-scene methods take the scenes' indices in `specs` order."""

    def __init__(self, specs, device=None, states=None, pair_headroom: float = 1.3, pairs: str = "cells",
                 tuning=None):
        if pairs not in ("cells", "csr"):
            raise ValueError("pairs must be 'cells' or 'csr'")
        self.pairs = pairs
        self.lib = N.load()
        self.device = torch.device(device or torch.device("cuda", torch.cuda.current_device()))
        dev = self.device
        specs = list(specs)
        if tuning is not None:
            for sp in specs:
                tuning.configure(sp)
        for sp in specs:
            if sp.tpp not in (1, 2, 4) or sp.cell_ratio not in (1, 2):
                raise ValueError("tpp must be 1, 2 or 4 and cell_ratio 1 or 2")
        lanes = [sp.tpp if pairs == "cells" else 1 for sp in specs]
        schemes = [DIFFUSION[sp.cfg.density_diffusion] for sp in specs]
        # scenes grouped by (lanes per particle, scheme), stable: _order[k] = the spec of batch scene k
        self._order = scene_order(lanes, schemes)
        self._slot = [0] * len(specs)
        for k, e in enumerate(self._order):
            self._slot[e] = k
        self.specs = [specs[e] for e in self._order]
        if states is not None:
            states = [states[e] for e in self._order]
        S = len(self.specs)
        upload_scenes(self.specs, dev)
        rec = self.lib.sph_scene_bytes()
        table = bytearray(rec * max(S, 1))
        self.grids, self.coff = [], []
        pos, vel, rho, area, sup = [], [], [], [], []
        wpos, wgh, war, nbs = [], [], [], []
        self.p_off = [0]
        total_cells = 0
        self.any_renorm = False
        as_dev = lambda a: torch.as_tensor(a, device=dev, dtype=torch.float32)
        for s, spec in enumerate(self.specs):
            cfg = spec.cfg
            if cfg.solver != "deltaSPH" or cfg.integration != "semiImplicitEuler":
                raise N.SPHError("batched serving runs deltaSPH with semi-implicit Euler")
            d = spec.on_device(dev)
            g = d["grid"]
            h = float(np.float32(spec.scene["support"][0]))
            P = _params_for(cfg, h, g.num_cells, spec.cell_ratio)
            buf = ctypes.create_string_buffer(rec)
            N.check(self.lib.sph_scene_encode(ctypes.byref(P), ctypes.byref(g), total_cells, cfg.dt, buf),
                    "scene_encode")
            table[s * rec:(s + 1) * rec] = buf.raw
            self.grids.append(g)
            self.coff.append(total_cells)
            total_cells += g.num_cells + 1      # the scene's cells and its outside slot
            self.any_renorm |= cfg.density_diffusion == "deltaSPH"
            st = states[s] if states is not None else None
            n = d["n"]
            pos.append(as_dev(st["x"]).reshape(n, 2) if st else d["pos"])
            vel.append(as_dev(st["v"]).reshape(n, 2) if st else d["vel"])
            rho.append(as_dev(st["rho"]) if st else d["rho"])
            area.append(d["area"])
            sup.append(d["sup"])
            self.p_off.append(self.p_off[-1] + n)
            nbs.append(d["nb"])
            if d["nb"]:
                wpos.append(d["wall_pos"])
                wgh.append(d["ghost_pos"])
                war.append(d["wall_area"])
        if total_cells >= MAX_CELLS:
            raise N.SPHError("batch cell tables too large")
        self.cap = max(total_cells, 1)
        self.scenes = torch.frombuffer(bytearray(table), dtype=torch.uint8).to(dev)
        # slot of each scene that holds its particles outside its grid
        self.outside_slot = torch.tensor([c + g.num_cells for c, g in zip(self.coff, self.grids)] or [0],
                                         dtype=torch.int64, device=dev)
        self.n = self.p_off[-1]
        n = self.n
        self.groups = force_groups(self.p_off, [(lanes[e], schemes[e]) for e in self._order])
        self._groups_c = (ForceGroupC * len(self.groups))(*[ForceGroupC(*g) for g in self.groups])
        # scene index and particle id of every particle; p_off_dev[sid] + uid is its slot in the
        # concatenation of the scenes in their own particle order
        counts = torch.tensor(np.diff(self.p_off), dtype=torch.int64, device=dev)
        self.p_off_dev = torch.tensor(self.p_off[:-1] or [0], dtype=torch.int64, device=dev)
        sid = torch.repeat_interleave(torch.arange(S, dtype=torch.int32, device=dev), counts)
        uid = (torch.arange(n, dtype=torch.int64, device=dev) - self.p_off_dev[sid.long()]).to(torch.int32)
        wsid = [torch.repeat_interleave(torch.arange(S, dtype=torch.int32, device=dev),
                                        torch.tensor(nbs, dtype=torch.int64, device=dev))] if sum(nbs) else []
        self.a = {"x": torch.cat(pos), "v": torch.cat(vel), "rho": torch.cat(rho), "area": torch.cat(area),
                  "sup": torch.cat(sup), "sid": sid, "uid": uid}
        self.b = {k: torch.empty_like(v) for k, v in self.a.items()}
        # x, v, rho: unsorted state in a, sorted copy in b (the update writes a).  The static
        # per-particle arrays alternate instead: the state's are in a (par 0) or b (par 1),
        # the sort writes the other set, which becomes the state's after the step.
        self.par = 0
        self.s = None            # the sorted working set of the current step
        self._inv = torch.empty(n, dtype=torch.int32, device=dev)
        self.ws = Workspace(dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.keys = torch.empty(n, dtype=torch.int32, device=dev)
        self.order = torch.empty(n, dtype=torch.int32, device=dev)
        self.skeys = torch.empty(n, dtype=torch.int32, device=dev)
        self.cell_start = torch.empty(self.cap + 2, dtype=torch.int32, device=dev)
        self.hist = torch.zeros(self.cap + 1, dtype=torch.int32, device=dev)
        self.cs_scratch = torch.empty((self.lib.sph_counting_sort_scratch_bytes(n, self.cap) + 7) // 8,
                                      dtype=torch.int64, device=dev)
        self.dpdt = torch.empty(n, dtype=torch.float32, device=dev)
        self.acc = torch.empty((n, 2), dtype=torch.float32, device=dev)
        self.grad_rho = torch.empty((n, 2), dtype=torch.float32, device=dev) if self.any_renorm else None
        self.forces_scratch = torch.empty((self.lib.sph_deltasph_scratch_bytes(n) + 7) // 8, dtype=torch.int64,
                                          device=dev)
        # walls: concatenated, sorted once by (scene, cell)
        self.nb = sum(len(w) for w in wpos)
        self._setup_walls(wpos, wgh, war, wsid)
        self.counts = self.offsets = self.cols = None
        self.pair_cap = 0
        if pairs == "csr":
            self.counts = torch.empty(n, dtype=torch.int32, device=dev)
            self.offsets = torch.empty(n + 1, dtype=torch.int32, device=dev)
            self.scan_scratch = torch.empty((self.lib.sph_scan_scratch_bytes(n) + 7) // 8, dtype=torch.int64,
                                            device=dev)
            # pair capacity from a first count
            self._sort_permute()
            self._count()
            P = int(self.offsets[n].item())
            self.pair_cap = int(P * pair_headroom) + 1024
            self.cols = torch.empty(self.pair_cap, dtype=torch.int32, device=dev)
        self.graph = None
        self._side = torch.cuda.Stream(dev)
        self.steps_done = 0

    def _setup_walls(self, wpos, wgh, war, wsid):
        dev = self.device
        nb = self.nb
        if nb == 0:
            z = torch.zeros(1, dtype=torch.float32, device=dev)
            self.w = {"x": torch.zeros((1, 2), device=dev), "ghost": torch.zeros((1, 2), device=dev), "area": z,
                      "rho": z.clone(), "vol": z.clone(), "p": z.clone(), "sid": torch.zeros(1, dtype=torch.int32, device=dev),
                      "cell_start": torch.zeros(self.cap + 2, dtype=torch.int32, device=dev), "order": None}
        else:
            x = torch.cat(wpos)
            sid = torch.cat(wsid)
            keys = torch.empty(nb, dtype=torch.int32, device=dev)
            order = torch.empty(nb, dtype=torch.int32, device=dev)
            skeys = torch.empty(nb, dtype=torch.int32, device=dev)
            cs = torch.empty(self.cap + 2, dtype=torch.int32, device=dev)
            hist = torch.zeros(self.cap + 1, dtype=torch.int32, device=dev)
            st = N.stream_ptr()
            N.call("sph_batch_cell_keys", N.ptr(x), nb, N.ptr(sid), N.ptr(self.scenes), self.cap, N.ptr(keys),
                   N.ptr(hist), N.ptr(self.status), st)
            scr = torch.empty((self.lib.sph_counting_sort_scratch_bytes(nb, self.cap) + 7) // 8, dtype=torch.int64,
                              device=dev)
            N.call("sph_counting_sort", N.ptr(keys), nb, self.cap, N.ptr(hist), N.ptr(cs), N.ptr(order), N.ptr(skeys),
                   N.ptr(self.status), N.ptr(scr), scr.numel() * 8, st)
            perm = lambda t: self._perm(order, t)
            self.w = {"x": perm(x), "ghost": perm(torch.cat(wgh)), "area": perm(torch.cat(war)),
                      "sid": perm(sid), "cell_start": cs, "rho": torch.ones(nb, device=dev),
                      "vol": torch.zeros(nb, device=dev), "p": torch.zeros(nb, device=dev), "order": order}
        self.wall_view = WallViewC(N.ptr(self.w["x"]), N.ptr(self.w["ghost"]), N.ptr(self.w["area"]),
                                   N.ptr(self.w["cell_start"]), nb, N.ptr(self.w["rho"]), N.ptr(self.w["vol"]),
                                   N.ptr(self.w["p"]))

    def _perm(self, order, t, out=None):
        if out is None:
            out = torch.empty_like(t)
        eb = t.element_size() * (t.shape[1] if t.dim() == 2 else 1)
        N.call("sph_permute", N.ptr(order), t.shape[0], eb, N.ptr(t), N.ptr(out), N.stream_ptr())
        return out

    # ------------------------------------------------------------------ one batch step
    @property
    def AUX(self):
        """The static per-particle arrays that follow the sort: the sorted supports only
        matter to the CSR search; with pairs from the cell rows the scene's support is used."""
        return ("area", "sup", "sid", "uid") if self.pairs == "csr" else ("area", "sid", "uid")

    def _aux(self, which: int) -> dict:
        return self.a if which == 0 else self.b

    def state_arrays(self) -> dict:
        """x, v, rho and the static per-particle arrays of the current (unsorted) state."""
        cur = self._aux(self.par)
        return {"x": self.a["x"], "v": self.a["v"], "rho": self.a["rho"], **{k: cur[k] for k in self.AUX}}

    def _sort_permute(self):
        st = N.stream_ptr()
        n = self.n
        cur, nxt = self._aux(self.par), self._aux(self.par ^ 1)
        N.call("sph_batch_cell_keys", N.ptr(self.a["x"]), n, N.ptr(cur["sid"]), N.ptr(self.scenes), self.cap,
               N.ptr(self.keys), N.ptr(self.hist), N.ptr(self.status), st)
        # inside a cell, order by particle id: a scene's order never depends on its history
        # or on the other scenes of the batch
        # the state moves into the sorted order in the same launches
        k, eb, ins, outs = N.array_set([(self.a[k], self.b[k]) for k in ("x", "v", "rho")] +
                                       [(cur[k], nxt[k]) for k in self.AUX])
        N.call("sph_counting_sort_permute", N.ptr(self.keys), n, self.cap, N.ptr(self.hist), N.ptr(self.cell_start),
               N.ptr(cur["uid"]), N.ptr(self.order), N.ptr(self.skeys), k, eb, ins, outs, N.ptr(self.status),
               N.ptr(self.cs_scratch), self.cs_scratch.numel() * 8, st)
        self.s = {"x": self.b["x"], "v": self.b["v"], "rho": self.b["rho"], **{k: nxt[k] for k in self.AUX}}

    def _count(self):
        st = N.stream_ptr()
        n = self.n
        b = self.s
        N.call("sph_batch_nl_count", N.ptr(b["x"]), N.ptr(b["sup"]), n, N.ptr(self.skeys), N.ptr(self.cell_start),
               N.ptr(self.scenes), N.ptr(b["sid"]), N.ptr(self.counts), st)
        N.call("sph_exclusive_scan_i32", N.ptr(self.counts), N.ptr(self.offsets), n, N.ptr(self.scan_scratch),
               self.scan_scratch.numel() * 8, st)

    def _pair_list(self):
        """The CSR neighbor list of the sorted batch (pairs = "csr" only)."""
        if self.pairs != "csr":
            return
        b = self.s
        self._count()
        N.call("sph_batch_nl_fill", N.ptr(b["x"]), N.ptr(b["sup"]), self.n, N.ptr(self.skeys),
               N.ptr(self.cell_start), N.ptr(self.scenes), N.ptr(b["sid"]), N.ptr(self.offsets), self.pair_cap,
               N.ptr(self.cols), N.ptr(self.status), N.stream_ptr())

    def fluid_view(self):
        """The sorted batch as the C ABI's fluid view (no CSR arrays with pairs = "cells")."""
        b = self.s
        return FluidViewC(N.ptr(b["x"]), N.ptr(b["v"]), N.ptr(b["rho"]), N.ptr(b["area"]), N.ptr(self.skeys),
                          N.ptr(self.offsets), N.ptr(self.cols), N.ptr(self.cell_start), self.n, self.pair_cap)

    def forces(self, out, phases=None):
        """The launches of sph_batch_deltasph_step selected by `phases` (all by default),
        writing the updated state to out["x"], out["v"], out["rho"]."""
        b = self.s
        fv = self.fluid_view()
        N.call("sph_batch_deltasph_step", ctypes.byref(fv), ctypes.byref(self.wall_view), N.ptr(self.scenes),
               N.ptr(b["sid"]), N.ptr(self.w["sid"]), N.ptr(self.dpdt), N.ptr(self.acc), N.ptr(self.grad_rho),
               int(self.any_renorm), N.ptr(out["x"]), N.ptr(out["v"]), N.ptr(out["rho"]), N.ptr(self.status),
               N.SPH_PHASE_ALL if phases is None else phases, len(self._groups_c),
               ctypes.cast(self._groups_c, ctypes.c_void_p), N.ptr(self.forces_scratch),
               self.forces_scratch.numel() * 8, N.stream_ptr())

    def step_kernels(self):
        """The batch step as a fixed kernel sequence (no host synchronisation).  The wall
        densities (mDBC) run on a side stream beside the neighbor records: they read the
        sorted fluid and write only the wall arrays, and pass 1 waits for both."""
        a = self.a
        self._sort_permute()
        self._pair_list()
        if self.nb:
            main = torch.cuda.current_stream()
            self._side.wait_stream(main)
            with torch.cuda.stream(self._side):
                self.forces(a, N.SPH_PHASE_WALLS)
            self.forces(a, N.SPH_PHASE_RECORDS)
            main.wait_stream(self._side)
            self.forces(a, N.SPH_PHASE_PASS1 | N.SPH_PHASE_DIFFUSION)
        else:
            self.forces(a)
        self.par ^= 1             # the sorted static arrays are the state's now

    # kernels of this library launched by one batch step (for the bench's launch count): keys 1,
    # counting sort with the state's permute (scan 1 + scatter + fix + fix_large), [csr: count
    # 1, scan 1, fill 1], mdbc 1, records 1, per force group pass1 + update 1 (+ diffusion +
    # update 1 for a group with deltaSPH scenes).  A scan is one kernel (above 16,384 items its tile words
    # are zeroed by a memset first, which is not a kernel).
    def launches_per_step(self):
        sort = 1 + 3
        csr = 1 + 1 + 1 if self.pairs == "csr" else 0
        p1 = sum(1 for lo, hi, _, _ in self.groups if hi > lo)
        dif = sum(1 for lo, hi, _, k in self.groups if hi > lo and k not in (0, 1)) if self.any_renorm else 0
        return 1 + sort + csr + (1 if self.nb else 0) + 1 + p1 + dif

    def capture(self):
        """Capture one batch step into a CUDA graph (after a warm-up step)."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.step_kernels()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        # one graph per parity of the static arrays; capturing runs nothing, so after the two
        # captures the parity is the device state's again
        graphs = [None, None]
        for _ in range(2):
            p = self.par
            graphs[p] = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graphs[p]):
                self.step_kernels()
        self.graph = graphs
        torch.cuda.synchronize()
        self.steps_done += 1

    def step(self):
        if self.graph is not None:
            self.graph[self.par].replay()
            self.par ^= 1
        else:
            self.step_kernels()
        self.steps_done += 1

    # flags that leave every scene's result valid: particles that left their scene's grid
    # (they move under body forces only, see escaped()), and a cell too large for the
    # reproducible in-cell order (summation order only)
    BENIGN = N.SPH_FLAG_OUT_OF_GRID | N.SPH_FLAG_CELL_ORDER

    def flags(self) -> int:
        return int(self.status.item())

    def check(self, allow: int = BENIGN):
        f = self.flags() & ~allow
        if f:
            raise N.SPHError(f"batch step: {N.decode_flags(f)}")
        if self.pairs == "csr" and int(self.offsets[self.n].item()) > self.pair_cap:
            raise N.SPHError("batch step: neighbor pair buffer too small")

    def escaped(self):
        """Per scene, how many of its particles were outside its grid at the last sort."""
        if not self.specs:
            return np.zeros(0, np.int64)
        cs = self.cell_start.long()
        per_slot = (cs[self.outside_slot + 1] - cs[self.outside_slot]).cpu().numpy()
        return per_slot[self._slot]

    def scene_finite(self, s: int) -> bool:
        k = self._slot[s]
        lo, hi = self.p_off[k], self.p_off[k + 1]
        return bool(torch.isfinite(self.a["x"][lo:hi]).all() and torch.isfinite(self.a["v"][lo:hi]).all()
                    and torch.isfinite(self.a["rho"][lo:hi]).all())

    # ------------------------------------------------------------------ output
    def states_device(self):
        """Positions, velocities and densities of every scene in its original particle order,
        concatenated scene after scene in batch order (device; take a scene with
        scene_state_device)."""
        cur = self._aux(self.par)
        dst = (self.p_off_dev[cur["sid"].long()] + cur["uid"].long()).to(torch.int32)
        out = {k: torch.empty_like(self.a[k]) for k in ("x", "v", "rho")}
        N.call("sph_invert_permutation", N.ptr(dst), self.n, N.ptr(self._inv), N.stream_ptr())
        N.permute_arrays(self._inv, [(self.a[k], out[k]) for k in ("x", "v", "rho")])
        return out

    def scene_state_device(self, s: int, states=None):
        """Positions, velocities and densities of scene s in its original particle order (device)."""
        states = states or self.states_device()
        k = self._slot[s]
        lo, hi = self.p_off[k], self.p_off[k + 1]
        return {key: v[lo:hi] for key, v in states.items()}

    def scene_state(self, s: int):
        """Positions, velocities and densities of scene s in its original particle order (numpy)."""
        return {k: v.cpu().numpy() for k, v in self.scene_state_device(s).items()}

    def device_bytes(self):
        tot = 0
        for d in (self.a, self.b):
            tot += sum(t.numel() * t.element_size() for t in d.values())
        if self.cols is not None:
            tot += self.cols.numel() * 4 + self.n * 8
        tot += self.forces_scratch.numel() * 8 + (self.cap + 2) * 8 + self.n * 32
        return tot


class ArenaFull(Exception):
    """The arena has no room for a scene (particles, walls, cells or slots)."""


class SceneArena(SceneBatch):
    """A pooled arena of fixed capacity for continuous batching: scenes are admitted into free
    particle slots and retired from them between steps, without rebuilding the batch or
    re-capturing its CUDA graphs.

    The arrays of SceneBatch are allocated for `particles` particles, `walls` wall particles,
    `cells` cell slots and `slots` scenes.  A slot of no scene carries scene index -1: the sort
    sends it to the sentinel cell after every scene's cells and the batch kernels skip it, so
    every step compacts the live scenes to the front of the sorted arrays.  Admission writes
    the scene's particles after the occupied ones, its static arrays, its scene-table entry
    and a cell range (first fit; the live scenes' ranges are packed again when no gap fits,
    which changes no result) and its walls; retirement reads the scene's state out in its own
    particle order and marks its particles and walls free.  The walls are sorted again once
    before the next step, however many scenes came or went.  Every scene runs with the arena's
    lanes per particle `tpp` and density-diffusion kernel `scheme` (-1: read per scene); pairs
    come from the cell rows.  A step processes only the occupied slots rounded up to a
    multiple of `extent_quantum` (by default the larger of 2^17 and a sixteenth of the
    capacity), and sorts into the cell slots up to the highest live scene's, rounded the same
    way, with a captured graph per extent, so an arena sized for a peak load steps a light
    load at the light load's cost.  A scene gives the same bits in the arena as alone."""

    def __init__(self, device=None, particles: int = 1 << 20, walls: int = 1 << 16, cells: int = 1 << 20,
                 slots: int = 256, tpp: int = 1, scheme: int = -1, extent_quantum: int | None = None):
        if tpp not in (1, 2, 4) or scheme not in (-1, 0, 1, 2):
            raise ValueError("tpp must be 1, 2 or 4 and scheme -1, 0, 1 or 2")
        self.pairs = "cells"
        self.lib = N.load()
        self.device = torch.device(device or torch.device("cuda", torch.cuda.current_device()))
        dev = self.device
        self.N, self.WC, self.C, self.S = int(particles), int(walls), int(cells), int(slots)
        if self.C + 1 >= MAX_CELLS:
            raise N.SPHError("arena cell tables too large")
        self.tpp, self.scheme = tpp, scheme
        self.rec = self.lib.sph_scene_bytes()
        self.scenes = torch.zeros(self.S * self.rec, dtype=torch.uint8, device=dev)
        self.cap = self.C
        self.n = self.N
        n = self.N
        self._quantum = int(extent_quantum) if extent_quantum else max(1 << 17, -(-self.N // 16))
        self._cell_quantum = int(extent_quantum) if extent_quantum else max(1 << 17, -(-self.C // 16))
        self._graphs = {}
        f2 = lambda m: torch.zeros((m, 2), dtype=torch.float32, device=dev)
        f1 = lambda m: torch.zeros(m, dtype=torch.float32, device=dev)
        i1 = lambda m, v=0: torch.full((m,), v, dtype=torch.int32, device=dev)
        self.a = {"x": f2(n), "v": f2(n), "rho": f1(n) + 1.0, "area": f1(n), "sup": f1(n), "sid": i1(n, -1),
                  "uid": i1(n)}
        self.b = {k: v.clone() for k, v in self.a.items()}
        self.par = 0
        self.s = None
        self._inv = i1(n)
        self.ws = Workspace(dev)
        self.status = i1(1)
        self.keys, self.order, self.skeys = i1(n), i1(n), i1(n)
        self.cell_start = i1(self.C + 2)
        self.hist = i1(self.C + 1)
        self.cs_scratch = torch.empty((self.lib.sph_counting_sort_scratch_bytes(n, self.C) + 7) // 8,
                                      dtype=torch.int64, device=dev)
        self.dpdt, self.acc = f1(n), f2(n)
        self.any_renorm = scheme in (-1, 2)
        self.grad_rho = f2(n) if self.any_renorm else None
        self.forces_scratch = torch.empty((self.lib.sph_deltasph_scratch_bytes(n) + 7) // 8, dtype=torch.int64,
                                          device=dev)
        self.groups = [[0, n, tpp, scheme]]
        self._groups_c = (ForceGroupC * 1)(ForceGroupC(0, n, tpp, scheme))
        # walls: an unsorted staging list (live walls first) and the sorted arrays the graph reads
        W = self.WC
        self.nb = W
        self.ws_w = {"x": f2(W), "ghost": f2(W), "area": f1(W), "sid": i1(W, -1), "uid": i1(W)}
        self.w = {"x": f2(W), "ghost": f2(W), "area": f1(W), "sid": i1(W, -1), "cell_start": i1(self.C + 2),
                  "rho": f1(W) + 1.0, "vol": f1(W), "p": f1(W), "order": i1(W)}
        self._wkeys, self._wskeys, self._whist = i1(W), i1(W), i1(self.C + 1)
        self._wcs = torch.empty((self.lib.sph_counting_sort_scratch_bytes(W, self.C) + 7) // 8, dtype=torch.int64,
                                device=dev)
        self.wall_view = WallViewC(N.ptr(self.w["x"]), N.ptr(self.w["ghost"]), N.ptr(self.w["area"]),
                                   N.ptr(self.w["cell_start"]), W, N.ptr(self.w["rho"]), N.ptr(self.w["vol"]),
                                   N.ptr(self.w["p"]))
        self.counts = self.offsets = self.cols = None
        self.pair_cap = 0
        self.graph = None
        self._side = torch.cuda.Stream(dev)
        self.steps_done = 0
        # host bookkeeping
        self.slots = {}                    # slot -> dict(spec, n, nb, coff, ncells, grid)
        self._cell_end = None              # end of the highest live cell range (None: recount)
        self.free_slots = list(range(self.S))
        self.occupied = 0                  # particle slots in use (live + retired before the next sort)
        self.live_n = 0
        self.walls_n = 0
        self.specs = []
        self._rows_host = torch.zeros(self.S * self.rec, dtype=torch.uint8, pin_memory=True)
        self._row_events = [None] * self.S
        self._cell_top = 0            # end of the highest cell range handed out
        self._walls_dirty = False     # walls admitted or retired since the last wall sort
        self._sort_walls()

    # ------------------------------------------------------------------ bookkeeping
    def _alloc_cells(self, size):
        # behind the highest range when it fits (no scan of the live ranges), else first fit
        top = self._cell_top
        if self.C - top >= size:
            self._cell_top = top + size
            return top
        used = sorted((d["coff"], d["ncells"]) for d in self.slots.values())
        at = 0
        for c, k in used:
            if c - at >= size:
                return at
            at = c + k
        if self.C - at >= size:
            return at
        if self.C - sum(k for _, k in used) >= size:   # pack the live scenes' ranges, then append
            self._pack_cells()
            at = sum(k for _, k in used)
            self._cell_top = at + size
            return at
        return None

    def _pack_cells(self):
        at = 0
        for slot in sorted(self.slots, key=lambda t: self.slots[t]["coff"]):
            d = self.slots[slot]
            d["coff"] = at
            self._write_scene(slot)
            at += d["ncells"]
        self._cell_top = at
        self._cell_end = None
        self._walls_dirty = True

    def _encode_row(self, slot):
        """The slot's scene-table row, into its row of the pinned staging table (a mirror of
        the device table); a row is rewritten only after the event behind its last copy."""
        d = self.slots[slot]
        sp = d["spec"]
        h = float(np.float32(sp.scene["support"][0]))
        P = _params_for(sp.cfg, h, d["grid"].num_cells, sp.cell_ratio)
        ev = self._row_events[slot]
        if ev is not None:
            ev.synchronize()
        row = self._rows_host[slot * self.rec:(slot + 1) * self.rec]
        buf = (ctypes.c_char * self.rec).from_address(row.data_ptr())
        N.check(self.lib.sph_scene_encode(ctypes.byref(P), ctypes.byref(d["grid"]), d["coff"], sp.cfg.dt, buf),
                "scene_encode")

    def _copy_rows(self, lo, hi):
        """Rows [lo, hi) of the staging table to the device table, behind the queued steps (no
        host wait); rows in between that did not change are copied unchanged."""
        a, b = lo * self.rec, hi * self.rec
        self.scenes[a:b].copy_(self._rows_host[a:b], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record()
        for k in range(lo, hi):
            self._row_events[k] = ev

    def _write_scene(self, slot):
        self._encode_row(slot)
        self._copy_rows(slot, slot + 1)

    def _sort_walls(self):
        """Sort the staging walls by (scene, cell) into the arrays the batch kernels read; the
        staging list becomes the sorted one (live walls first)."""
        st = N.stream_ptr()
        W = self.WC
        s = self.ws_w
        N.call("sph_batch_cell_keys", N.ptr(s["x"]), W, N.ptr(s["sid"]), N.ptr(self.scenes), self.C,
               N.ptr(self._wkeys), N.ptr(self._whist), N.ptr(self.status), st)
        N.call("sph_counting_sort", N.ptr(self._wkeys), W, self.C, N.ptr(self._whist), N.ptr(self.w["cell_start"]),
               N.ptr(self.w["order"]), N.ptr(self._wskeys), N.ptr(self.status), N.ptr(self._wcs),
               self._wcs.numel() * 8, st)
        for k in ("x", "ghost", "area", "sid"):
            self._perm(self.w["order"], s[k], out=self.w[k])
            s[k].copy_(self.w[k])

    def fits(self, spec) -> bool:
        n = len(spec.scene["pos"])
        nb = len(spec.scene.get("wall_pos", ()))
        return bool(self.free_slots) and self.occupied + n <= self.N and self.walls_n + nb <= self.WC

    # ------------------------------------------------------------------ admission / retirement
    def admit(self, spec, state=None) -> int:
        """Put a scene into the arena between steps; returns its slot.  Raises ArenaFull when
        its particles, walls, cells or a slot do not fit.  `state` (x, v, rho device or host
        arrays in the scene's particle order) continues a scene instead of starting it."""
        cfg = spec.cfg
        if cfg.solver != "deltaSPH" or cfg.integration != "semiImplicitEuler":
            raise N.SPHError("batched serving runs deltaSPH with semi-implicit Euler")
        if self.scheme >= 0 and DIFFUSION[cfg.density_diffusion] != self.scheme:
            raise N.SPHError("the scene's density diffusion is not the arena's")
        spec.tpp = self.tpp
        d = spec.on_device(self.device)
        n, nb = d["n"], d["nb"]
        if not self.fits(spec):
            raise ArenaFull("no room for the scene's particles, walls or a slot")
        ncells = d["grid"].num_cells + 1
        coff = self._alloc_cells(ncells)
        if coff is None:
            raise ArenaFull("no room in the cell tables")
        slot = self.free_slots.pop(0)
        self.slots[slot] = {"spec": spec, "n": n, "nb": nb, "coff": coff, "ncells": ncells, "grid": d["grid"]}
        self._cell_end = None
        self._write_scene(slot)
        st = N.stream_ptr()
        lo, hi = self.occupied, self.occupied + n
        if hi > self.n:
            self._set_extent(self._extent_for(hi))   # before the scene's slots are written
        cur = self._aux(self.par)
        as_dev = lambda t: torch.as_tensor(t, dtype=torch.float32, device=self.device)
        self.a["x"][lo:hi].copy_(as_dev(state["x"]).reshape(n, 2) if state else d["pos"])
        self.a["v"][lo:hi].copy_(as_dev(state["v"]).reshape(n, 2) if state else d["vel"])
        self.a["rho"][lo:hi].copy_(as_dev(state["rho"]) if state else d["rho"])
        cur["area"][lo:hi].copy_(d["area"])
        N.call("sph_arena_set_ids", N.ptr(cur["sid"]), N.ptr(cur["uid"]), lo, n, slot, st)
        self.occupied = hi
        self.live_n += n
        if nb:
            w0, w1 = self.walls_n, self.walls_n + nb
            self.ws_w["x"][w0:w1].copy_(d["wall_pos"])
            self.ws_w["ghost"][w0:w1].copy_(d["ghost_pos"])
            self.ws_w["area"][w0:w1].copy_(d["wall_area"])
            N.call("sph_arena_set_ids", N.ptr(self.ws_w["sid"]), N.ptr(self.ws_w["uid"]), w0, nb, slot, st)
            self.walls_n = w1
            self._walls_dirty = True
        self._specs = None
        return slot

    _PARTICLE_FIELDS = (("pos", "x"), ("vel", "v"), ("rho", "rho"), ("area", "area"))
    _WALL_FIELDS = (("wall_pos", "x"), ("ghost_pos", "ghost"), ("wall_area", "area"))

    def admit_many(self, specs):
        """admit() for several new scenes at once: the bookkeeping per scene, then one copy per
        field for each run of scenes that were uploaded side by side (upload_scenes), one
        copy of their scene-table rows, and the id stamps.  Returns their slots, or None
        (admitting none) when they do not all fit behind the occupied particles, walls and
        cell ranges; admit() one by one then finds gaps or raises ArenaFull."""
        if not specs:
            return []
        for sp in specs:
            cfg = sp.cfg
            if cfg.solver != "deltaSPH" or cfg.integration != "semiImplicitEuler":
                raise N.SPHError("batched serving runs deltaSPH with semi-implicit Euler")
            if self.scheme >= 0 and DIFFUSION[cfg.density_diffusion] != self.scheme:
                raise N.SPHError("the scene's density diffusion is not the arena's")
            sp.tpp = self.tpp
        upload_scenes(specs, self.device)
        ds = [sp.dev for sp in specs]
        n_tot = sum(d["n"] for d in ds)
        nb_tot = sum(d["nb"] for d in ds)
        cells = [d["grid"].num_cells + 1 for d in ds]
        if (len(self.free_slots) < len(specs) or self.occupied + n_tot > self.N or
                self.walls_n + nb_tot > self.WC or self.C - self._cell_top < sum(cells)):
            return None
        if self.occupied + n_tot > self.n:
            self._set_extent(self._extent_for(self.occupied + n_tot))   # before any slot is written
        slots = self.free_slots[:len(specs)]
        del self.free_slots[:len(specs)]
        for sp, d, slot, nc in zip(specs, ds, slots, cells):
            self.slots[slot] = {"spec": sp, "n": d["n"], "nb": d["nb"], "coff": self._cell_top, "ncells": nc,
                                "grid": d["grid"]}
            self._cell_top += nc
            self._encode_row(slot)
        self._cell_end = None
        self._copy_rows(min(slots), max(slots) + 1)
        st = N.stream_ptr()
        cur = self._aux(self.par)
        p, w = self.occupied, self.walls_n
        for d, slot in zip(ds, slots):
            N.call("sph_arena_set_ids", N.ptr(cur["sid"]), N.ptr(cur["uid"]), p, d["n"], slot, st)
            if d["nb"]:
                N.call("sph_arena_set_ids", N.ptr(self.ws_w["sid"]), N.ptr(self.ws_w["uid"]), w, d["nb"], slot, st)
            p += d["n"]
            w += d["nb"]
        dst = {"x": self.a["x"], "v": self.a["v"], "rho": self.a["rho"], "area": cur["area"]}
        self._copy_runs(ds, self._PARTICLE_FIELDS, dst, self.occupied)
        if nb_tot:
            self._copy_runs(ds, self._WALL_FIELDS, self.ws_w, self.walls_n)
            self._walls_dirty = True
        self.occupied = p
        self.live_n += n_tot
        self.walls_n = w
        self._specs = None
        return slots

    @staticmethod
    def _copy_runs(ds, fields, dst, start):
        """dst[name][start + ...] <- the scenes' rows of each field in order, one copy per run
        of scenes whose rows lie side by side in one upload buffer."""
        for name, key in fields:
            at = start
            run = None            # [buffer, lo, hi, dst offset]
            for d in ds:
                src = d["src"].get(name)
                if src is None:
                    continue
                t, lo, hi = src
                if run is not None and run[0] is t and run[2] == lo:
                    run[2] = hi
                else:
                    if run is not None:
                        dst[key][run[3]:run[3] + run[2] - run[1]].copy_(run[0][run[1]:run[2]])
                    run = [t, lo, hi, at]
                at += hi - lo
            if run is not None:
                dst[key][run[3]:run[3] + run[2] - run[1]].copy_(run[0][run[1]:run[2]])

    def scene_state_device(self, slot, states=None):
        """x, v, rho of the scene in `slot` in its own particle order (device, fresh tensors)."""
        d = self.slots[slot]
        n = d["n"]
        cur = self._aux(self.par)
        out = {"x": torch.empty((n, 2), dtype=torch.float32, device=self.device),
               "v": torch.empty((n, 2), dtype=torch.float32, device=self.device),
               "rho": torch.empty(n, dtype=torch.float32, device=self.device)}
        N.call("sph_arena_extract", N.ptr(self.a["x"]), N.ptr(self.a["v"]), N.ptr(self.a["rho"]), N.ptr(cur["sid"]),
               N.ptr(cur["uid"]), self.n, slot, N.ptr(out["x"]), N.ptr(out["v"]), N.ptr(out["rho"]), N.stream_ptr())
        return out

    def scene_state(self, slot):
        return {k: v.cpu().numpy() for k, v in self.scene_state_device(slot).items()}

    def scene_finite(self, slot) -> bool:
        s = self.scene_state_device(slot)
        return bool(all(torch.isfinite(t).all() for t in s.values()))

    def retire(self, slot):
        """Take the scene in `slot` out of the arena; returns its final x, v, rho (device)."""
        out = self.scene_state_device(slot)
        d = self.slots.pop(slot)
        self._cell_end = None
        st = N.stream_ptr()
        N.call("sph_arena_retire", N.ptr(self._aux(self.par)["sid"]), self.n, slot, st)
        if d["nb"]:
            N.call("sph_arena_retire", N.ptr(self.ws_w["sid"]), self.WC, slot, st)
            self.walls_n -= d["nb"]
            self._walls_dirty = True
        self.live_n -= d["n"]
        bisect.insort(self.free_slots, slot)
        self._specs = None
        return out

    @property
    def specs(self):
        """The live scenes' specs in slot order (built when asked for)."""
        if self._specs is None:
            self._specs = [self.slots[k]["spec"] for k in sorted(self.slots)]
        return self._specs

    @specs.setter
    def specs(self, value):
        self._specs = list(value)

    def _walls_ready(self):
        # one wall sort for all the admissions and retirements since the last step
        if self._walls_dirty:
            self._sort_walls()
            self._walls_dirty = False

    # ------------------------------------------------------------------ active extent
    # A step processes the slots [0, n) only, n the occupied slots rounded up to a multiple of
    # the extent quantum: the sort keeps the live scenes in front, so free capacity behind the
    # extent costs nothing.  Each extent has its own pair of captured graphs (cached).  Slots
    # that join the extent are first marked free in both copies of the static arrays (stale
    # scene indices may linger there from an earlier, larger extent); nothing reads a slot
    # outside the extent.
    def _extent_for(self, occupied: int) -> int:
        q = self._quantum
        return min(self.N, max(q, -(-occupied // q) * q))

    def _cell_extent(self) -> int:
        """The cell slots a step sorts into: up to the end of the highest live cell range,
        rounded up to the cell quantum (the sentinel cell of free slots sits right behind)."""
        if self._cell_end is None:   # recounted only after admissions and retirements
            self._cell_end = max((d["coff"] + d["ncells"] for d in self.slots.values()), default=0)
        end = self._cell_end
        q = self._cell_quantum
        return min(self.C, max(q, -(-end // q) * q))

    def _set_extent(self, n: int, cap: int | None = None):
        cap = self.cap if cap is None else cap
        if n == self.n and cap == self.cap:
            return
        if n > self.n:
            for which in (0, 1):
                self._aux(which)["sid"][self.n:n].fill_(-1)
        self.n = n
        self.cap = cap   # the histogram past it is zero (every sort leaves it so) and unread
        self.groups = [[0, n, self.tpp, self.scheme]]
        self._groups_c = (ForceGroupC * 1)(ForceGroupC(0, n, self.tpp, self.scheme))
        self.graph = self._graphs.get((n, cap))

    def _capture_extent(self):
        """Both parities' graphs of a step over the current extent (capturing runs nothing)."""
        graphs = [None, None]
        for _ in range(2):
            p = self.par
            graphs[p] = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graphs[p]):
                self.step_kernels()
        self.graph = graphs
        self._graphs[(self.n, self.cap)] = graphs

    def retire_many(self, slots):
        """retire() for several scenes at once: one pass over the particle slots extracts their
        states and frees them (one more frees their walls).  Returns (rows, (x, v, rho)):
        rows[slot] = (first row, count) of that scene in the three device buffers, each in
        the scene's own particle order."""
        if not slots:
            return {}, None
        dev = self.device
        row0 = np.full(self.S, -1, np.int64)
        nrows = np.zeros(self.S, np.int32)
        wrow0 = np.full(self.S, -1, np.int64)
        rows, at = {}, 0
        for sl in slots:
            d = self.slots[sl]
            row0[sl], nrows[sl] = at, d["n"]
            rows[sl] = (at, d["n"])
            at += d["n"]
            if d["nb"]:
                wrow0[sl] = 0
        t_row0, t_rows, t_wrow0 = (_pinned(a, dt).to(dev, non_blocking=True) for a, dt in
                                   ((row0, torch.int64), (nrows, torch.int32), (wrow0, torch.int64)))
        out = (torch.empty((at, 2), dtype=torch.float32, device=dev), torch.empty((at, 2), dtype=torch.float32, device=dev),
               torch.empty(at, dtype=torch.float32, device=dev))
        st = N.stream_ptr()
        cur = self._aux(self.par)
        N.call("sph_arena_extract_many", N.ptr(self.a["x"]), N.ptr(self.a["v"]), N.ptr(self.a["rho"]),
               N.ptr(cur["sid"]), N.ptr(cur["uid"]), self.n, N.ptr(t_row0), N.ptr(t_rows), self.S, N.ptr(out[0]),
               N.ptr(out[1]), N.ptr(out[2]), 1, st)
        if (wrow0 >= 0).any():
            N.call("sph_arena_extract_many", None, None, None, N.ptr(self.ws_w["sid"]), None, self.WC, N.ptr(t_wrow0),
                   N.ptr(t_rows), self.S, None, None, None, 1, st)
            self._walls_dirty = True
        for sl in slots:
            d = self.slots.pop(sl)
            self._cell_end = None
            self.walls_n -= d["nb"]
            self.live_n -= d["n"]
            bisect.insort(self.free_slots, sl)
        self._specs = None
        return rows, out

    def step(self):
        self._walls_ready()
        self._set_extent(self._extent_for(self.occupied), self._cell_extent())   # shrinks after retirements
        if self.graph is None and self._graphs:
            self._capture_extent()     # a new extent of an arena already captured once
        super().step()
        self.occupied = self.live_n    # the sort moved every free slot behind the live scenes

    def capture(self):
        self._walls_ready()
        self._set_extent(self._extent_for(self.occupied), self._cell_extent())
        super().capture()              # one step run eagerly, then the graphs recorded
        self._graphs[(self.n, self.cap)] = self.graph
        self.occupied = self.live_n

    def escaped(self):
        """Per live slot, how many of its particles were outside its grid at the last sort."""
        cs = self.cell_start.long()
        return {slot: int(cs[d["coff"] + d["ncells"]] - cs[d["coff"] + d["ncells"] - 1])
                for slot, d in self.slots.items()}

    def launches_per_step(self):
        return 1 + 4 + 1 + 1 + 1 + (1 if self.any_renorm else 0)


def estimate_bytes(scene, pairs: str = "cells") -> int:
    """Device bytes one scene needs in a batch: state x2, sort, force records and segment lists,
    and with pairs = "csr" the CSR list at ~30 pairs/particle."""
    n = len(scene["pos"])
    nb = len(scene.get("wall_pos", ()))
    csr = 8 + 30 * 4 * 1.3 if pairs == "csr" else 0
    return int(n * (2 * 36 + 32 + 68 + csr) + nb * 60 + 4096)


# ----------------------------------------------------------------------------- continuous batching
def _timing_event():
    return torch.cuda.Event(enable_timing=True)


class _PinnedPool:
    """Pinned host memory handed out as views of large chunks: one page-locking allocation per
    chunk instead of one per array (page-locking costs far more than the copy it enables).  A
    chunk stays allocated while any view of it is alive."""

    def __init__(self, chunk_bytes: int = 1 << 26):
        self.chunk = int(chunk_bytes)
        self.cur = None
        self.off = 0

    def take(self, shape, dtype):
        nbytes = int(np.prod(shape)) * torch.empty(0, dtype=dtype).element_size()
        step = (nbytes + 255) & ~255
        if self.cur is None or self.off + step > self.cur.numel():
            self.cur = torch.empty(max(self.chunk, step), dtype=torch.uint8, pin_memory=True)
            self.off = 0
        v = self.cur[self.off:self.off + nbytes].view(dtype).view(tuple(shape))
        self.off += step
        return v


@dataclass
class Request:
    rid: int
    arrival: float           # seconds from the start of the trace
    spec: SceneSpec
    admitted: float = -1.0
    finished: float = -1.0
    steps_done: int = 0
    final: dict | None = None
    escaped: int = 0            # particles outside the scene's grid at its last step
    error: str | None = None    # set when the request was retired without completing
    slot: int = -1              # its slot in the server's arena while live (pooled serving)


class Server:
    """Continuous batching: admit arrived requests while the memory budget allows, step all
    live scenes together, retire each scene exactly when it reaches its step count (its
    final state is kept in `Request.final`).  Membership changes rebuild the batch (and its
    CUDA graph) between steps; new arrivals wait at most `rebuild_every` batch steps.

    The batch status word is read after every step.  A step whose neighbor list overflowed
    was not applied by the device: the batch is rebuilt with a fresh pair count (and more
    headroom) and the step runs again.  A scene whose state became non-finite is retired
    with `Request.error` set; the other scenes, which share no data with it, carry on."""

    def __init__(self, device=None, budget_bytes: float = 60e9, rebuild_every: int = 20, use_graph: bool = True,
                 keep_final: bool = True, pair_headroom: float = 1.3, pairs: str = "cells", tuning=None,
                 pooled: bool = True):
        self.device = torch.device(device or torch.device("cuda", torch.cuda.current_device()))
        self.budget = budget_bytes
        self.rebuild_every = rebuild_every
        self.use_graph = use_graph
        self.keep_final = keep_final
        self.pair_headroom = pair_headroom
        self.pairs = pairs
        self.tuning = tuning          # tune.Tuning: per-scene cell ratio and lanes by size
        self.live: list[Request] = []
        self.batch: SceneBatch | None = None
        self.particle_steps = 0
        self.batch_steps = 0
        self.rebuilds = 0
        self.pair_overflows = 0
        self.failed: list[Request] = []
        self.step_latency = []      # (batch step seconds, live scenes) per batch step
        self.rebuild_seconds = 0.0
        self._flags = torch.zeros(1, dtype=torch.int32, pin_memory=True)
        self._last_flags = 0
        # pooled: the scenes live in a SceneArena (admission and retirement write free slots, the
        # CUDA graph is captured again only when the arena grows); else the batch is rebuilt
        self.pooled = pooled and pairs == "cells" and use_graph
        self.arena: SceneArena | None = None
        self.arena_grows = 0

    def _read_flags(self) -> int:
        """Wait for the batch's work and read its status word (4 bytes over a pinned buffer)."""
        self._flags.copy_(self.batch.status, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        self._last_flags = int(self._flags[0])
        return self._last_flags

    def _rebuild(self, queue, now):
        t = time.perf_counter()
        states, keep = [], []
        if self.batch is not None:
            nonfinite = bool(self._read_flags() & N.SPH_FLAG_NONFINITE)
            escaped = self.batch.escaped()
            all_states = self.batch.states_device()
            # final states to the host: one copy per field of the whole batch when the retiring
            # requests hold a large part of it (many small copies cost more), else per request
            host_states = None
            retiring = sum(len(r.spec.scene["pos"]) for r in self.live if r.steps_done >= r.spec.steps)
            if self.keep_final and retiring * 4 >= self.batch.n:
                host_states = {k: v.cpu().numpy() for k, v in all_states.items()}
            for s, r in enumerate(self.live):
                r.escaped = int(escaped[s])
                if nonfinite and not self.batch.scene_finite(s):
                    r.error = "non-finite state"
                    r.finished = now
                    r.spec.dev = None
                    self.failed.append(r)
                    continue
                st = self.batch.scene_state_device(s, all_states)
                if r.steps_done >= r.spec.steps:
                    r.finished = now
                    if self.keep_final and host_states is not None:
                        k0 = self.batch.p_off[self.batch._slot[s]]
                        k1 = self.batch.p_off[self.batch._slot[s] + 1]
                        r.final = {k: v[k0:k1].copy() for k, v in host_states.items()}
                    elif self.keep_final:
                        r.final = {k: v.cpu().numpy() for k, v in st.items()}
                    r.spec.dev = None          # release the scene's device copies
                else:
                    keep.append(r)
                    states.append(st)
        used = sum(estimate_bytes(r.spec.scene, self.pairs) for r in keep)
        while queue and queue[0].arrival <= now:
            need = estimate_bytes(queue[0].spec.scene, self.pairs)
            if used + need > self.budget and keep:
                break
            r = queue.pop(0)
            r.admitted = now
            keep.append(r)
            states.append(None)
            used += need
        self.live = keep
        self.batch = None
        self._last_flags = 0
        if keep:
            self.batch = SceneBatch([r.spec for r in keep], self.device, states=states,
                                    pair_headroom=self.pair_headroom, pairs=self.pairs, tuning=self.tuning)
            self.rebuilds += 1
            if self.use_graph:
                self.batch.capture()          # runs one step eagerly, then records it
                self._after_step(0.0, self._read_flags())
        self.rebuild_seconds += time.perf_counter() - t

    def _after_step(self, seconds, flags) -> bool:
        """Book one batch step; False if the device did not apply it (neighbor list overflow)."""
        if flags & N.SPH_FLAG_PAIR_CAPACITY:
            self.pair_overflows += 1
            self.pair_headroom *= 1.5
            return False
        for r in self.live:
            r.steps_done += 1
        self.particle_steps += self.batch.n
        self.batch_steps += 1
        if seconds > 0:
            self.step_latency.append((seconds, len(self.live)))
        return True

    def _must_rebuild(self) -> bool:
        f = self._last_flags
        return bool(f & (N.SPH_FLAG_PAIR_CAPACITY | N.SPH_FLAG_NONFINITE)) or \
            any(r.steps_done >= r.spec.steps for r in self.live)

    # ------------------------------------------------------------------ pooled serving
    def _arena_kind(self, specs):
        schemes = {DIFFUSION[sp.cfg.density_diffusion] for sp in specs}
        return schemes.pop() if len(schemes) == 1 else -1

    def _grow(self, need_specs, queue=()):
        """A larger arena holding the live scenes (their states carried over) and room for
        `need_specs`; the one place the batch is rebuilt and its graph captured again.  It is
        sized at 1.5x the need for the arrivals still to come, but no larger than what the
        requests still queued could add: every slot costs sort work each step, used or not."""
        t = time.perf_counter()
        live_specs = [r.spec for r in self.live]
        allsp = live_specs + list(need_specs)
        n = sum(len(sp.scene["pos"]) for sp in allsp)
        nb = sum(len(sp.scene.get("wall_pos", ())) for sp in allsp)
        cells = sum(sp.dev["grid"].num_cells + 1 for sp in allsp)
        # a queued scene's cells are unknown before its upload: bounded by its particles over
        # the fewest particles per cell among the scenes at hand, plus its outside slot
        ppc = min(len(sp.scene["pos"]) / max(sp.dev["grid"].num_cells, 1) for sp in allsp)
        more = {"n": sum(len(r.spec.scene["pos"]) for r in queue),
                "nb": sum(len(r.spec.scene.get("wall_pos", ())) for r in queue),
                "c": sum(int(len(r.spec.scene["pos"]) / max(ppc, 1e-3)) + 1 for r in queue)}
        old = self.arena
        grow = lambda need, cur, lo, key: max(lo, min(int(need * 1.5), need + more[key]), cur)
        new = SceneArena(self.device, particles=grow(n, old.N if old else 0, 1 << 16, "n"),
                         walls=grow(nb, old.WC if old else 0, 1 << 12, "nb"),
                         cells=grow(cells, old.C if old else 0, 1 << 16, "c"),
                         slots=max(256, 2 * len(allsp), old.S if old else 0), tpp=self._tpp,
                         scheme=self._scheme)
        for r in self.live:
            st = old.retire(r.slot)
            r.slot = new.admit(r.spec, state=st)
        self.arena = new
        self.arena_grows += 1
        self.rebuilds += 1
        self.rebuild_seconds += time.perf_counter() - t

    def _admit_pooled(self, queue, now):
        """Admit the requests staged one step ago, then stage the ones that have arrived: their
        upload and grid launch are queued now and finished at the next step, so the host
        never waits for the step in flight."""
        t = time.perf_counter()
        admitted_any = False
        staged, self._staged = self._staged, []
        for pending, reqs in staged:
            if pending is not None:
                pending.finish()
            self._admit_staged(reqs, queue, now)
            admitted_any = True
        arrived = []
        used = self._used_bytes
        while queue and queue[0].arrival <= now:
            need = estimate_bytes(queue[0].spec.scene, self.pairs)
            if used + need > self.budget and (self.live or arrived or staged):
                break
            arrived.append(queue.pop(0))
            used += need
        if arrived:
            for r in arrived:
                if self.tuning is not None:
                    self.tuning.configure(r.spec)
                r.spec.tpp = self._tpp
            self._used_bytes = used
            # one upload and grid launch for all of them, finished at the next step
            self._staged.append((upload_scenes([r.spec for r in arrived], self.device, wait=False), arrived))
        self.admit_seconds += time.perf_counter() - t
        return admitted_any

    def _admit_staged(self, arrived, queue, now):
        def admitted(r, slot):
            r.slot = slot
            r.admitted = now
            self.live.append(r)

        # all behind the occupied slots at once when they fit, else one by one (gaps, packing)
        # and a larger arena when those run out
        slots = self.arena.admit_many([r.spec for r in arrived]) if self.arena is not None else None
        if slots is not None:
            for r, slot in zip(arrived, slots):
                admitted(r, slot)
            return
        for k, r in enumerate(arrived):
            try:
                if self.arena is None:
                    raise ArenaFull("no arena yet")
                admitted(r, self.arena.admit(r.spec))
            except ArenaFull:
                self._grow([q.spec for q in arrived[k:]], queue)   # moves the live scenes over
                rest = arrived[k:]
                slots = self.arena.admit_many([q.spec for q in rest])
                if slots is None:
                    slots = [self.arena.admit(q.spec) for q in rest]
                for q, slot in zip(rest, slots):
                    admitted(q, slot)
                return

    def _retire_pooled_many(self, reqs, now):
        """The requests that completed this step, retired together (one extract pass; with
        keep_final one pinned block and one copy per field for all their final states)."""
        rows, out = self.arena.retire_many([r.slot for r in reqs])
        host = None
        if self.keep_final:
            host = [self._pinned.take(t.shape, t.dtype) for t in out]
            for h, t in zip(host, out):
                h.copy_(t, non_blocking=True)
        for r in reqs:
            self._used_bytes -= estimate_bytes(r.spec.scene, self.pairs)
            r.finished = now
            if host is not None:
                a, n = rows[r.slot]
                r.final = {"x": host[0][a:a + n], "v": host[1][a:a + n], "rho": host[2][a:a + n]}
            r.spec.dev = None
        gone = {id(r) for r in reqs}
        self.live = [r for r in self.live if id(r) not in gone]

    def _retire_pooled(self, r, now, error=None):
        st = self.arena.retire(r.slot)
        self._used_bytes -= estimate_bytes(r.spec.scene, self.pairs)
        r.finished = now
        if error:
            r.error = error
            self.failed.append(r)
        elif self.keep_final:
            host = {k: self._pinned.take(v.shape, v.dtype) for k, v in st.items()}
            for k in st:
                host[k].copy_(st[k], non_blocking=True)
            r.final = host                     # numpy after the run's last synchronisation
        r.spec.dev = None
        self.live.remove(r)

    def _run_pooled(self, queue, t0, max_wall):
        self._scheme = self._arena_kind([r.spec for r in queue])
        self._tpp = 1
        self.admit_seconds = 0.0
        self._pinned = _PinnedPool()
        self._used_bytes = 0
        self._staged = []             # (pending upload, requests) admitted at the next step
        flags = torch.zeros(2, dtype=torch.int32, pin_memory=True)
        done = [None, None]          # event after each of the last two steps' status copies
        timed = []                   # (start event, end event, live scenes) per step
        k = 0
        while queue or self.live or self._staged:
            now = time.perf_counter() - t0
            if now > max_wall:
                break
            e0 = _timing_event()
            e0.record()
            self._admit_pooled(queue, now)
            if not self.live:
                if queue and not self._staged:
                    time.sleep(max(0.0, min(queue[0].arrival - (time.perf_counter() - t0), 0.01)))
                continue
            a = self.arena
            if a.graph is None:
                a.capture()          # runs one step eagerly, then records the step's graphs
            else:
                a.step()
            # the status word of this step to pinned memory, then cleared for the next one
            flags[k % 2:k % 2 + 1].copy_(a.status, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            a.status.zero_()
            e1 = _timing_event()
            e1.record()
            timed.append((e0, e1, len(self.live)))
            done[k % 2] = ev
            n_live = a.live_n
            for r in list(self.live):
                r.steps_done += 1
            self.particle_steps += n_live
            self.batch_steps += 1
            now = time.perf_counter() - t0
            finished = [r for r in self.live if r.steps_done >= r.spec.steps]
            if finished:
                self._retire_pooled_many(finished, now)
            # the previous step's status (its work is done once this step has been queued)
            prev = done[(k - 1) % 2] if k else None
            if prev is not None:
                prev.synchronize()
                f = int(flags[(k - 1) % 2])
                self._last_flags = f
                if f & N.SPH_FLAG_NONFINITE:
                    torch.cuda.synchronize()
                    for r in list(self.live):
                        if not a.scene_finite(r.slot):
                            self._retire_pooled(r, time.perf_counter() - t0, error="non-finite state")
            k += 1
        torch.cuda.synchronize()
        for r in self.requests_all:
            if isinstance(r.final, dict) and r.final and isinstance(next(iter(r.final.values())), torch.Tensor):
                r.final = {kk: v.numpy() for kk, v in r.final.items()}
        for e0, e1, nl in timed:
            self.step_latency.append((e0.elapsed_time(e1) / 1e3, nl))
        if self.arena is not None:
            self.arena.check()
        return time.perf_counter() - t0

    def run(self, requests, time_scale: float = 1.0, max_wall: float = 600.0):
        """Serve `requests` (arrival times scaled by time_scale); returns the wall seconds."""
        queue = sorted(requests, key=lambda r: r.arrival)
        for r in queue:
            r.arrival *= time_scale
        t0 = time.perf_counter()
        if self.pooled:
            self.requests_all = list(queue)
            return self._run_pooled(queue, t0, max_wall)
        since = 0
        while queue or self.live:
            now = time.perf_counter() - t0
            if now > max_wall:
                break
            arrived = bool(queue) and queue[0].arrival <= now
            if self.batch is None or self._must_rebuild() or (arrived and since >= self.rebuild_every):
                self._rebuild(queue, now)
                since = 0
                if self.batch is None:
                    if queue:
                        time.sleep(max(0.0, min(queue[0].arrival - (time.perf_counter() - t0), 0.01)))
                    continue
                if self._must_rebuild():
                    continue
            t = time.perf_counter()
            self.batch.step()
            flags = self._read_flags()          # waits for the step
            since += self._after_step(time.perf_counter() - t, flags)
        if self.batch is not None:
            self.batch.check()
        return time.perf_counter() - t0

    def latency_percentiles(self, qs=(50, 99)):
        """Per-scene step latency percentiles (each batch step counts once per live scene)."""
        if not self.step_latency:
            return {q: None for q in qs}
        sec = np.array([s for s, _ in self.step_latency])
        w = np.array([k for _, k in self.step_latency], np.float64)
        o = np.argsort(sec)
        cw = np.cumsum(w[o]) / w.sum()
        return {q: float(sec[o][min(np.searchsorted(cw, q / 100.0), len(o) - 1)]) for q in qs}
