"""Autotuning of the GB300 path per scene-size bucket, by measurement on the device.

Knobs:
  * serving batch (per scene, `SceneSpec.cell_ratio` / `SceneSpec.tpp`): the cell size as
    a fraction of the support (cells of h / cell_ratio searched cell_ratio cells out: fewer
    candidates per particle, more segments), and the lanes per particle of the force
    passes (1, 2 or 4: a particle's segments split over the lanes, sums added by warp
    shuffles).  A scene's configuration depends only on its particle count, so a scene's
    result is the same alone and in any mix of scenes.
  * one-scene neighbor search (`GridSearch`): counting sort, or LSD radix sort and its
    digit width, and the cell size (cells of h or of h / 2; the same pair set either way).

A bucket is floor(log2 N).  `Autotuner.tune_serving` times, for each bucket's size, a
loaded batch (about `batch_particles` particles of scenes of that size, half dam breaks,
half drops) under every candidate and keeps the fastest; `tune_search` times
`GridSearch.run` likewise.  The resulting `Tuning` is plain data: it saves to and loads
from JSON, and configures specs (`SceneBatch(..., tuning=t)`, `Server(..., tuning=t)`).
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field

import numpy as np
import torch

SERVING_CANDIDATES = ((1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4))   # (cell_ratio, tpp)
SEARCH_CANDIDATES = (("counting", 0, 1), ("counting", 0, 2), ("radix", 4, 1), ("radix", 6, 1), ("radix", 8, 1),
                     ("radix", 8, 2))   # (sort, digit bits, cell ratio)


def bucket(n: int) -> int:
    return int(math.floor(math.log2(max(int(n), 1))))


def _nearest(table: dict, n: int):
    if not table:
        return None
    b = bucket(n)
    keys = sorted(table)
    return table[min(keys, key=lambda k: (abs(k - b), k))]


@dataclass
class Tuning:
    """Chosen configuration per size bucket (and what each candidate measured)."""
    serving: dict = field(default_factory=dict)   # bucket -> {"cell_ratio", "tpp", "measured": {...}}
    search: dict = field(default_factory=dict)    # bucket -> {"sort", "digit_bits", "cell_ratio", "measured"}
    device: str = ""

    def scene_config(self, n: int) -> dict:
        e = _nearest(self.serving, n)
        return {"cell_ratio": 1, "tpp": 1} if e is None else {"cell_ratio": e["cell_ratio"], "tpp": e["tpp"]}

    def configure(self, spec) -> None:
        """Set a SceneSpec's cell_ratio and tpp from its particle count."""
        c = self.scene_config(len(spec.scene["pos"]))
        spec.cell_ratio, spec.tpp = c["cell_ratio"], c["tpp"]

    def search_config(self, n: int) -> dict:
        e = _nearest(self.search, n)
        if e is None:
            return {"sort": "counting", "digit_bits": 8, "cell_ratio": 1}
        return {"sort": e["sort"], "digit_bits": e["digit_bits"], "cell_ratio": int(e.get("cell_ratio", 1))}

    def to_json(self) -> dict:
        return {"device": self.device, "serving": {str(k): v for k, v in self.serving.items()},
                "search": {str(k): v for k, v in self.search.items()}}

    @classmethod
    def from_json(cls, d: dict) -> "Tuning":
        return cls({int(k): v for k, v in d.get("serving", {}).items()},
                   {int(k): v for k, v in d.get("search", {}).items()}, d.get("device", ""))

    def save(self, path: str) -> None:
        with open(path, "w") as f:
            json.dump(self.to_json(), f, indent=1)

    @classmethod
    def load(cls, path: str) -> "Tuning":
        with open(path) as f:
            return cls.from_json(json.load(f))


def _time_steps(batch, steps: int) -> float:
    """Milliseconds per step of a captured batch (CUDA events, after warm-up)."""
    batch.capture()
    for _ in range(3):
        batch.step()
    st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    st.record()
    for _ in range(steps):
        batch.step()
    en.record()
    torch.cuda.synchronize()
    return st.elapsed_time(en) / steps


class Autotuner:
    def __init__(self, device=None):
        self.device = torch.device(device or torch.device("cuda", torch.cuda.current_device()))

    def _specs(self, size: int, count: int, steps: int):
        from . import workloads
        from .serve import SceneSpec
        from .sim import SimConfig
        specs = []
        for k in range(count):
            kind = "dam_break" if k % 2 == 0 else "drop"
            shape = 0.5 + 1.5 * ((k * 0.618034) % 1.0)
            sc, p = workloads.make_request_scene({"kind": kind, "n": size, "shape": shape})
            cfg = SimConfig(solver="deltaSPH", integration="semiImplicitEuler", dt=p["dt"], c0=p["c0"],
                            gravity=p["gravity"], point_source=p["point_source"], density_diffusion=p["diffusion"])
            specs.append(SceneSpec(sc, cfg, steps))
        return specs

    def tune_serving(self, sizes=(2048, 8192, 32768, 131072), batch_particles: int = 1 << 20, steps: int = 10,
                     candidates=SERVING_CANDIDATES) -> dict:
        """bucket -> the fastest (cell_ratio, tpp) for a loaded batch of scenes of that size."""
        from .serve import SceneBatch
        out = {}
        for size in sizes:
            count = max(1, batch_particles // size)
            specs = self._specs(size, count, steps)
            n = sum(len(s.scene["pos"]) for s in specs)
            measured = {}
            for ratio, tpp in candidates:
                for s in specs:
                    s.cell_ratio, s.tpp = ratio, tpp
                b = SceneBatch(specs, self.device)
                ms = _time_steps(b, steps)
                b.check()
                measured[f"{ratio},{tpp}"] = {"ms_per_step": ms, "particle_steps_per_s": n / (ms / 1e3)}
                del b
            best = min(measured, key=lambda k: measured[k]["ms_per_step"])
            r, t = (int(v) for v in best.split(","))
            out[bucket(size)] = {"size": size, "scenes": count, "cell_ratio": r, "tpp": t, "measured": measured}
            for s in specs:
                s.dev = None
            torch.cuda.empty_cache()
        return out

    def tune_search(self, sizes=(1 << 16, 1 << 18, 1 << 20), steps: int = 5, candidates=SEARCH_CANDIDATES,
                    data=None) -> dict:
        """bucket -> the fastest configuration of GridSearch.run (+ density) on a jittered
        lattice of each size, or on `data` = (pos, support, area, run keywords) when given
        (the caller's own particles: one bucket)."""
        from .search import GridSearch
        out = {}
        for size in (sizes if data is None else (int(data[0].shape[0]),)):
            if data is None:
                side = int(round(math.sqrt(size)))
                dx = 1.0 / side
                g = torch.Generator().manual_seed(0)
                ij = torch.stack(torch.meshgrid(torch.arange(side), torch.arange(side), indexing="ij"),
                                 -1).reshape(-1, 2)
                pos = ((ij.float() + 0.5) * dx + (torch.rand(ij.shape, generator=g) - 0.5) * 0.2 * dx).to(self.device)
                h = torch.full((pos.shape[0],), 3 * dx, dtype=torch.float32, device=self.device)
                area = torch.full_like(h, dx * dx)
                kw = dict(kernel_support=3 * dx, min_coord=(0.0, 0.0), max_coord=(1.0, 1.0))
            else:
                pos, h, area, kw = data
            measured = {}
            for sort, bits, ratio in candidates:
                gs = GridSearch(self.device, sort=sort, digit_bits=bits or 8, cell_ratio=ratio)
                res = gs.run(pos, h, area, **kw)
                cap, pcap = res.cell_capacity, int(res.num_pairs * 1.05) + 1024
                for _ in range(2):
                    gs.run(pos, h, area, cell_capacity=cap, pair_capacity=pcap, sync=False, **kw)
                st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                st.record()
                for _ in range(steps):
                    gs.run(pos, h, area, cell_capacity=cap, pair_capacity=pcap, sync=False, **kw)
                en.record()
                torch.cuda.synchronize()
                ms = st.elapsed_time(en) / steps
                measured[f"{sort},{bits},{ratio}"] = {"ms": ms, "particles_per_s": pos.shape[0] / (ms / 1e3)}
            best = min(measured, key=lambda k: measured[k]["ms"])
            sort, bits, ratio = best.split(",")
            out[bucket(size)] = {"size": int(pos.shape[0]), "sort": sort, "digit_bits": int(bits) or 8,
                                 "cell_ratio": int(ratio), "measured": measured}
        return out

    def tune(self, serving_sizes=(2048, 8192, 32768, 131072), search_sizes=(1 << 16, 1 << 18, 1 << 20),
             batch_particles: int = 1 << 20, steps: int = 10) -> Tuning:
        t = Tuning(device=torch.cuda.get_device_name(self.device))
        if serving_sizes:
            t.serving = self.tune_serving(serving_sizes, batch_particles, steps)
        if search_sizes:
            t.search = self.tune_search(search_sizes)
        return t
