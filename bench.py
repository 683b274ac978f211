"""Benchmarks of the GB300 SPH hot path; rank 0 prints one JSON line.

Workloads (--workload):
  serving (default)   1024 deltaSPH scene requests (Poisson arrivals at 50/s, 2,048-131,072
                      particles log-uniform, half random-aspect dam breaks, half oscillating
                      drops, 1000 steps each, 60 GB budget), served by continuous batching.
                      value = particle-steps/s of the device-resident batch of all requests
                      (K timed batch steps); e2e = the whole trace through the Server (scene
                      upload, admission, batch rebuilds, final states read back) with every
                      request queued at t=0; `serving` adds the real-time trace's p50/p99
                      step latency and time-to-completion and the one-scene-at-a-time GPU path.
                      First the autotuner measures each scene-size bucket's cell ratio and
                      lanes per particle (`tuning`; --no-tune: cells of h, one lane).
  search_density_A/B  neighbor search + density over N = 2^20 particles (sort: the
                      autotuner's pick for N unless --sort counting|radix).
  dambreak_deltasph   8,192-particle dam break, renormalized deltaSPH, 3-layer walls.
  dambreak_dfsph      262,144-particle dam break, DFSPH with walls, adaptive dt.
  diff_drop           16,384-particle oscillating drop, 200 float64 steps: forward + adjoint
                      (gradients w.r.t. v0 and alpha) checked against finite differences.

  python bench.py [--workload W] [--steps K] [--warmup W]
  python bench.py --impl reference ...   # the reference algorithm on the host cores

With torchrun (N>1) every rank runs an independent replica (no exchange step exists on
this path) and `value` sums over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="serving")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sort", default="auto", choices=["auto", "counting", "radix"],
                    help="search workloads: auto = the autotuner's pick for this N")
    ap.add_argument("--digit-bits", type=int, default=8)
    ap.add_argument("--cell-ratio", type=int, default=1,
                    help="search workloads with --sort counting|radix: grid cells of h / cell_ratio")
    ap.add_argument("--requests", type=int, default=1024)
    ap.add_argument("--trace-steps", type=int, default=1000)
    ap.add_argument("--no-trace", action="store_true", help="serving: skip the e2e and real-time trace runs")
    ap.add_argument("--no-tune", action="store_true",
                    help="serving: one lane per particle and cells of h for every scene instead of the autotuner's picks")
    ap.add_argument("--pairs", default="cells", choices=["cells", "csr"],
                    help="serving: pairs from the cell rows, or a CSR neighbor list built every step")
    return ap.parse_args()


# ----------------------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([s.strip() for s in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        num = lambda s: s.replace(".", "", 1).isdigit()
        sm = [float(s[1]) for s in self.samples if num(s[1])]
        mx = [float(s[2]) for s in self.samples if num(s[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 5 + k and s[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def sync_ranks(world):
    """Device synchronisation and, with several ranks, a barrier: brackets every timed region."""
    import torch
    import torch.distributed as dist
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()


def max_over_ranks(x, world):
    """The maximum of x over all ranks (the slowest replica sets the whole job's time)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def hbm_peak():
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(p["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


def make_event():
    import torch
    try:  # an event recorded inside a captured graph becomes a timed node only when external
        return torch.cuda.Event(enable_timing=True, external=True)
    except TypeError:
        return torch.cuda.Event(enable_timing=True)


def traffic_from_profiles(workload, kernel, units):
    """DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) of one launch of `kernel`
    scaled to `units` particles: profiles/traffic.json holds the bytes per particle of a
    smaller captured case of the same kernel (its traffic grows in proportion to the
    particles processed)."""
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        e = prof[workload][kernel]
        return e["dram_bytes"] / e["particles"] * units
    except Exception:
        return None


def base_line(args, world, value, ms, unit, config):
    # the solver workloads report the serving metric (particle-steps/s); the search
    # workloads count particles searched (with density) per second
    return {"metric": METRIC if unit == METRIC else unit, "value": value, "unit": unit, "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config}


# ----------------------------------------------------------------------------- CPU (oracle port) arms
def cpu_search_density(pos, h, area, vmin, vmax, L, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import nsearch as ns
    si = ns.SortInfo(pos, h, vmin, vmax, L)
    rows, cols = ns.nl_cells(si, threads=threads)
    off, c = ns.canonical_csr(rows, cols, si.n)
    ns.density(off, c, pos, area, float(h[0]))
    return len(rows)


def cpu_deltasph_steps(scene, params, steps, diffusion="MOG"):
    """Seconds for `steps` of the restated reference step (oracle/sph_torch.py, float32, torch CPU)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch
    import sph_torch as S
    p = S.Params(h=scene["h"], c0=params["c0"], diffusion=diffusion, vmin=scene["vmin"], vmax=scene["vmax"],
                 gravity=params.get("gravity", (0.0, -9.81)), point_source=params.get("point_source", False))
    walls = S.Walls(torch.from_numpy(scene["wall_pos"]), torch.from_numpy(scene["ghost_pos"]),
                    torch.from_numpy(scene["wall_area"])) if len(scene["wall_pos"]) else None
    st = {"x": torch.from_numpy(scene["pos"]), "v": torch.from_numpy(scene["vel"]),
          "rho": torch.from_numpy(scene["rho"]), "area": torch.from_numpy(scene["area"])}
    t0 = time.perf_counter()
    for _ in range(steps):
        new, _ = S.step(st, walls, p, params["dt"], "semiImplicitEuler", "deltaSPH", torch.float32)
        st = {"x": new["x"].float(), "v": new["v"], "rho": new["rho"], "area": st["area"]}
    return time.perf_counter() - t0


def cpu_baseline_serving(n_requests=1024, steps=2, sizes=(2048, 16384, 131072)):
    """The restated reference step (oracle/sph_torch.py, float32, torch CPU, every host thread)
    timed on requests spanning the trace's sizes, for both scene kinds (dam break with walls,
    drop without), then a log-log fit of seconds per step against particle count per kind,
    applied to every request of the trace: the CPU's particle-steps/s on the trace's own size
    and kind mix, and its milliseconds to advance every request by one step."""
    import torch
    from pytorchsph_gb300 import workloads
    meas = {}
    for kind in ("dam_break", "drop"):
        pts = []
        for n in sizes:
            sc, p = workloads.make_request_scene({"kind": kind, "n": n, "shape": 1.0})
            cpu_deltasph_steps(sc, p, 1, p["diffusion"])
            t = cpu_deltasph_steps(sc, p, steps, p["diffusion"]) / steps
            pts.append((len(sc["pos"]), t))
        meas[kind] = pts
    fit = {}
    for kind, pts in meas.items():
        ln = np.log([q[0] for q in pts])
        lt = np.log([q[1] for q in pts])
        fit[kind] = np.polyfit(ln, lt, 1)
    trace = workloads.serving_trace(n_requests, 50.0, 2048, 131072, 1, seed=0)
    tot_n = float(sum(r["n"] for r in trace))
    tot_s = float(sum(np.exp(np.polyval(fit[r["kind"]], np.log(r["n"]))) for r in trace))
    samples = "; ".join(f"{k}: " + ", ".join(f"{n} particles {1e3 * t:.1f} ms" for n, t in v) for k, v in meas.items())
    return {"value": tot_n / tot_s, "unit": "particle-steps/s", "cores": torch.get_num_threads(), "kind": "port",
            "ms_per_trace_step": 1e3 * tot_s,
            "sample": f"{steps} semi-implicit-Euler deltaSPH steps (restated reference step, float32, torch CPU) "
                      f"of requests of {', '.join(str(n) for n in sizes)} particles per scene kind ({samples}); "
                      f"seconds per step fitted log-log in the particle count per kind and summed over the "
                      f"{n_requests}-request trace"}


def cpu_dfsph_steps(scene, steps):
    """Seconds for `steps` DFSPH steps of the restated reference step (oracle/sph_torch.py,
    float32, torch CPU, solid walls, the bench's solver settings and adaptive dt)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch
    import sph_torch as S
    p = S.Params(h=scene["h"], c0=float(10 * np.sqrt(2 * 9.81 * scene["column_height"])), kinematic=0.01,
                 vmin=scene["vmin"], vmax=scene["vmax"], density_threshold=1e-4, divergence_threshold=1e-3,
                 max_density_iters=100, max_divergence_iters=100)
    walls = S.Walls(torch.from_numpy(scene["wall_pos"]), torch.from_numpy(scene["ghost_pos"]),
                    torch.from_numpy(scene["wall_area"]))
    walls.density_term = S.wall_density_term(walls, scene["h"], torch.float32)
    st = {"x": torch.from_numpy(scene["pos"]), "v": torch.from_numpy(scene["vel"]),
          "rho": torch.from_numpy(scene["rho"]), "area": torch.from_numpy(scene["area"])}
    dt = 2e-4
    t0 = time.perf_counter()
    for _ in range(steps):
        new, _ = S.step(st, walls, p, dt, "semiImplicitEuler", "dfsph", torch.float32)
        st = {"x": new["x"].float(), "v": new["v"], "rho": new["rho"], "area": st["area"]}
        dt = S.update_dt(new, p, dt, 1e-6, 1e-3)
    return time.perf_counter() - t0


def served_accuracy(spec, req, final):
    """Relative density error (max and mean over particles) and position error (max, in
    supports) of a served request's final state against the float64 restated reference step
    (oracle/sph_torch.py) run for the request's steps on the host."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch
    import sph_torch as S
    from pytorchsph_gb300 import workloads
    sc, p = workloads.make_request_scene(req)
    P = S.Params(h=sc["h"], c0=p["c0"], diffusion=p["diffusion"], vmin=sc["vmin"], vmax=sc["vmax"],
                 gravity=p["gravity"], point_source=p["point_source"])
    walls = S.Walls(torch.from_numpy(sc["wall_pos"]), torch.from_numpy(sc["ghost_pos"]),
                    torch.from_numpy(sc["wall_area"]))
    st = {"x": torch.from_numpy(sc["pos"]), "v": torch.from_numpy(sc["vel"]), "rho": torch.from_numpy(sc["rho"]),
          "area": torch.from_numpy(sc["area"])}
    t0 = time.perf_counter()
    for _ in range(spec.steps):
        new, _ = S.step(st, walls, P, p["dt"], "semiImplicitEuler", "deltaSPH", torch.float64)
        st = {"x": new["x"], "v": new["v"], "rho": new["rho"], "area": st["area"]}
    r64 = st["rho"].numpy()
    rel = np.abs(np.asarray(final["rho"], np.float64) - r64) / np.abs(r64)
    return {"particles": len(sc["pos"]), "steps": spec.steps, "rho_rel_err_max": float(rel.max()),
            "rho_rel_err_mean": float(rel.mean()),
            "x_err_max_over_h": float(np.abs(np.asarray(final["x"], np.float64) - st["x"].numpy()).max() / sc["h"]),
            "float64_reference_s": time.perf_counter() - t0}


def serving_workload(args, world):
    """The serving workload's description, the same in both arms."""
    return {"workload": "serving", "requests": args.requests, "trace_steps": args.trace_steps,
            "arrivals": "Poisson 50/s", "sizes": "log-uniform 2048-131072",
            "mix": "50% dam break (aspect U[0.5,2]) / 50% oscillating drop (A U[0.5,2])",
            "solver": "deltaSPH (renormalized density diffusion), semi-implicit Euler, dt = 0.1 h / c0, "
                      "3-layer walls", "parallelism": f"replicas{world}"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if args.workload.startswith("search_density_"):
        from pytorchsph_gb300 import workloads
        pos, h, area, vmin, vmax, L = workloads.search_density_case(args.workload.rsplit("_", 1)[1])
        cpu_search_density(pos[:4096], h[:4096], area[:4096], vmin, vmax, -1, 1)
        for _ in range(args.warmup):
            cpu_search_density(pos, h, area, vmin, vmax, L, threads)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            cpu_search_density(pos, h, area, vmin, vmax, L, threads)
        ms = 1e3 * (time.perf_counter() - t0) / args.steps
        value = len(pos) / (ms / 1e3)
        sample = f"full {args.workload} step x {args.steps} (sort + hash map + buildNeighborList + density)"
        unit, cores = "particles/s", threads
        config = {"workload": args.workload, "particles": len(pos)}
    elif args.workload in ("dambreak_deltasph", "dambreak_dfsph"):
        import torch
        from pytorchsph_gb300 import workloads
        torch.set_num_threads(threads)
        steps = max(1, min(args.steps, 3))
        if args.workload == "dambreak_deltasph":
            sc = workloads.dam_break(64, 128, 0.01, (4.0, 2.0))
            c0 = float(10 * np.sqrt(2 * 9.81 * sc["column_height"]))
            params = {"c0": c0, "dt": 0.25 * sc["h"] / c0}
            cpu_deltasph_steps(sc, params, 1, "deltaSPH")
            t = cpu_deltasph_steps(sc, params, steps, "deltaSPH")
            sample = f"{steps} steps of the same 8192-particle dam break (restated reference step, float32, torch CPU)"
        else:   # the 262,144-particle block takes minutes per CPU step: a 64 x 64 block of the same tank
            sc = workloads.dam_break(64, 64, 0.016, (4.096, 2.048))
            t = cpu_dfsph_steps(sc, steps)
            sample = (f"{steps} DFSPH steps of a {len(sc['pos'])}-particle block of the same tank (restated "
                      f"reference step, float32, torch CPU)")
        value, unit, cores = len(sc["pos"]) * steps / t, "particle-steps/s", torch.get_num_threads()
        ms = 1e3 * t / steps
        config = {"workload": args.workload}
    elif args.workload == "diff_drop":
        import torch
        from pytorchsph_gb300 import workloads
        torch.set_num_threads(threads)
        start = workloads.oscillating_drop(16384, 0.5, 0.8)
        dt, steps = 0.1 * start["h"] / 10.0, max(1, min(args.steps, 3))
        cpu_autograd_drop(start, dt, 1)
        t = cpu_autograd_drop(start, dt, steps)
        value, unit, cores = len(start["pos"]) * steps / t, "particle-steps/s", torch.get_num_threads()
        ms = 1e3 * t / steps
        sample = f"forward + torch autograd backward of {steps} float64 steps of the drop (restated reference step)"
        config = {"workload": "diff_drop"}
    else:
        import torch
        torch.set_num_threads(threads)
        cb = cpu_baseline_serving(args.requests, steps=max(1, min(args.steps, 2)))
        value, unit, sample, cores = cb["value"], cb["unit"], cb["sample"], cb["cores"]
        ms = cb["ms_per_trace_step"]
        config = serving_workload(args, world)
    line = base_line(args, world, value, ms, unit, config)
    line["impl"] = "reference"
    line["cpu_baseline"] = {"value": value, "unit": unit, "cores": cores, "kind": "port", "sample": sample}
    line["e2e"] = {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU: serving
def serving_specs(n_requests, steps):
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.serve import SceneSpec
    from pytorchsph_gb300.sim import SimConfig
    trace = workloads.serving_trace(n_requests, 50.0, 2048, 131072, steps, seed=0)
    specs = []
    for t in trace:
        sc, p = workloads.make_request_scene(t)
        cfg = SimConfig(solver="deltaSPH", integration="semiImplicitEuler", dt=p["dt"], c0=p["c0"],
                        gravity=p["gravity"], point_source=p["point_source"], density_diffusion=p["diffusion"])
        specs.append(SceneSpec(sc, cfg, t["steps"], name=f"r{t['rid']}"))
    return trace, specs


def pass1_alg_bytes(batch):
    """Algorithmic HBM bytes of one k_batch_pass1 launch over renormalized scenes.
    Per particle: its two 16-byte neighbor records (read once; the other 27-odd reads of
    them are L1/L2 hits), relative density 4, key 4, scene index 4 read, dpdt 4 + acc 8 +
    <grad rho> V 8 written.  Pairs from the cell rows: the segment count 4 and 8 per stored
    segment (start, mask) read (68 per particle + 8 per segment).  CSR pairs: offsets 4 (64)
    and 4 per column.  Per wall: position 8 + volume, density, pressure 12."""
    import ctypes
    import torch
    from pytorchsph_gb300 import _native as N
    if batch.pairs == "csr":
        P = int(batch.offsets[batch.n].item())
        return batch.n * 64 + 4 * P + batch.nb * 20
    n = batch.n
    mo, so, co, ms = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int32()
    N.call("sph_deltasph_segment_lists", n, ctypes.byref(mo), ctypes.byref(so), ctypes.byref(co), ctypes.byref(ms))
    # the scratch tensor is 256-byte aligned, so its first 32-byte boundary is its start
    nseg = batch.forces_scratch.view(torch.int32)[co.value // 4:co.value // 4 + n]
    segments = int(torch.clamp(nseg, min=0).sum().item())
    return n * 68 + 8 * segments + batch.nb * 20


def phase_times(batch, reps=5):
    """Mean milliseconds of each phase of one batch step (eager, events between the calls;
    the step is run into scratch outputs so the batch state does not advance)."""
    import torch
    from pytorchsph_gb300 import _native as N
    acc = {}
    out = {"x": torch.empty_like(batch.a["x"]), "v": torch.empty_like(batch.a["v"]),
           "rho": torch.empty_like(batch.a["rho"])}
    names = ["sort+permute", "pair list", "walls+records", "pass1", "diffusion"]
    for _ in range(reps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
        torch.cuda.synchronize()
        e[0].record()
        batch._sort_permute()
        e[1].record()
        batch._pair_list()
        e[2].record()
        for k, mask in enumerate([N.SPH_PHASE_WALLS | N.SPH_PHASE_RECORDS, N.SPH_PHASE_PASS1,
                                  N.SPH_PHASE_DIFFUSION]):
            batch.forces(out, mask)
            e[3 + k].record()
        torch.cuda.synchronize()
        for k, name in enumerate(names):
            acc[name] = acc.get(name, 0.0) + e[k].elapsed_time(e[k + 1]) / reps
    if batch.pairs != "csr":
        del acc["pair list"]
    return acc


def run_serving(args, dev, world, rank):
    import torch
    from pytorchsph_gb300.serve import SceneBatch, Server, Request
    t_gen = time.perf_counter()
    trace, specs = serving_specs(args.requests, args.trace_steps)
    gen_s = time.perf_counter() - t_gen
    total_p = sum(len(s.scene["pos"]) for s in specs)
    budget = 60e9

    # the autotuner's picks per scene-size bucket (cells of h / cell_ratio, lanes per particle),
    # measured here: in a loaded batch of ~2M particles (the resident batch and the request
    # loop) and for a scene stepped alone (the one-scene comparison path)
    tuned, tune_s = {"loaded": None, "one_scene": None}, 0.0
    if not args.no_tune and args.pairs == "cells":
        from pytorchsph_gb300.tune import Autotuner, Tuning
        t0 = time.perf_counter()
        tuner = Autotuner(dev)
        sizes = (2048, 8192, 32768, 131072)
        tuned["loaded"] = Tuning(serving=tuner.tune_serving(sizes, batch_particles=1 << 21, steps=10))
        tuned["one_scene"] = Tuning(serving=tuner.tune_serving(sizes, batch_particles=1, steps=20))
        tune_s = time.perf_counter() - t0
        torch.cuda.empty_cache()

    # (a) device-resident batch of every request: W warm-up + K timed batch steps
    batch = SceneBatch(specs, dev, pairs=args.pairs, tuning=tuned["loaded"])
    batch.capture()
    for _ in range(max(args.warmup, 3)):
        batch.step()
    torch.cuda.synchronize()
    batch.check()
    st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index or 0) as clk:
        sync_ranks(world)
        st.record()
        for _ in range(args.steps):
            batch.step()
        en.record()
        sync_ranks(world)
    ms = max_over_ranks(st.elapsed_time(en) / args.steps, world)
    batch.check()
    value = total_p * world / (ms / 1e3)
    phases = phase_times(batch)
    alg = pass1_alg_bytes(batch)
    peak, peak_src = hbm_peak()
    achieved = alg / (phases["pass1"] / 1e3) / 1e9 if phases.get("pass1") else None
    launches = batch.launches_per_step()
    batch_bytes = batch.device_bytes()
    del batch
    for s in specs:
        s.dev = None
    torch.cuda.empty_cache()

    # (b) one-scene-at-a-time GPU path on 16 requests spread over the sizes
    order = sorted(range(len(specs)), key=lambda k: len(specs[k].scene["pos"]))
    pick = sorted(set(order[int(q * (len(order) - 1))] for q in np.linspace(0, 1, 16)))
    one = []
    for k in pick:
        b1 = SceneBatch([specs[k]], dev, pairs=args.pairs, tuning=tuned["one_scene"])
        b1.capture()
        for _ in range(3):
            b1.step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(20):
            b1.step()
        torch.cuda.synchronize()
        one.append((len(specs[k].scene["pos"]), (time.perf_counter() - t0) / 20))
        del b1
        specs[k].dev = None
    ln = np.log([n for n, _ in one])
    lt = np.log([t for _, t in one])
    t_of = lambda n: float(np.exp(np.interp(np.log(n), ln, lt)))
    one_scene_time = sum(t_of(len(s.scene["pos"])) * s.steps for s in specs)
    total_work = sum(len(s.scene["pos"]) * s.steps for s in specs)
    one_scene_value = total_work / one_scene_time

    e2e, realtime, accuracy = None, None, None
    if not args.no_trace:
        # (c) end to end: every request queued at t = 0, continuous batching to completion
        reqs = [Request(t["rid"], 0.0, specs[k]) for k, t in enumerate(trace)]
        sync_ranks(world)
        srv = Server(dev, budget_bytes=budget, rebuild_every=50, keep_final=True,   # final states to host
                     pairs=args.pairs, tuning=tuned["loaded"])
        wall = srv.run(reqs, time_scale=0.0, max_wall=600)
        sync_ranks(world)
        wall = max_over_ranks(wall, world)
        done = sum(r.steps_done >= r.spec.steps and r.error is None and r.final is not None for r in reqs)
        # accuracy of served results: the smallest dam break and the smallest drop of the trace,
        # as served in the mix, against the float64 restated reference step over their steps
        accuracy = None
        if rank == 0 and not args.no_cpu_baseline:
            accuracy = {}
            for kind in ("dam_break", "drop"):
                cand = [k for k, t in enumerate(trace) if t["kind"] == kind and reqs[k].final is not None]
                if cand:
                    k = min(cand, key=lambda q: len(specs[q].scene["pos"]))
                    accuracy[kind] = served_accuracy(specs[k], trace[k], reqs[k].final)
        for r in reqs:
            r.final = None
        h2d = sum(s.scene["pos"].nbytes * 2 + s.scene["rho"].nbytes * 3 + s.scene["wall_pos"].nbytes * 2 +
                  s.scene["wall_area"].nbytes for s in specs)
        d2h = sum(s.scene["pos"].nbytes * 2 + s.scene["rho"].nbytes for s in specs) + 4 * srv.batch_steps
        e2e = {"value": srv.particle_steps * world / wall, "unit": "particle-steps/s",
               "h2d_bytes_per_step": h2d / max(srv.batch_steps, 1), "d2h_bytes_per_step": d2h / max(srv.batch_steps, 1),
               "wall_s": wall, "requests_completed": done, "batch_steps": srv.batch_steps, "rebuilds": srv.rebuilds,
               "rebuild_s": srv.rebuild_seconds, "requests_failed": len(srv.failed),
               "pair_overflows": srv.pair_overflows, "particles_escaped": int(sum(r.escaped for r in reqs)),
               "pooled": srv.pooled, "arena_grows": srv.arena_grows,
               "admit_s": getattr(srv, "admit_seconds", None)}
        for s in specs:
            s.dev = None
        # (d) real-time trace: Poisson arrivals at 50 / s
        reqs = [Request(t["rid"], t["arrival"], specs[k]) for k, t in enumerate(trace)]
        srv = Server(dev, budget_bytes=budget, rebuild_every=20, keep_final=False, pairs=args.pairs,
                     tuning=tuned["loaded"])
        wall = srv.run(reqs, time_scale=1.0, max_wall=600)
        lat = srv.latency_percentiles((50, 99))
        ttc = [r.finished - r.arrival for r in reqs if r.finished >= 0 and r.error is None]
        realtime = {"wall_s": wall, "particle_steps_per_s": srv.particle_steps / wall,
                    "step_latency_ms_p50": lat[50] * 1e3 if lat[50] else None,
                    "step_latency_ms_p99": lat[99] * 1e3 if lat[99] else None,
                    "time_to_completion_s_p50": float(np.percentile(ttc, 50)) if ttc else None,
                    "time_to_completion_s_p99": float(np.percentile(ttc, 99)) if ttc else None,
                    "requests_completed": len(ttc), "requests_failed": len(srv.failed),
                    "rebuilds": srv.rebuilds, "rebuild_s": srv.rebuild_seconds, "pooled": srv.pooled,
                    "arena_grows": srv.arena_grows, "admit_s": getattr(srv, "admit_seconds", None),
                    "latency": "per batch step, device time from before its admissions to after the step"}

    cpu = cpu_baseline_serving(args.requests) if rank == 0 and not args.no_cpu_baseline else None
    if rank == 0:
        line = base_line(args, world, value, ms, "particle-steps/s", {
            **serving_workload(args, world), "requests": len(specs), "particles_resident": total_p,
            "budget_gb": budget / 1e9,
            "batch_bytes": batch_bytes, "l2": f"state of {total_p} particles >> L2 (no flush needed)",
            "graph": "one CUDA graph per batch step",
            "pairs": "from the cell rows (no neighbor list)" if args.pairs == "cells" else "CSR list every step",
            "scene_generation_s": gen_s})
        line["phases_ms"] = {k: round(v, 4) for k, v in phases.items()}
        if tuned["loaded"] is not None:
            pick = lambda t: {str(b): {"cell_ratio": e["cell_ratio"], "tpp": e["tpp"],
                                       "ms_per_step": {k: round(m["ms_per_step"], 4) for k, m in e["measured"].items()}}
                              for b, e in t.serving.items()}
            line["tuning"] = {"loaded_batch": pick(tuned["loaded"]), "one_scene": pick(tuned["one_scene"]),
                              "candidates": "cell_ratio,tpp", "seconds": round(tune_s, 2)}
        line["roofline"] = {"bound": "hbm", "kernel": "deltaSPH forces (k_batch_pass1)", "achieved": achieved,
                            "peak": peak, "unit": "GB/s", "frac": achieved / peak if achieved else None,
                            "traffic": traffic_from_profiles("serving", f"k_batch_pass1[{args.pairs}]", total_p),
                            "algorithmic_bytes": alg,
                            "peak_source": peak_src}
        line["serving"] = {"one_scene_gpu_path": {"value": one_scene_value, "unit": "particle-steps/s",
                                                  "sample": [{"n": n, "ms_per_step": t * 1e3} for n, t in one]},
                           "batched_over_one_scene": value / one_scene_value, "realtime_trace": realtime,
                           "served_accuracy": accuracy if not args.no_trace else None}
        line["e2e"] = e2e or {"value": None, "unit": "particle-steps/s", "h2d_bytes_per_step": None,
                              "d2h_bytes_per_step": None}
        line["gpu_launches"] = launches * args.steps
        line["clocks"] = clk.summary()
        line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU: search + density
def run_search_density(args, dev, world, rank):
    import torch
    from pytorchsph_gb300 import _native as N
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.search import GridSearch
    pos, h, area, vmin, vmax, L = workloads.search_density_case(args.workload.rsplit("_", 1)[1])
    n = len(pos)
    pin = lambda a: torch.from_numpy(a).pin_memory()
    h_pos, h_h, h_a = pin(pos), pin(h), pin(area)
    d_pos, d_h, d_a = h_pos.to(dev), h_h.to(dev), h_a.to(dev)
    support = float(h[0])
    tuned = None
    if args.sort == "auto":
        from pytorchsph_gb300.tune import Autotuner, Tuning
        t = Tuning(search=Autotuner(dev).tune_search(
            data=(d_pos, d_h, d_a, dict(kernel_support=support, min_coord=vmin, max_coord=vmax))))
        tuned = t.search
        cfg = t.search_config(n)
        args.sort, args.digit_bits, args.cell_ratio = cfg["sort"], cfg["digit_bits"], cfg["cell_ratio"]
    gs = GridSearch(dev, sort=args.sort, digit_bits=args.digit_bits, cell_ratio=args.cell_ratio)
    first = gs.run(d_pos, d_h, d_a, kernel_support=support, min_coord=vmin, max_coord=vmax)
    cells, P = first.cell_capacity, first.num_pairs
    pair_cap = int(P * 1.05) + 1024
    rho_out = torch.empty(n, dtype=torch.float32, device=dev)
    events = {}

    def marks(name):
        e = events.get(name)
        if e is None:
            e = events[name] = make_event()
        e.record()

    def step():
        r = gs.run(d_pos, d_h, d_a, kernel_support=support, min_coord=vmin, max_coord=vmax, cell_capacity=cells,
                   pair_capacity=pair_cap, sync=False, marks=marks)
        N.call("sph_scatter_f32", N.ptr(r.order), N.ptr(r.rho), n, N.ptr(rho_out), N.stream_ptr())
        marks("end")
        return r

    # grid (bounds, final), keys, sort, gather, count, scan, fill, dense rows, scatter; a scan
    # is one kernel (the zeroing of its tile words is a memset); counting sort: scan,
    # scatter, in-cell fix of small and of large cells, which also gather the positions,
    # supports and areas; radix: per digit histogram, scan, scatter, then the cell starts
    # and the gather
    if args.sort == "counting":
        sort_launches = 4
    else:
        sort_launches = ((N.load().sph_key_bits(cells) + args.digit_bits - 1) // args.digit_bits) * 3 + 1 + 1
    launches_per_step = 2 + 1 + sort_launches + 1 + 1 + 1 + 1 + 1
    s = torch.cuda.Stream(dev)
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(2):
            step()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        res = step()
    flush = torch.empty(2 * 129 * 1024 * 1024 // 4 * 2, dtype=torch.float32, device=dev)
    for _ in range(max(args.warmup, 3)):
        g.replay()
    torch.cuda.synchronize()
    res.check()
    names = ["start", "keys", "sort", "gather", "count", "scan", "fill", "end"]
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    phase_acc = {k: 0.0 for k in names[1:]}
    ok = True
    with ClockSampler(dev.index or 0) as clk:
        sync_ranks(world)
        for k in range(args.steps):
            flush.zero_()
            starts[k].record()
            g.replay()
            ends[k].record()
            ends[k].synchronize()
            try:
                for a_, b_ in zip(names[:-1], names[1:]):
                    phase_acc[b_] += events[a_].elapsed_time(events[b_])
            except Exception:
                ok = False
        sync_ranks(world)
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps, world)
    value = n * world / (ms / 1e3)
    phases = {k: v / args.steps for k, v in phase_acc.items()} if ok else {}
    dom = max(["count", "fill"], key=lambda k: phases.get(k, 0.0)) if phases else "fill"
    kern = {"count": "nl_count", "fill": "nl_fill"}[dom]
    S = gs.stored_segments(n)
    # count: position 8, support 4, area 4, key 4 read; count 4, density 4, nseg 4 written; 8 per
    # stored segment; the cell table once.  fill: key 4, nseg 4, offset 4 read, 8 per segment
    # read, 4 per column written.
    alg = n * 32 + 8 * S + 4 * (cells + 2) if kern == "nl_count" else n * 12 + 8 * S + 4 * P
    peak, peak_src = hbm_peak()
    achieved = alg / (phases[dom] / 1e3) / 1e9 if phases else None
    e2e_ms = []
    rho_host = torch.empty(n, dtype=torch.float32).pin_memory()
    cnt_host = torch.empty(1, dtype=torch.int32).pin_memory()
    for k in range(args.steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_pos.copy_(h_pos, non_blocking=True)
        d_h.copy_(h_h, non_blocking=True)
        d_a.copy_(h_a, non_blocking=True)
        g.replay()
        rho_host.copy_(rho_out, non_blocking=True)
        cnt_host.copy_(res.offsets[n:n + 1], non_blocking=True)
        torch.cuda.synchronize()
        if k >= 2:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    assert int(cnt_host[0]) == P
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        reps, tt = 0, 0.0
        while reps < 10 and (reps < 1 or tt < 20.0):
            t0 = time.perf_counter()
            cpu_search_density(pos, h, area, vmin, vmax, L, threads)
            tt += time.perf_counter() - t0
            reps += 1
        cpu = {"value": n * reps / tt, "unit": "particles/s", "cores": threads, "kind": "port",
               "sample": f"{reps} full steps of {args.workload} (N={n}) with the oracle port (OpenMP)"}
    if rank == 0:
        line = base_line(args, world, value, ms, "particles/s", {
            "workload": args.workload, "particles": n, "pairs": P, "cells": cells, "support": "3dx", "sort": args.sort,
            "digit_bits": args.digit_bits if args.sort == "radix" else None,
            "cell_ratio": args.cell_ratio, "sort_chosen_by": "autotuner (measured on this workload in this run)" if tuned else "command line",
            "l2": "flushed between timed steps (flush not timed)", "graph": "one CUDA graph per step",
            "parallelism": f"replicas{world}", "segments": S})
        line["phases_ms"] = {k: round(v, 5) for k, v in phases.items()}
        if tuned:
            line["tuning"] = {str(b): {k: (round(x["ms"], 4) if isinstance(x, dict) else x)
                                       for k, x in e["measured"].items()} for b, e in tuned.items()}
        # the whole step against the search + density byte budget of the workload: per
        # particle 16 key generation, 60 sort (three 8-bit radix passes of 20), 28 reorder,
        # 12 cell table, 8 count, 8 scan, 8 fill read, 4 offsets, 4 density (148), plus 4 per
        # pair written as a CSR column and 4 read back by an unfused density pass
        step_alg = n * 148 + 8 * P
        step_gbs = step_alg / (ms / 1e3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak if achieved else None,
                            "traffic": traffic_from_profiles(args.workload, kern, n), "algorithmic_bytes": alg,
                            "peak_source": peak_src,
                            "step": {"algorithmic_bytes": step_alg, "achieved": step_gbs, "frac": step_gbs / peak,
                                     "unit": "GB/s", "bytes": "148 per particle + 8 per pair"}}
        line["e2e"] = {"value": n * world / (statistics.mean(e2e_ms) / 1e3), "unit": "particles/s",
                       "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 4 * n + 4}
        line["gpu_launches"] = launches_per_step * args.steps
        line["clocks"] = clk.summary()
        line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU: single dam breaks
def run_dambreak(args, dev, world, rank):
    import torch
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.sim import SimConfig, Simulation
    from pytorchsph_gb300.serve import SceneBatch, SceneSpec
    cpu = None
    if args.workload == "dambreak_deltasph":
        sc = workloads.dam_break(64, 128, 0.01, (4.0, 2.0))
        c0 = float(10 * np.sqrt(2 * 9.81 * sc["column_height"]))
        cfg = SimConfig(solver="deltaSPH", integration="semiImplicitEuler", dt=0.25 * sc["h"] / c0, c0=c0,
                        density_diffusion="deltaSPH")
        spec = SceneSpec(sc, cfg, 500)
        tuned = None
        if not args.no_tune:   # the autotuner's one-scene pick for this size
            from pytorchsph_gb300.tune import Autotuner, Tuning
            tuned = Tuning(serving=Autotuner(dev).tune_serving(sizes=(len(sc["pos"]),), batch_particles=1, steps=20))
        b = SceneBatch([spec], dev, tuning=tuned)
        b.capture()
        for _ in range(max(args.warmup, 3)):
            b.step()
        torch.cuda.synchronize()
        with ClockSampler(dev.index or 0) as clk:
            st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            sync_ranks(world)
            st.record()
            for _ in range(args.steps):
                b.step()
            en.record()
            sync_ranks(world)
        b.check()
        ms = max_over_ranks(st.elapsed_time(en) / args.steps, world)
        n, launches = b.n, b.launches_per_step()
        config = {"workload": args.workload, "particles": n, "walls": b.nb,
                  "solver": "deltaSPH renormalized, semi-implicit Euler", "c0": c0, "graph": "one CUDA graph per step",
                  "cell_ratio": spec.cell_ratio, "lanes_per_particle": spec.tpp,
                  "chosen_by": "autotuner (one scene, measured in this run)" if tuned else "defaults"}
        if rank == 0 and not args.no_cpu_baseline:
            t = cpu_deltasph_steps(sc, {"c0": c0, "dt": cfg.dt}, 2, "deltaSPH")
            cpu = {"value": n * 2 / t, "unit": "particle-steps/s", "cores": torch.get_num_threads(), "kind": "port",
                   "sample": "2 steps of the same scene with the restated reference step (float32, torch CPU)"}
    else:
        sc = workloads.dam_break(512, 512, 0.002, (4.096, 2.048))
        cfg = SimConfig(solver="dfsph", integration="semiImplicitEuler", dt=2e-4, c0=float(10 * np.sqrt(2 * 9.81 * 1.024)),
                        kinematic=0.01, fixed_dt=False, dt_min=1e-6, dt_max=1e-3, density_threshold=1e-4,
                        divergence_threshold=1e-3, max_density_iters=100, max_divergence_iters=100)
        sim = Simulation(sc, cfg, dev)
        # the block at rest first settles under gravity: the density solve runs to its
        # 100-iteration cap for the first ~50 steps (the reference does the same on smaller
        # blocks), then converges in 2-10 iterations for the rest of the 2000-step run; the
        # timed steps follow that start-up transient
        transient = []
        for k in range(max(args.warmup, 60)):
            sim.step(sync=False)
            transient.append(sim.last["density_iters"])
        transient = [int(t.item()) for t in transient]
        torch.cuda.synchronize()

        def timed(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(k):
                sim.step(sync=False)
            b.record()
            b.synchronize()
            return a.elapsed_time(b) / k

        eager_ms = timed(5)           # host-issued launches, for comparison
        try:
            sim.capture()             # the whole step as one CUDA graph
            graph = "one CUDA graph per step (cooperative solves inside)"
            for _ in range(3):
                sim.step(sync=False)
        except Exception as e:        # eager launches then
            graph = f"eager launches (capture failed: {e})"
        torch.cuda.synchronize()
        with ClockSampler(dev.index or 0) as clk:
            st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            sync_ranks(world)
            st.record()
            for _ in range(args.steps):
                sim.step(sync=False)
            en.record()
            sync_ranks(world)
        sim.check()
        ms = max_over_ranks(st.elapsed_time(en) / args.steps, world)
        n, launches = sim.n, 40
        config = {"workload": args.workload, "particles": n, "walls": sim.nb,
                  "solver": "DFSPH, divergence + density solves, semi-implicit Euler, adaptive dt",
                  "density_iters_last": int(sim.last["density_iters"].item()),
                  "warmup_steps_density_iters": transient,
                  "timed_steps": "after the start-up transient (the warm-up steps above)",
                  "graph": graph, "eager_ms_per_step": eager_ms}
        if rank == 0 and not args.no_cpu_baseline:
            # the full block takes minutes per CPU step: a 64 x 64 block of the same tank
            small = workloads.dam_break(64, 64, 0.016, (4.096, 2.048))
            t = cpu_dfsph_steps(small, 2)
            cpu = {"value": len(small["pos"]) * 2 / t, "unit": "particle-steps/s",
                   "cores": torch.get_num_threads(), "kind": "port",
                   "sample": f"2 DFSPH steps of a {len(small['pos'])}-particle block of the same tank with the "
                             f"restated reference step (oracle/sph_torch.py, float32, torch CPU)"}
    value = n * world / (ms / 1e3)
    if rank == 0:
        line = base_line(args, world, value, ms, "particle-steps/s", config)
        peak, peak_src = hbm_peak()
        line["roofline"] = {"bound": "hbm", "kernel": "step", "achieved": None, "peak": peak, "unit": "GB/s",
                            "frac": None, "traffic": None, "peak_source": peak_src}
        line["e2e"] = {"value": None, "unit": "particle-steps/s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None}
        line["gpu_launches"] = launches * args.steps
        line["clocks"] = clk.summary()
        line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def cpu_autograd_drop(sc, dt, steps):
    """Seconds for forward + torch autograd backward of `steps` restated reference steps
    (oracle/sph_torch.py, float64, torch CPU) with respect to v0 and alpha."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch
    import sph_torch as S
    alpha = torch.tensor(0.01, dtype=torch.float64, requires_grad=True)
    p = S.Params(h=sc["h"], c0=10.0, diffusion="MOG", vmin=sc["vmin"], vmax=sc["vmax"], gravity=(0.0, 0.0),
                 point_source=True, alpha=alpha, kinematic=0.001)
    v0 = torch.from_numpy(sc["vel"]).double().requires_grad_(True)
    t0 = time.perf_counter()
    st = {"x": torch.from_numpy(sc["pos"]).double(), "v": v0, "rho": torch.from_numpy(sc["rho"]).double(),
          "area": torch.from_numpy(sc["area"]).double()}
    for _ in range(steps):
        new, _ = S.step(st, None, p, dt, "semiImplicitEuler", "deltaSPH", torch.float64)
        st = {"x": new["x"], "v": new["v"], "rho": new["rho"], "area": st["area"]}
    ((st["x"] - torch.from_numpy(sc["pos"]).double()) ** 2).sum().backward()
    return time.perf_counter() - t0


def run_diff_drop(args, dev, world, rank):
    """Differentiable drop (config 5): 16,384-particle disc, 200-step rollout in float32
    forward and adjoint, loss against a target rollout (A = 1.0, alpha = 0.02) from A = 0.8,
    alpha = 0.01; gradient with respect to v0 and alpha by the GPU adjoint with checkpoints
    every 20 steps, checked against float64 central finite differences (eps 1e-4) on 64
    seeded velocity components and on alpha.  The float64 rollout's time is reported beside."""
    import torch
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.adjoint import DropRollout
    steps = 200
    start = workloads.oscillating_drop(16384, 0.5, 0.8)
    tgt = workloads.oscillating_drop(16384, 0.5, 1.0)
    dt = 0.1 * start["h"] / 10.0
    r64 = DropRollout(start, 10.0, dt, fp64=True, checkpoint_every=20, device=dev)
    r = DropRollout(start, 10.0, dt, fp64=False, checkpoint_every=20, device=dev)
    target, _ = r64.rollout(torch.as_tensor(tgt["vel"], dtype=torch.float64, device=dev), 0.02, steps)
    v0 = torch.as_tensor(start["vel"], dtype=torch.float32, device=dev)
    for _ in range(max(args.warmup, 3)):
        r.loss_and_grad(v0, 0.01, target, steps)
    torch.cuda.synchronize()
    reps = max(1, args.steps)
    with ClockSampler(dev.index or 0) as clk:
        st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sync_ranks(world)
        st.record()
        for _ in range(reps):
            loss, gv, ga = r.loss_and_grad(v0, 0.01, target, steps)
        en.record()
        sync_ranks(world)
    ms = max_over_ranks(st.elapsed_time(en) / reps, world)
    t0 = time.perf_counter()
    r.loss(v0, 0.01, target, steps)
    torch.cuda.synchronize()
    fwd_ms = (time.perf_counter() - t0) * 1e3
    v64 = v0.double()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r64.loss_and_grad(v64, 0.01, target, steps)
    torch.cuda.synchronize()
    f64_ms = (time.perf_counter() - t0) * 1e3
    # float64 central finite differences
    rng = np.random.default_rng(0)
    idx = rng.choice(v64.numel(), 64, replace=False)
    eps = 1e-4
    fd, ad = [], []
    for k in idx:
        e = torch.zeros(v64.numel(), dtype=torch.float64, device=dev)
        e[int(k)] = eps
        e = e.reshape(v64.shape)
        fd.append((r64.loss(v64 + e, 0.01, target, steps) - r64.loss(v64 - e, 0.01, target, steps)) / (2 * eps))
        ad.append(float(gv.reshape(-1)[int(k)]))
    fd, ad = np.array(fd), np.array(ad)
    fa = (r64.loss(v64, 0.01 + eps, target, steps) - r64.loss(v64, 0.01 - eps, target, steps)) / (2 * eps)
    n = r.n
    value = n * steps * world / (ms / 1e3)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu_steps = 3
        cpu_autograd_drop(start, dt, 1)
        t = cpu_autograd_drop(start, dt, cpu_steps)
        cpu = {"value": n * cpu_steps / t, "unit": "particle-steps/s", "cores": torch.get_num_threads(),
               "kind": "port", "sample": f"forward + torch autograd backward of {cpu_steps} float64 steps of the "
                                         f"same {n}-particle drop through the restated reference step "
                                         f"(oracle/sph_torch.py)"}
    if rank == 0:
        line = base_line(args, world, value, ms, "particle-steps/s", {
            "workload": "diff_drop", "particles": n, "rollout_steps": steps, "checkpoint_every": 20,
            "dtype": "f32", "loss": "mean |x_T - x*_T|^2", "target": "A = 1.0, alpha = 0.02",
            "start": "A = 0.8, alpha = 0.01", "dt": "0.1 h / c0", "density_diffusion": "MOG",
            "unit_of_work": "one forward + adjoint of the 200-step rollout per timed step"})
        line["dtype"] = "f32"
        line["float64_forward_adjoint_ms"] = f64_ms
        line["gradient_check"] = {
            "components": 64, "eps": eps,
            "max_abs_err_over_max_fd": float(np.abs(ad - fd).max() / max(np.abs(fd).max(), 1e-300)),
            "median_rel_err": float(np.median(np.abs(ad - fd) / np.maximum(np.abs(fd), 1e-300))),
            "alpha_adjoint": ga, "alpha_fd": fa, "alpha_rel_err": abs(ga - fa) / max(abs(fa), 1e-300),
            "loss": loss}
        line["forward_ms"] = fwd_ms
        peak, peak_src = hbm_peak()
        line["roofline"] = {"bound": "hbm", "kernel": "k_drop_adjoint (float32)", "achieved": None, "peak": peak,
                            "unit": "GB/s", "frac": None, "traffic": None, "peak_source": peak_src,
                            "note": "the dual-number pair products bound this kernel, not HBM"}
        line["e2e"] = {"value": None, "unit": "particle-steps/s", "h2d_bytes_per_step": None,
                       "d2h_bytes_per_step": None}
        line["gpu_launches"] = None
        line["clocks"] = clk.summary()
        line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from pytorchsph_gb300 import build as B
    B.build()
    from pytorchsph_gb300 import _native as N
    N.load()
    if world > 1:
        dist.barrier()
    if args.workload == "serving":
        run_serving(args, dev, world, rank)
    elif args.workload.startswith("search_density_"):
        run_search_density(args, dev, world, rank)
    elif args.workload in ("dambreak_deltasph", "dambreak_dfsph"):
        run_dambreak(args, dev, world, rank)
    elif args.workload == "diff_drop":
        run_diff_drop(args, dev, world, rank)
    else:
        raise SystemExit(f"unknown workload {args.workload}")
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
