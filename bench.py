"""Benchmark of the GB300 SPH hot path (one JSON line on rank 0).

Workload `search_density_A` (default) / `search_density_B`: one step = the full hashed-grid
neighbor search plus the density summation over N = 2^20 particles in [0,1]^2 (h = 3 dx,
A = dx^2, domain [0,1]^2): grid bounds -> cell keys -> radix sort -> sorted SoA -> cell
table -> CSR count with fused density -> scan -> CSR fill -> density back to particle order.

  python bench.py [--steps K] [--warmup W] [--workload search_density_A|search_density_B]
  python bench.py --impl reference ...   # the reference algorithm on the host cores

`value` (particles searched per second) is timed on the device with the inputs resident
in HBM, L2 flushed between steps; `e2e` times the same step through the public API from
pinned host buffers (H2D of positions/supports/areas, D2H of the density and pair count).
With torchrun (N>1) every rank runs an independent replica (the path has no exchange
step) and `value` sums over ranks.
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
    ap.add_argument("--workload", default="search_density_A")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sort", default="counting", choices=["counting", "radix"])
    ap.add_argument("--digit-bits", type=int, default=8)
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
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 5 + k and s[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ----------------------------------------------------------------------------- CPU arm
def cpu_search_density(pos, h, area, vmin, vmax, L, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import nsearch as ns
    si = ns.SortInfo(pos, h, vmin, vmax, L)
    rows, cols = ns.nl_cells(si, threads=threads)
    off, c = ns.canonical_csr(rows, cols, si.n)
    rho = ns.density(off, c, pos, area, float(h[0]))
    return len(rows), rho


def time_cpu(pos, h, area, vmin, vmax, L, budget_s=20.0, max_reps=10):
    threads = os.cpu_count() or 1
    reps, t_total = 0, 0.0
    while reps < max_reps and (reps < 1 or t_total < budget_s):
        t0 = time.perf_counter()
        cpu_search_density(pos, h, area, vmin, vmax, L, threads)
        t_total += time.perf_counter() - t0
        reps += 1
    return len(pos) * reps / t_total, threads, reps


def load_workload(name):
    from pytorchsph_gb300 import workloads
    if name.startswith("search_density_"):
        v = name.rsplit("_", 1)[1]
        return workloads.search_density_case(v)
    raise SystemExit(f"unknown workload {name}")


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pos, h, area, vmin, vmax, L = load_workload(args.workload)
    # the reference compiles only where its checkout exists; elsewhere the oracle port
    # (oracle/nsearch_oracle.c, the same algorithm) stands in for it
    kind = "port"
    cpu_search_density(pos[:4096], h[:4096], area[:4096], vmin, vmax, -1, 1)  # build + warm
    threads = os.cpu_count() or 1
    times = []
    for _ in range(args.warmup):
        cpu_search_density(pos, h, area, vmin, vmax, L, threads)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_search_density(pos, h, area, vmin, vmax, L, threads)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = len(pos) / (ms / 1e3)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "particles": len(pos), "support": "3dx", "hash_len": L},
            "cpu_baseline": {"value": value, "unit": "particles/s", "cores": threads, "kind": kind,
                             "sample": f"full {args.workload} step x {args.steps} (sort + hash map + "
                                       f"buildNeighborList + density)"},
            "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm
# algorithmic bytes per particle of each kernel of the step (measurement)
def algorithmic_bytes(kernel, n, P, cells):
    if kernel == "nl_count":   # xy (8) + h (4) + A (4) + key (4) read, count (4) + rho (4) written, cell table once
        return n * 28 + 4 * (cells + 2)
    if kernel == "nl_fill":    # xy (8) + h (4) + key (4) + offsets (4) read, cols written (4 per pair)
        return n * 20 + 4 * P + 4 * (cells + 2)
    if kernel == "radix_sort": # per pass: keys+vals read twice (hist + scatter), written once
        return n * 24
    return n * 16


def make_event():
    import torch
    try:  # an event recorded inside a captured graph becomes a timed node only when external
        return torch.cuda.Event(enable_timing=True, external=True)
    except TypeError:
        return torch.cuda.Event(enable_timing=True)


PHASES = ["start", "keys", "sort", "gather", "count", "scan", "fill", "end"]


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
    from pytorchsph_gb300.search import GridSearch
    N.load()

    pos, h, area, vmin, vmax, L = load_workload(args.workload)
    n = len(pos)
    pin = lambda a: torch.from_numpy(a).pin_memory()
    h_pos, h_h, h_a = pin(pos), pin(h), pin(area)
    d_pos, d_h, d_a = h_pos.to(dev), h_h.to(dev), h_a.to(dev)
    support = float(h[0])
    gs = GridSearch(dev, sort=args.sort, digit_bits=args.digit_bits)
    first = gs.run(d_pos, d_h, d_a, kernel_support=support, min_coord=vmin, max_coord=vmax)
    cells = first.cell_capacity
    P = first.num_pairs
    pair_cap = int(P * 1.05) + 1024
    rho_out = torch.empty(n, dtype=torch.float32, device=dev)
    events = {}

    def marks(name):
        e = events.get(name)
        if e is None:
            e = events[name] = make_event()
        e.record()

    def step():
        r = gs.run(d_pos, d_h, d_a, kernel_support=support, min_coord=vmin, max_coord=vmax,
                   cell_capacity=cells, pair_capacity=pair_cap, sync=False, marks=marks)
        N.call("sph_scatter_f32", N.ptr(r.order), N.ptr(r.rho), n, N.ptr(rho_out), N.stream_ptr())
        marks("end")
        return r

    # kernels per step: grid 2, keys 1, sort (counting: scan 3 + scatter + fix + fix_large = 6,
    # plus one memset; radix: passes x 5 + cell starts), gather 1, count 1, scan 3, fill 1,
    # scatter 1 (and one torch fill of the status word)
    if args.sort == "counting":
        sort_launches = 6
    else:
        sort_launches = ((N.load().sph_key_bits(cells) + args.digit_bits - 1) // args.digit_bits) * 5 + 1
    launches_per_step = 2 + 1 + sort_launches + 1 + 1 + 3 + 1 + 1

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
    flush = torch.empty(2 * 129 * 1024 * 1024 // 4 * 2, dtype=torch.float32, device=dev)  # 2x L2
    for _ in range(max(args.warmup, 3)):
        g.replay()
    torch.cuda.synchronize()
    res.check()
    assert res.num_pairs == P

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    phase_acc = {k: 0.0 for k in PHASES[1:]}
    phase_ok = True
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            starts[k].record()
            g.replay()
            ends[k].record()
            ends[k].synchronize()
            try:
                for a_, b_ in zip(PHASES[:-1], PHASES[1:]):
                    phase_acc[b_] += events[a_].elapsed_time(events[b_])
            except Exception:
                phase_ok = False
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    if world > 1:
        dist.barrier()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps
    ms_t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms = float(ms_t.item())
    value = n * world / (ms / 1e3)
    phases = {k: v / args.steps for k, v in phase_acc.items()} if phase_ok else {}
    dom = max(["count", "fill"], key=lambda k: phases.get(k, 0.0)) if phases else "fill"
    dom_kernel = {"count": "nl_count", "fill": "nl_fill"}[dom]
    alg = algorithmic_bytes(dom_kernel, n, P, cells)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg / (phases[dom] / 1e3) / 1e9 if phases else None
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
        traffic = prof.get(args.workload, {}).get(dom_kernel)
    except Exception:
        pass

    # end to end through the public API from pinned host memory
    e2e_ms = []
    h2d = h_pos.numel() * 4 + h_h.numel() * 4 + h_a.numel() * 4
    d2h = n * 4 + 4
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
    e2e_value = n * world / (statistics.mean(e2e_ms) / 1e3)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, cores, reps_cpu = time_cpu(pos, h, area, vmin, vmax, L)
        cpu = {"value": v, "unit": "particles/s", "cores": cores, "kind": "port",
               "sample": f"{reps_cpu} full steps of {args.workload} (N={n}) with the oracle port "
                         f"(oracle/nsearch_oracle.c, OpenMP)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": args.workload, "particles": n, "pairs": P, "cells": cells,
                           "support": "3dx", "sort": args.sort,
                           "l2": "flushed between timed steps (flush not timed)",
                           "graph": "one CUDA graph per step", "parallelism": f"replicas{world}"},
                "phases_ms": {k: round(v, 5) for k, v in phases.items()},
                "roofline": {"bound": "hbm", "kernel": dom_kernel, "achieved": achieved, "peak": peak,
                             "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                             "algorithmic_bytes": alg,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
                "e2e": {"value": e2e_value, "unit": "particles/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches_per_step * args.steps,
                "clocks": clk.summary(), "wall_s_timed_loop": t_wall,
                "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
