"""Build the sm_103a shared library `libsph_gb300.so` in-tree with nvcc.

Every translation unit under csrc/ is compiled in parallel for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`), without fast-math (the pair predicate and
the cell-key arithmetic must round exactly like the reference), then linked into one
C-ABI library (include/sph_gb300.h).  No torch headers are involved, so the library
does not depend on the PyTorch version it is loaded next to.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB_NAME = "libsph_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the GB300 library cannot be built")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "sph_gb300.h"))
    return hs


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


def build(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
             "-I", os.path.join(ROOT, "include")] + ARCH + list(extra_flags or [])
    objs, jobs = [], []
    for src in sources():
        obj = os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([cc] + flags + ["-c", src, "-o", obj])
    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(o) > os.path.getmtime(LIB_PATH) for o in objs):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        run([cc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
