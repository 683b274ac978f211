"""Known answers for the full-size search + density inputs (N = 2^20, variants A and B of
pytorchsph_gb300.workloads.search_density_case), computed with the reference's own compiled
CPU neighbor search (cppSrc/neighSearch.cpp via oracle/build_ref.py) on the reference's
sortPositions / constructHashMap outputs.  Writes tests/golden/full_size.json:
pair count, max neighbors and an order-independent checksum of the pair set.
Usage: python tests/golden/make_full_size.py   (needs the reference checkout)
"""
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import ref_harness  # noqa: E402
from pytorchsph_gb300 import workloads  # noqa: E402


def pair_checksum(rows, cols, n):
    """sum over pairs of (i * n + j) * golden-ratio constant, mod 2^64 (order independent)."""
    k = rows.astype(np.uint64) * np.uint64(n) + cols.astype(np.uint64)
    return int(np.sum(k * np.uint64(0x9E3779B97F4A7C15), dtype=np.uint64))


def main():
    R = ref_harness.load()
    torch.set_num_threads(os.cpu_count())
    out = {}
    for v in ("A", "B"):
        pos, h, area, vmin, vmax, L = workloads.search_density_case(v)
        rows, cols, *_ = R.neighborSearch.constructNeighborhoods(
            torch.from_numpy(pos), torch.from_numpy(h), L, minCoord=torch.from_numpy(vmin),
            maxCoord=torch.from_numpy(vmax))
        rows, cols = rows.numpy(), cols.numpy()
        n = len(pos)
        cnt = np.bincount(rows, minlength=n)
        import hashlib
        out[v] = {"input_sha256": hashlib.sha256(pos.tobytes()).hexdigest(), "n": n, "pairs": int(len(rows)), "max_neighbors": int(cnt.max()),
                  "checksum": pair_checksum(rows, cols, n), "hash_len": int(L)}
        print(v, out[v], flush=True)
    with open(os.path.join(HERE, "full_size.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
