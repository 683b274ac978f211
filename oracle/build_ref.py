"""Test infrastructure only (oracle): compile the reference's own CPU neighbor search.

Builds `cppSrc/neighSearch.cpp` of wi-re/pytorchSPH, from the file where it lies in the
read-only reference checkout, with the reference's own flags
(`-fopenmp -O3 -march=native`, src/modules/neighborSearch.py:28) plus
`oracle/ref_cuda_stub.cpp` for the two CUDA symbols it declares.  The result is a Python
extension module written only into `oracle/_ref/` (git-ignored).

The reference checkout only exists in the development container; on a machine without
it this script reports that and returns None.  Nothing in the product imports this.
This recipe is the one place that names where the checkout lies (`REF_ROOT`, overridden by
the environment variable PYTORCHSPH_REFERENCE); the harness and the tests take it from here.
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PYTORCHSPH_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "cppSrc", "neighSearch.cpp")
OUT_DIR = os.path.join(HERE, "_ref")


def build(verbose: bool = False):
    """Compile (or load the cached build of) the reference CPU extension; None if absent."""
    if not os.path.exists(REF_SRC):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    import torch.utils.cpp_extension as ce

    return ce.load(
        name="refNeighborSearch",
        sources=[REF_SRC, os.path.join(HERE, "ref_cuda_stub.cpp")],
        extra_cflags=["-fopenmp", "-O3", "-march=native"],
        extra_ldflags=["-fopenmp"],
        build_directory=OUT_DIR,
        verbose=verbose,
    )


if __name__ == "__main__":
    mod = build(verbose=True)
    print("reference extension:", mod if mod is not None else "unavailable (no reference checkout)")
    sys.exit(0)
