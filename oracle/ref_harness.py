"""Test infrastructure only (oracle): import the reference's own Python code on CPU.

wi-re/pytorchSPH is a TorchScript research code with third-party imports that are not
installed here (torch_geometric, torch_scatter, matplotlib, h5py, skimage, tomli,
ipywidgets, yaml).  This harness makes its hot-path modules importable so that
golden vectors can be generated from the reference itself:

* TorchScript is switched off (`torch.jit._state.disable()`, the in-process form of
  `PYTORCH_JIT=0`): torch 2.x rejects the numpy-scalar `h` the reference passes to
  unannotated Tensor arguments (src/kernels.py:21).
* `torch.utils.cpp_extension.load` is redirected to the CPU build of the reference's own
  `cppSrc/neighSearch.cpp` made by `oracle/build_ref.py`
  (src/modules/neighborSearch.py:28 calls `load` at import time).
* Missing third-party modules are replaced by small stand-ins.  `torch_scatter.scatter`
  is restated with `Tensor.index_add_` (sum/add) and `scatter_reduce` (max/min/mean);
  `torch_geometric.nn.radius` by a brute-force `<= r` radius search (its exact tie
  semantics are not pinned; the fluid-side results of the paths covered here do not
  depend on it, see solidBoundary.py:180 usage).  Plotting/IO modules are inert.

Only the development container has the reference checkout; the generated vectors are
committed under tests/golden/ so the tests never need this module.  Nothing in the
product imports it.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from build_ref import REF_ROOT  # noqa: E402  (the checkout's location is set in the build recipe)

_loaded = None


def available() -> bool:
    return os.path.exists(os.path.join(REF_ROOT, "src", "modules", "neighborSearch.py"))


class _Anything(types.ModuleType):
    """Module stand-in whose every attribute is a callable no-op object."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Callable()


class _Callable:
    def __call__(self, *a, **k):
        return _Callable()

    def __getattr__(self, name):
        return _Callable()


def _install_stubs():
    import torch

    def scatter(src, index, dim=-1, out=None, dim_size=None, reduce="sum"):
        if dim < 0:
            dim = src.dim() + dim
        if dim_size is None:
            dim_size = int(index.max()) + 1 if index.numel() > 0 else 0
        size = list(src.shape)
        size[dim] = dim_size
        if reduce in ("sum", "add"):
            res = torch.zeros(size, dtype=src.dtype, device=src.device)
            return res.index_add_(dim, index, src)
        idx = index
        while idx.dim() < src.dim():
            idx = idx.unsqueeze(-1)
        idx = idx.expand_as(src)
        res = torch.zeros(size, dtype=src.dtype, device=src.device)
        red = {"max": "amax", "min": "amin", "mean": "mean"}[reduce]
        return res.scatter_reduce(dim, idx, src, reduce=red, include_self=False)

    ts = types.ModuleType("torch_scatter")
    ts.scatter = scatter
    sys.modules["torch_scatter"] = ts

    def radius(x, y, r, batch_x=None, batch_y=None, max_num_neighbors=32):
        d = torch.cdist(y.double(), x.double())
        yi, xi = torch.nonzero(d <= r, as_tuple=True)
        return torch.stack([yi, xi], 0)

    tg = types.ModuleType("torch_geometric")
    tgnn = _Anything("torch_geometric.nn")
    tgnn.radius = radius
    tg.nn = tgnn
    sys.modules["torch_geometric"] = tg
    sys.modules["torch_geometric.nn"] = tgnn
    sys.modules["torch_geometric.loader"] = _Anything("torch_geometric.loader")

    import tomllib

    sys.modules.setdefault("tomli", tomllib)
    for name in [
        "matplotlib", "matplotlib.pyplot", "matplotlib.patches", "matplotlib.colors",
        "matplotlib.ticker", "matplotlib.cm", "mpl_toolkits", "mpl_toolkits.axes_grid1",
        "h5py", "ipywidgets", "yaml", "skimage", "skimage.measure", "tqdm.notebook",
        "src.modules.implicitShifting",
    ]:
        if name not in sys.modules or name.startswith(("matplotlib", "mpl_toolkits")):
            sys.modules[name] = _Anything(name)


def load():
    """Import and return the reference package `src` with its hot-path modules loaded."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not available():
        raise RuntimeError("reference checkout not present")
    import torch
    import torch.jit._state as jit_state
    import torch.utils.cpp_extension as ce

    jit_state.disable()
    _install_stubs()
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    import build_ref  # noqa: E402

    ref_ext = build_ref.build()
    orig_load = ce.load
    ce.load = lambda *a, **k: ref_ext
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    try:
        mods = {}
        for name in [
            "src.kernels", "src.util", "src.module",
            "src.modules.neighborSearch", "src.modules.density", "src.modules.momentum",
            "src.modules.densityDiffusion", "src.modules.pressure", "src.modules.diffusion",
            "src.modules.laminar", "src.modules.gravity", "src.modules.dfsph",
            "src.modules.solidBoundary", "src.modules.adaptiveDT",
        ]:
            mods[name.split(".")[-1]] = importlib.import_module(name)
    finally:
        ce.load = orig_load
    mods["ext"] = ref_ext
    _loaded = types.SimpleNamespace(**mods)
    return _loaded
