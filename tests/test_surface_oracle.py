"""The delta+ restatement (oracle/sph_torch.py: surface_detect, shift) against the reference's
own detectSurface and shift (tests/golden/surface_golden.npz, made by
tests/golden/make_surface_golden.py): float32 restatement vs the reference's float32 run on
the same inputs, float64 vs its float64 run."""
import json
import os

import numpy as np
import pytest
import torch

import sph_torch as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "surface_golden.npz")


def rel(a, b):
    a = a.detach().double().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module")
def gold():
    g = np.load(GOLDEN)
    return g, json.loads(str(g["meta"]))


def _unit(d):
    r = torch.linalg.norm(d, dim=1)
    return torch.where((r < 1e-7)[:, None], torch.zeros_like(d), d / torch.where(r < 1e-7, 1.0, r)[:, None]), r


def inputs(g, part, dtype, h, recompute=False):
    """Fluid / wall / wall-wall dicts from the golden's float32 inputs; recompute=True derives
    distances and q from the positions in `dtype` (what the reference's float64 run sees)."""
    G = lambda k: torch.from_numpy(np.ascontiguousarray(g[f"{part}/in_{k}"]))
    x = G("fluidPosition").to(dtype)
    nb = G("fluidNeighbors").long()
    fl = {"x": x, "v": G("fluidVelocity"), "rho": G("fluidDensity"), "area": G("fluidArea"),
          "volume": G("fluidVolume"), "i": nb[0], "j": nb[1], "e": G("fluidDistances"),
          "q": G("fluidRadialDistances")}
    bp = G("boundaryToFluidNeighbors").long()
    W = lambda k: torch.from_numpy(np.ascontiguousarray(g[f"{'f64_' if dtype == torch.float64 else ''}{part}/in_{k}"]))
    xb = W("boundaryPositions").to(dtype)
    wl = {"bb": bp[0], "bf": bp[1], "e": G("boundaryToFluidNeighborDistances"),
          "q": G("boundaryToFluidNeighborRadialDistances"), "x": xb, "area": W("boundaryVolume"),
          "rho": W("boundaryDensity")}
    ww = None
    if f"{part}/in_boundaryToBoundaryNeighbors" in g.files:
        wp = G("boundaryToBoundaryNeighbors").long()
        ww = {"i": wp[0], "j": wp[1], "e": G("boundaryToBoundaryNeighborDistances"),
              "q": G("boundaryToBoundaryNeighborRadialDistances")}
    if recompute:
        e, r = _unit(x[fl["i"]] - x[fl["j"]])
        fl["e"], fl["q"] = e, r / h
        e, r = _unit(xb[wl["bb"]] - x[wl["bf"]])
        wl["e"], wl["q"] = e, r / h
        fl["volume"] = fl["area"].to(dtype) / fl["rho"].to(dtype)
        if ww is not None:
            e, r = _unit(xb[ww["j"]] - xb[ww["i"]])
            ww["e"], ww["q"] = e, r / h
    return fl, wl, ww


KEYS = ("fluidLambda", "eigVals", "normalizationMatrix", "fluidL", "lambdaGrad", "fluidNormal", "angleMin",
        "angleMax", "boundaryNormalizationMatrix", "boundaryEigVals")


def test_surface_detection_float32(gold):
    g, m = gold
    fl, wl, ww = inputs(g, "surface", torch.float32, m["h"])
    out = S.surface_detect(fl, wl, ww, m["h"], torch.float32)
    for k in KEYS:
        assert rel(out[k], g[f"surface/out_{k}"]) < 1e-4, k
    assert np.array_equal(out["fluidSurfaceMask"].numpy(), g["surface/out_fluidSurfaceMask"])


def test_surface_detection_float64(gold):
    g, m = gold
    fl, wl, ww = inputs(g, "surface", torch.float64, m["h"], recompute=True)
    out = S.surface_detect(fl, wl, ww, np.float32(m["h"]), torch.float64)
    for k in KEYS:
        assert rel(out[k], g[f"f64_surface/out_{k}"]) < 1e-9, k
    assert np.array_equal(out["fluidSurfaceMask"].numpy(), g["f64_surface/out_fluidSurfaceMask"])


@pytest.mark.parametrize("tag,dtype,tol", [("", torch.float32, 1e-5), ("f64_", torch.float64, 1e-10)])
def test_shift(gold, tag, dtype, tol):
    g, m = gold
    G = lambda k: torch.from_numpy(np.ascontiguousarray(g[f"{tag}shift/in_{k}"]))
    nb = G("fluidNeighbors").long()
    bp = G("boundaryToFluidNeighbors").long()
    fl = {"v": G("fluidVelocity"), "rho": G("fluidDensity"), "area": G("fluidArea"), "i": nb[0], "j": nb[1],
          "e": G("fluidDistances"), "q": G("fluidRadialDistances")}
    wl = {"bb": bp[0], "bf": bp[1], "e": G("boundaryToFluidNeighborDistances"),
          "q": G("boundaryToFluidNeighborRadialDistances"), "area": G("boundaryVolume"), "rho": G("boundaryDensity")}
    raw, upd, mask = S.shift(fl, wl, G("fluidNormal"), G("fluidSurfaceMask"), np.float32(m["h"]), m["c0"], m["packing"],
                              dtype)
    assert rel(raw, g[f"{tag}shift/out_shiftAmount"]) < tol
    assert rel(upd, g[f"{tag}shift/out_fluidUpdate"]) < tol
    assert np.array_equal(mask.numpy(), g[f"{tag}shift/out_fluidSurfaceMask"])


def test_reference_float32_surface_noise(gold):
    """States the float32 reference's own error against its float64 run: lambda and the mask
    are stable, the normal (a normalised gradient that is small in the bulk) much less."""
    g, _ = gold
    assert rel(g["surface/out_fluidLambda"], g["f64_surface/out_fluidLambda"]) < 1e-4
    assert np.array_equal(g["surface/out_fluidSurfaceMask"], g["f64_surface/out_fluidSurfaceMask"])
