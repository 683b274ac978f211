"""Dataset export in the reference's layout (pytorchsph_gb300.export; src/simulationBase.py:
443-492, 742-780): the file holds root attributes, boundaryInformation and one
simulationExport/%05d group per exported step with the reference's dataset names and the
attributes time, timestep, dt.  CPU: the writer's layout round trip; GPU: a dam break exported
asynchronously every step and read back against the engine's own state."""
import json
import zipfile

import numpy as np
import pytest
import torch


def test_npz_tree_writer_round_trip(tmp_path):
    from pytorchsph_gb300.export import NpzTreeWriter
    p = str(tmp_path / "run.npz")
    w = NpzTreeWriter(p)
    w.set_attrs("/", {"simulationScheme": "deltaSPH", "c0": np.float32(10.0), "fluidGravity": np.array([0, -9.81])})
    w.write("boundaryInformation", "boundaryPosition", np.ones((3, 2), np.float32))
    for k in range(2):
        g = "simulationExport/%05d" % k
        w.set_attrs(g, {"time": 0.1 * (k + 1), "timestep": k + 1, "dt": 0.1})
        w.write(g, "fluidPosition", np.full((4, 2), k, np.float32))
        w.write(g, "UID", np.arange(4, dtype=np.int32))
    w.close()
    z = np.load(p)
    assert set(z.files) >= {"boundaryInformation/boundaryPosition", "simulationExport/00000/fluidPosition",
                            "simulationExport/00001/UID"}
    assert np.array_equal(z["simulationExport/00001/fluidPosition"], np.ones((4, 2), np.float32))
    attrs = json.loads(zipfile.ZipFile(p).read("attributes.json"))
    assert attrs["/"]["simulationScheme"] == "deltaSPH" and attrs["/"]["fluidGravity"] == [0.0, -9.81]
    assert attrs["simulationExport/00001"]["timestep"] == 2


@pytest.mark.gpu
def test_simulation_export_matches_state(cuda, tmp_path):
    from pytorchsph_gb300 import workloads
    from pytorchsph_gb300.export import SnapshotExporter
    from pytorchsph_gb300.sim import Simulation, SimConfig
    sc = workloads.dam_break(24, 40, 0.01, (1.0, 1.0))
    c0 = float(10 * np.sqrt(2 * 9.81 * sc["column_height"]))
    cfg = SimConfig(solver="deltaSPH", integration="semiImplicitEuler", dt=0.25 * sc["h"] / c0, c0=c0,
                    density_diffusion="deltaSPH")
    sim = Simulation(sc, cfg, cuda)
    p = str(tmp_path / "dam.npz")
    ex = SnapshotExporter(p, attrs=sim.export_attributes(), boundary=sim.boundary_information(), depth=2,
                          device=cuda)
    states = []
    for _ in range(5):
        sim.step(sync=False)
        sim.export(ex)
        states.append(sim.state())
    ex.close()
    z = np.load(p)
    attrs = json.loads(zipfile.ZipFile(p).read("attributes.json"))
    assert attrs["/"]["densityDiffusionScheme"] == "deltaSPH" and attrs["/"]["densityScheme"] == "continuum"
    assert np.array_equal(z["boundaryInformation/boundaryPosition"], sc["wall_pos"])
    for k, s in enumerate(states):
        g = "simulationExport/%05d" % k
        uid = z[f"{g}/UID"].astype(np.int64)
        assert sorted(uid.tolist()) == list(range(len(sc["pos"])))
        for name, key in (("fluidPosition", "x"), ("fluidVelocity", "v"), ("fluidAcceleration", "acc")):
            got = np.empty_like(s[key])
            got[uid] = z[f"{g}/{name}"]
            assert np.array_equal(got, s[key]), (k, name)
        a = attrs[g]
        assert a["timestep"] == k + 1
        assert abs(a["dt"] - cfg.dt) <= 1e-6 * cfg.dt and abs(a["time"] - (k + 1) * cfg.dt) <= 1e-5 * a["time"]
        for name in ("finalPosition", "finalVelocity", "fluidArea", "fluidDensity", "fluidSupport", "fluidPressure",
                     "fluidDpdt", "boundaryDensity"):
            assert f"{g}/{name}" in z.files, name
