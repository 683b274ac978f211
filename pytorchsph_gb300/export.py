"""Per-step dataset export of the reference's layout, without stalling the GPU.

The reference writes one HDF5 file per simulation (src/simulationBase.py:443-492, 742-780):
root attributes (schemes, fluid and kernel parameters), a `boundaryInformation` group with the
static wall arrays, and a group `simulationExport/%05d` per exported step holding the fluid
arrays (UID, fluidPosition, fluidVelocity, finalPosition, finalVelocity, fluidArea,
fluidDensity, fluidSupport, fluidPressure, fluidAcceleration, fluidGravity for a point
source, fluidDpdt for continuum density) plus what the modules add (boundaryDensity,
fluidShifting), with the attributes time, timestep and dt.  It does so synchronously with
`.cpu()` on every array.

Here a step's arrays are copied device -> pinned host on a copy stream that first waits on
an event recorded on the compute stream, so the copies overlap the following steps; a writer
thread waits for each copy and writes the group.  At most `depth` snapshots are in flight;
`submit` blocks only when all of them are (back-pressure).

Writers: `HDF5Writer` (h5py, when importable) and `NpzTreeWriter`, which keeps the same group
and dataset paths as members of a zip of .npy arrays (`np.load(path)["simulationExport/00000/
fluidPosition"]`) with every attribute in the member `attributes.json`.  Arrays are written
in the engine's row order together with the UID of each row, as the reference's are.
"""
from __future__ import annotations

import io
import json
import os
import queue
import threading
import zipfile

import numpy as np
import torch


def _jsonable(v):
    if isinstance(v, (np.generic,)):
        return v.item()
    if isinstance(v, np.ndarray):
        return v.tolist()
    if isinstance(v, (list, tuple)):
        return [_jsonable(x) for x in v]
    return v


class NpzTreeWriter:
    """Groups and datasets as members '<group>/<name>.npy' of a zip archive (np.load reads it);
    attributes of the root and of every group in 'attributes.json'."""

    def __init__(self, path: str):
        self.path = path
        self.zf = zipfile.ZipFile(path, "w", compression=zipfile.ZIP_STORED, allowZip64=True)
        self.attrs = {"/": {}}

    def set_attrs(self, group: str, attrs: dict):
        self.attrs.setdefault(group or "/", {}).update({k: _jsonable(v) for k, v in attrs.items()})

    def write(self, group: str, name: str, array: np.ndarray):
        buf = io.BytesIO()
        np.lib.format.write_array(buf, np.ascontiguousarray(array), allow_pickle=False)
        self.zf.writestr(f"{group}/{name}.npy" if group else f"{name}.npy", buf.getvalue())

    def close(self):
        self.zf.writestr("attributes.json", json.dumps(self.attrs, indent=1, sort_keys=True))
        self.zf.close()


class HDF5Writer:
    """The reference's own file format through h5py."""

    def __init__(self, path: str):
        import h5py
        self.f = h5py.File(path, "w")

    def _group(self, group):
        return self.f.require_group(group) if group and group != "/" else self.f

    def set_attrs(self, group: str, attrs: dict):
        g = self._group(group)
        for k, v in attrs.items():
            g.attrs[k] = v

    def write(self, group: str, name: str, array: np.ndarray):
        self._group(group).create_dataset(name, data=array)

    def close(self):
        self.f.close()


def open_writer(path: str, kind: str = "auto"):
    """kind: 'hdf5', 'npz' or 'auto' (HDF5 when h5py is importable and the path ends in .hdf5 / .h5)."""
    if kind == "auto":
        try:
            import h5py  # noqa: F401
            kind = "hdf5" if path.endswith((".hdf5", ".h5")) else "npz"
        except ImportError:
            kind = "npz"
    return HDF5Writer(path) if kind == "hdf5" else NpzTreeWriter(path)


class SnapshotExporter:
    """Asynchronous per-step export in the reference's layout (see the module docstring).

    exporter = SnapshotExporter(path, attrs=root_attributes, boundary=wall_arrays)
    exporter.submit(fields, time=t, timestep=k, dt=dt)   # device tensors, returns at once
    exporter.close()                                      # drains the queue, closes the file
    """

    def __init__(self, path: str, attrs: dict | None = None, boundary: dict | None = None, interval: int = 1,
                 depth: int = 3, writer: str = "auto", device=None):
        self.dev = torch.device(device or torch.device("cuda", torch.cuda.current_device()))
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        self.w = open_writer(path, writer)
        self.w.set_attrs("/", attrs or {})
        if boundary:
            for k, v in boundary.items():
                self.w.write("boundaryInformation", k, np.asarray(v.detach().cpu() if isinstance(v, torch.Tensor)
                                                                  else v))
        self.interval = max(1, int(interval))
        self.calls = 0
        self.counter = 0
        self.copy_stream = torch.cuda.Stream(device=self.dev)
        self.free = queue.Queue()
        for _ in range(max(1, int(depth))):
            self.free.put({})
        self.todo = queue.Queue()
        self.error = None
        self.thread = threading.Thread(target=self._run, name="sph-export", daemon=True)
        self.thread.start()

    def submit(self, fields: dict, time: float | None = None, timestep: int = 0, dt: float | None = None,
               group_attrs: dict | None = None) -> bool:
        """Queue one step's arrays (device tensors, read after the work already queued on the
        current stream).  A field named '@name' (a one-element device tensor) becomes the group
        attribute `name` (e.g. '@time', '@dt' kept on the device); time / dt given as numbers
        are written directly.  Only every `interval`-th call is exported; returns whether this
        one is."""
        if self.error is not None:
            raise RuntimeError(f"export failed: {self.error}")
        self.calls += 1
        if (self.calls - 1) % self.interval:
            return False
        slot = self.free.get()          # back-pressure: wait for a free set of pinned buffers
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(ev)
            for k, t in fields.items():
                host = slot.get(k)
                if host is None or host.shape != t.shape or host.dtype != t.dtype:
                    host = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                    slot[k] = host
                host.copy_(t, non_blocking=True)
                t.record_stream(self.copy_stream)   # the caller may free t; keep it until copied
            done = torch.cuda.Event()
            done.record(self.copy_stream)
        for k in list(slot):
            if k not in fields:
                del slot[k]
        attrs = {"timestep": int(timestep)}
        if time is not None:
            attrs["time"] = float(time)
        if dt is not None:
            attrs["dt"] = float(dt)
        attrs.update(group_attrs or {})
        self.todo.put(("simulationExport/%05d" % self.counter, slot, done, attrs))
        self.counter += 1
        return True

    def _run(self):
        while True:
            item = self.todo.get()
            if item is None:
                return
            group, slot, done, attrs = item
            try:
                done.synchronize()
                for k, host in slot.items():
                    if k.startswith("@"):
                        attrs[k[1:]] = host.reshape(-1)[0].item()
                self.w.set_attrs(group, attrs)
                for k, host in slot.items():
                    if not k.startswith("@"):
                        self.w.write(group, k, host.numpy())
            except Exception as e:   # surfaced by the next submit / close
                self.error = repr(e)
            finally:
                self.free.put(slot)

    def close(self):
        self.todo.put(None)
        self.thread.join()
        self.w.close()
        if self.error is not None:
            raise RuntimeError(f"export failed: {self.error}")
