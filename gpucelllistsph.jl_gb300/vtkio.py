"""On-disk results: VTK XML PolyData (.vtp), ParaView collections (.pvd) and
CSV, as the reference writes them.

Reference: `writevtk`/`create_vtp_file` (src/writevtk.jl:1-42) write a .vtp
through WriteVTK.jl (points with empty verts and polys, one point-data array
per requested variable, zlib-compressed inline binary); `timesolve!`
(src/sphproblem.jl:445-503) names frames OUTPUT_00000.vtp, ... and collects
them in OUTPUT_PVC.pvd with the simulated time; `makedf`/`writecsv`
(src/auxillary.jl:24-70) write x, y[, z] and the variables, vector fields as
<name>_x, <name>_y[, <name>_z].

Files are written from host snapshots: `snapshot` copies the requested
fields into pinned host memory on the library's stream (ordered after the
step that produced them, without waiting for it), and `AsyncWriter` writes
them on a background thread while the next steps run on the device.
"""
from __future__ import annotations

import base64
import os
import queue
import struct
import threading
import zlib
from xml.sax.saxutils import quoteattr

import numpy as np

VTKVARS = ("Density", "Pressure", "Type", "Acceleration", "Velocity", "∑W", "∑∇W", "DPC")
_AXES = ("x", "y", "z")


# --------------------------------------------------------------------------- encoding
def _encode(arr: np.ndarray, compress: bool) -> str:
    raw = np.ascontiguousarray(arr).tobytes()
    if not compress:
        return base64.b64encode(struct.pack("<Q", len(raw)) + raw).decode("ascii")
    comp = zlib.compress(raw)
    # vtkZLibDataCompressor, UInt64 header: blocks, block size, last block size, compressed sizes
    head = struct.pack("<4Q", 1, len(raw), len(raw), len(comp))
    return base64.b64encode(head).decode("ascii") + base64.b64encode(comp).decode("ascii")


def decode(text: str, dtype, compressed: bool = True) -> np.ndarray:
    """Inverse of the inline binary encoding (used by the tests and readers)."""
    if not compressed:
        raw = base64.b64decode(text)
        n = struct.unpack("<Q", raw[:8])[0]
        return np.frombuffer(raw[8:8 + n], dtype=dtype)
    head_len = len(base64.b64encode(b"\0" * 32))
    head = base64.b64decode(text[:head_len])
    nblocks, bsize, last, csize = struct.unpack("<4Q", head)
    data = zlib.decompress(base64.b64decode(text[head_len:]))
    assert nblocks == 1 and len(data) == bsize == last
    return np.frombuffer(data, dtype=dtype)


_VTK_TYPES = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32", np.dtype(np.int32): "Int32",
              np.dtype(np.int64): "Int64"}


def _data_array(name: str, arr: np.ndarray, ncomp: int, compress: bool) -> str:
    t = _VTK_TYPES[arr.dtype]
    comp = f' NumberOfComponents="{ncomp}"' if ncomp > 1 else ""
    return (f'        <DataArray type="{t}" Name={quoteattr(name)}{comp} format="binary">'
            f"{_encode(arr, compress)}</DataArray>\n")


def write_vtp(filename: str, points, fields: dict, compress: bool = True) -> str:
    """create_vtp_file (src/writevtk.jl:1-13).  points: D arrays of N
    coordinates (padded to 3-D with zeros, as WriteVTK does); fields: name ->
    array of N (scalar) or tuple/list of D arrays (vector, D components).
    Returns the path written (".vtp" appended if missing)."""
    if not filename.endswith(".vtp"):
        filename += ".vtp"
    pts = [np.asarray(p, dtype=np.float64) for p in points]
    n = pts[0].size
    while len(pts) < 3:
        pts.append(np.zeros(n))
    xyz = np.stack(pts, axis=1).reshape(-1)
    empty = np.zeros(0, dtype=np.int64)
    head = ('<?xml version="1.0" encoding="utf-8"?>\n'
            '<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64"'
            + (' compressor="vtkZLibDataCompressor"' if compress else "") + ">\n"
            "  <PolyData>\n"
            f'    <Piece NumberOfPoints="{n}" NumberOfVerts="0" NumberOfLines="0" NumberOfStrips="0" '
            'NumberOfPolys="0">\n')
    body = ["      <Points>\n", _data_array("Points", xyz, 3, compress), "      </Points>\n",
            "      <PointData>\n"]
    for name, v in fields.items():
        if isinstance(v, (tuple, list)):
            comps = [np.asarray(c) for c in v]
            arr = np.stack(comps, axis=1).reshape(-1)
            body.append(_data_array(name, arr, len(comps), compress))
        else:
            body.append(_data_array(name, np.asarray(v), 1, compress))
    body.append("      </PointData>\n")
    for cells in ("Verts", "Polys"):
        body += [f"      <{cells}>\n", _data_array("connectivity", empty, 1, compress),
                 _data_array("offsets", empty, 1, compress), f"      </{cells}>\n"]
    tail = "    </Piece>\n  </PolyData>\n</VTKFile>\n"
    os.makedirs(os.path.dirname(os.path.abspath(filename)), exist_ok=True)
    with open(filename, "w", encoding="utf-8") as f:
        f.write(head + "".join(body) + tail)
    return filename


def write_pvd(filename: str, entries) -> str:
    """paraview_collection + vtk_save: entries = [(time, vtp path)], paths
    written relative to the collection's directory."""
    if not filename.endswith(".pvd"):
        filename += ".pvd"
    base = os.path.dirname(os.path.abspath(filename))
    lines = ['<?xml version="1.0" encoding="utf-8"?>\n',
             '<VTKFile type="Collection" version="1.0" byte_order="LittleEndian">\n', "  <Collection>\n"]
    for t, path in entries:
        rel = os.path.relpath(os.path.abspath(path), base)
        lines.append(f'    <DataSet timestep="{float(t)!r}" part="0" file={quoteattr(rel)}/>\n')
    lines += ["  </Collection>\n", "</VTKFile>\n"]
    with open(filename, "w", encoding="utf-8") as f:
        f.write("".join(lines))
    return filename


def write_csv(path: str, points, fields: dict) -> str:
    """writecsv/makedf (src/auxillary.jl:24-70): x, y[, z], then each
    variable; vector fields as <name>_x, <name>_y[, <name>_z]."""
    dirn = os.path.dirname(os.path.abspath(path))
    if not os.path.isdir(dirn):
        raise ValueError("Wrong path.")
    cols, names = [], []
    for d, p in enumerate(points):
        cols.append(np.asarray(p, dtype=np.float64))
        names.append(_AXES[d])
    for name, v in fields.items():
        if isinstance(v, (tuple, list)):
            for d, c in enumerate(v):
                cols.append(np.asarray(c, dtype=np.float64))
                names.append(f"{name}_{_AXES[d]}")
        else:
            cols.append(np.asarray(v, dtype=np.float64))
            names.append(name)
    table = np.stack(cols, axis=1)
    with open(path, "w", encoding="utf-8") as f:
        f.write(",".join(names) + "\n")
        np.savetxt(f, table, delimiter=",", fmt="%.17g")
    return path


# --------------------------------------------------------------------------- snapshots
def _device_fields(prob, vtkvars):
    """The getters (src/sphproblem.jl:348-390) of each requested variable,
    as device tensors (vector fields as tuples)."""
    from . import sphproblem as sp
    get = {"Density": sp.get_density, "Pressure": sp.get_pressure, "Type": sp.get_ptype,
           "Acceleration": sp.get_acceleration, "Velocity": sp.get_velocity, "∑W": sp.get_sumw,
           "∑∇W": sp.get_sumgradw, "DPC": sp.get_dpccorr}
    out = {}
    for name in vtkvars:
        if name not in get:
            raise ValueError(f"unknown variable {name!r}; known: {VTKVARS}")
        out[name] = get[name](prob)
    return out


class Snapshot:
    """Fields of one moment, copied into pinned host memory on the current
    stream; `wait()` blocks until the copies have landed."""

    def __init__(self, prob, vtkvars, etime=None):
        import torch
        self.etime = float(prob.etime if etime is None else etime)
        self.points = tuple(self._pin(t) for t in prob.system.points)
        self.fields = {}
        for name, v in _device_fields(prob, vtkvars).items():
            self.fields[name] = tuple(self._pin(t) for t in v) if isinstance(v, tuple) else self._pin(v)
        self.event = torch.cuda.Event()
        self.event.record()

    @staticmethod
    def _pin(t):
        import torch
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        return h

    def wait(self):
        self.event.synchronize()

    def numpy(self):
        self.wait()
        conv = lambda v: tuple(c.numpy() for c in v) if isinstance(v, tuple) else v.numpy()  # noqa: E731
        return [p.numpy() for p in self.points], {k: conv(v) for k, v in self.fields.items()}


def writevtk(prob, filename, vtkvars=("Acceleration", "Velocity", "Pressure"), cpupoints=None, pvd=None,
             writetime=False):
    """writevtk (src/writevtk.jl:30-42): one .vtp of the current state;
    `pvd` (a list) collects (etime, path) when writetime is set."""
    snap = Snapshot(prob, vtkvars)
    pts, fields = snap.numpy()
    if cpupoints is not None:
        pts = [np.asarray(p) for p in cpupoints]
    path = write_vtp(filename, pts, fields)
    if pvd is not None and writetime:
        pvd.append((snap.etime, path))
    return path


def writecsv(prob, path, vtkvars=("Density", "Acceleration", "Velocity")):
    """writecsv (src/auxillary.jl:66-70)."""
    pts, fields = Snapshot(prob, vtkvars).numpy()
    return write_csv(path, pts, fields)


class AsyncWriter:
    """Writes .vtp frames from snapshots on a background thread, so that file
    output overlaps the next steps on the device; `close()` drains it and
    writes the .pvd collection."""

    def __init__(self, path: str, pvc: bool = False, depth: int = 4):
        self.path = path
        self.pvc = pvc
        self.entries = []
        self.q = queue.Queue(maxsize=depth)
        self.err = None
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def _run(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            name, snap = item
            try:
                pts, fields = snap.numpy()
                p = write_vtp(os.path.join(self.path, name), pts, fields)
                self.entries.append((snap.etime, p))
            except Exception as e:  # noqa: BLE001
                self.err = e

    def submit(self, name: str, snap: Snapshot):
        self.q.put((name, snap))

    def close(self):
        self.q.put(None)
        self.t.join()
        if self.err is not None:
            raise self.err
        if self.pvc:
            write_pvd(os.path.join(self.path, "OUTPUT_PVC"), self.entries)
        return self.entries
