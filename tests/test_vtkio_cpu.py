"""VTK/CSV writers (the reference's writevtk / paraview collection /
writecsv formats) -- written, parsed back and compared, no GPU."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest


def _arrays(path):
    root = ET.parse(path).getroot()
    compressed = root.get("compressor") == "vtkZLibDataCompressor"
    return root, compressed


def _read(pkg, el, compressed):
    dt = {"Float64": np.float64, "Float32": np.float32, "Int32": np.int32, "Int64": np.int64}[el.get("type")]
    return pkg.vtkio.decode(el.text or "", dt, compressed) if el.text else np.zeros(0, dt)


@pytest.mark.parametrize("compress", [True, False])
@pytest.mark.parametrize("D", [2, 3])
def test_vtp_round_trip(pkg, tmp_path, compress, D):
    rng = np.random.default_rng(3)
    n = 257
    pts = [rng.random(n) for _ in range(D)]
    fields = {"Density": 1000 + rng.random(n), "Velocity": tuple(rng.random(n) for _ in range(D)),
              "Type": rng.integers(0, 3, n).astype(np.int32)}
    path = pkg.vtkio.write_vtp(str(tmp_path / "OUTPUT_00000"), pts, fields, compress=compress)
    assert path.endswith(".vtp") and os.path.exists(path)
    root, compressed = _arrays(path)
    assert root.get("type") == "PolyData" and compressed == compress
    piece = root.find("PolyData/Piece")
    assert piece.get("NumberOfPoints") == str(n) and piece.get("NumberOfVerts") == "0"
    xyz = _read(pkg, piece.find("Points/DataArray"), compressed).reshape(n, 3)
    for d in range(3):
        want = pts[d] if d < D else np.zeros(n)
        assert np.array_equal(xyz[:, d], want)
    got = {el.get("Name"): el for el in piece.find("PointData")}
    assert np.array_equal(_read(pkg, got["Density"], compressed), fields["Density"])
    assert got["Velocity"].get("NumberOfComponents") == str(D)
    vel = _read(pkg, got["Velocity"], compressed).reshape(n, D)
    for d in range(D):
        assert np.array_equal(vel[:, d], fields["Velocity"][d])
    assert np.array_equal(_read(pkg, got["Type"], compressed), fields["Type"])


def test_pvd_collection(pkg, tmp_path):
    a = pkg.vtkio.write_vtp(str(tmp_path / "OUTPUT_00000"), [np.zeros(2), np.ones(2)], {})
    b = pkg.vtkio.write_vtp(str(tmp_path / "OUTPUT_00003"), [np.zeros(2), np.ones(2)], {})
    p = pkg.vtkio.write_pvd(str(tmp_path / "OUTPUT_PVC"), [(0.0, a), (1.5e-4, b)])
    root = ET.parse(p).getroot()
    ds = root.findall("Collection/DataSet")
    assert [d.get("file") for d in ds] == ["OUTPUT_00000.vtp", "OUTPUT_00003.vtp"]
    assert [float(d.get("timestep")) for d in ds] == [0.0, 1.5e-4]


def test_csv_columns(pkg, tmp_path):
    rng = np.random.default_rng(5)
    pts = [rng.random(9), rng.random(9)]
    fields = {"Density": rng.random(9), "Acceleration": (rng.random(9), rng.random(9))}
    path = pkg.vtkio.write_csv(str(tmp_path / "out.csv"), pts, fields)
    with open(path) as f:
        head = f.readline().strip().split(",")
    assert head == ["x", "y", "Density", "Acceleration_x", "Acceleration_y"]
    tab = np.loadtxt(path, delimiter=",", skiprows=1)
    assert np.array_equal(tab[:, 0], pts[0]) and np.array_equal(tab[:, 3], fields["Acceleration"][0])
    with pytest.raises(ValueError):
        pkg.vtkio.write_csv(str(tmp_path / "missing" / "out.csv"), pts, fields)
