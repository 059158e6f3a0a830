"""timesolve! with on-disk output: frames written from pinned snapshots by a
background thread hold exactly the state at the moment they were taken."""
import glob
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_timesolve_writes_vtp_frames_and_collection(gpu_pkg, tmp_path):
    case = gpu_pkg.workloads.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0))
    system = gpu_pkg.GPUCellList(tuple(case.x), case.cellsize, case.dist)
    prob = gpu_pkg.SPHProblem(system, case.dx, case.h, case.H, gpu_pkg.WendlandC2(dim=2), case.rho, case.ptype,
                              case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL)
    seen = []

    def cb(p, i):
        seen.append((i, p.etime, p.rho.cpu().numpy().copy(), np.stack([t.cpu().numpy() for t in p.system.points])))

    gpu_pkg.timesolve(prob, batch=5, timeframe=2e-4, writetime=5e-5, path=str(tmp_path), pvc=True,
                      vtkvars=("Density", "Velocity", "Pressure", "Type"), verbose=False, callback=cb)
    frames = sorted(glob.glob(os.path.join(str(tmp_path), "OUTPUT_*.vtp")))
    assert len(frames) == len(seen) >= 3
    for path, (i, t, rho, x) in zip(frames, seen):
        assert os.path.basename(path) == f"OUTPUT_{i:05d}.vtp"
        piece = ET.parse(path).getroot().find("PolyData/Piece")
        arrs = {el.get("Name"): el for el in piece.find("PointData")}
        dens = gpu_pkg.vtkio.decode(arrs["Density"].text, np.float64)
        assert np.array_equal(dens, rho)
        xyz = gpu_pkg.vtkio.decode(piece.find("Points/DataArray").text, np.float64).reshape(-1, 3)
        assert np.array_equal(xyz[:, 0], x[0]) and np.array_equal(xyz[:, 1], x[1])
        assert np.array_equal(gpu_pkg.vtkio.decode(arrs["Type"].text, np.int32), case.ptype)
    ds = ET.parse(os.path.join(str(tmp_path), "OUTPUT_PVC.pvd")).getroot().findall("Collection/DataSet")
    assert [float(d.get("timestep")) for d in ds] == [t for _, t, _, _ in seen]


def test_writecsv_matches_getters(gpu_pkg, tmp_path):
    case = gpu_pkg.workloads.dam_break_2d(dx=0.05, fluid=(0.5, 0.6), tank=(1.0, 1.0))
    system = gpu_pkg.GPUCellList(tuple(case.x), case.cellsize, case.dist)
    prob = gpu_pkg.SPHProblem(system, case.dx, case.h, case.H, gpu_pkg.WendlandC2(dim=2), case.rho, case.ptype,
                              case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL)
    prob.stepsolve(7)
    path = gpu_pkg.writecsv(prob, str(tmp_path / "out.csv"))
    tab = np.loadtxt(path, delimiter=",", skiprows=1)
    assert np.array_equal(tab[:, 2], gpu_pkg.get_density(prob).cpu().numpy())
    v = gpu_pkg.get_velocity(prob)
    assert np.array_equal(tab[:, 5], v[0].cpu().numpy())
