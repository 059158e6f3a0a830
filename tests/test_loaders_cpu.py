"""Particle loaders for the reference's CSV layout (quoted header, ParaView
point columns) -- written here in that layout, read back, no GPU."""
import numpy as np


def _write(path, names, rows):
    with open(path, "w") as f:
        f.write(",".join(f'"{n}"' for n in names) + "\n")
        for r in rows:
            f.write(",".join(repr(float(v)) if not float(v).is_integer() else str(int(v)) for v in r) + "\n")


def test_loadparticles_and_case(pkg, tmp_path):
    names_f = ["Idp", "Vel:0", "Vel:1", "Vel:2", "Rhop", "Press", "Type", "Points:0", "Points:1", "Points:2",
               "ptype"]
    names_b = ["Idp", "Vel:0", "Vel:1", "Vel:2", "Rhop", "Type", "Points:0", "Points:1", "Points:2", "ptype"]
    fl = [[i, 0, 0, 0, 1002.5 - i * 0.1, 19031, 3, 0.06 + 0.02 * i, 0, 0.06, 2] for i in range(5)]
    bd = [[i, 0, 0, 0, 1000.0, 0, 0.01 * i, 0, -0.02, 1 if i < 2 else 0] for i in range(4)]
    _write(tmp_path / "f.csv", names_f, fl)
    _write(tmp_path / "b.csv", names_b, bd)
    w = pkg.workloads
    x, F, B = w.loadparticles(str(tmp_path / "f.csv"), str(tmp_path / "b.csv"))
    assert x.shape == (2, 9)
    assert np.array_equal(x[0], [r[7] for r in fl] + [r[6] for r in bd])
    assert np.array_equal(x[1], [r[9] for r in fl] + [r[8] for r in bd])
    assert np.array_equal(F["Rhop"], [r[4] for r in fl])
    case = w.case_from_csv(str(tmp_path / "f.csv"), str(tmp_path / "b.csv"), dx=0.02)
    assert case.ptype.tolist() == [2] * 5 + [1, 1, 0, 0]
    assert np.allclose(case.H, 2 * 1.2 * np.sqrt(2) * 0.02) and case.dist == case.H
    x3, _, _ = w.loadparticles(str(tmp_path / "f.csv"), str(tmp_path / "b.csv"),
                               fluidcols=("Points:0", "Points:2", "Points:1"),
                               boundarycols=("Points:0", "Points:2", "Points:1"))
    assert x3.shape == (3, 9)
