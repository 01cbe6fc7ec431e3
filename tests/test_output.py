"""Host-side VTK, Gmsh MSH and CSV writers of particle state (prestige_gb300.output); no GPU."""
import numpy as np

from prestige_gb300 import output


def _read_vtk(path):
    data = open(path, "rb").read()
    head, rest = data.split(b"POINTS ", 1)
    assert head.startswith(b"# vtk DataFile Version 3.0\n") and b"BINARY\nDATASET POLYDATA\n" in head
    line, rest = rest.split(b"\n", 1)
    n = int(line.split()[0])
    pts = np.frombuffer(rest[:24 * n], ">f8").reshape(n, 3)
    out = {"points": pts}
    rest = rest[24 * n:]
    assert rest.startswith(b"\nVERTICES %d %d\n" % (n, 2 * n))
    rest = rest[len(b"\nVERTICES %d %d\n" % (n, 2 * n)):]
    cells = np.frombuffer(rest[:8 * n], ">i4").reshape(n, 2)
    assert (cells[:, 0] == 1).all() and (cells[:, 1] == np.arange(n)).all()
    rest = rest[8 * n:]
    if rest.startswith(b"\nPOINT_DATA"):
        rest = rest.split(b"\n", 2)[2]
        while rest:
            line, rest = rest.split(b"\n", 1)
            kind, name = line.split()[:2]
            if kind == b"SCALARS":
                rest = rest.split(b"\n", 1)[1]  # LOOKUP_TABLE
                out[name.decode()] = np.frombuffer(rest[:8 * n], ">f8")
                rest = rest[8 * n + 1:]
            else:
                out[name.decode()] = np.frombuffer(rest[:24 * n], ">f8").reshape(n, 3)
                rest = rest[24 * n + 1:]
    return out


def test_vtk_round_trip_3d(tmp_path):
    rng = np.random.default_rng(0)
    pos = rng.normal(size=(57, 3))
    vel = rng.normal(size=(57, 3))
    rho = rng.uniform(990, 1010, size=57)
    p = str(tmp_path / "a.vtk")
    output.write_vtk(p, pos, {"vel": vel, "rho": rho})
    back = _read_vtk(p)
    assert np.array_equal(back["points"], pos)
    assert np.array_equal(back["vel"], vel)
    assert np.array_equal(back["rho"], rho)


def test_vtk_2d_pads_z(tmp_path):
    pos = np.arange(10.0).reshape(5, 2)
    p = str(tmp_path / "b.vtk")
    output.write_vtk(p, pos, {"vel": pos * 2})
    back = _read_vtk(p)
    assert np.array_equal(back["points"][:, :2], pos) and np.all(back["points"][:, 2] == 0)
    assert np.array_equal(back["vel"][:, :2], pos * 2)


def test_csv_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    pos = rng.normal(size=(9, 2))
    rho = rng.normal(size=9)
    p = str(tmp_path / "c.csv")
    output.write_csv(p, pos, {"rho": rho, "vel": pos})
    head = open(p).readline().strip()
    assert head == "x,y,rho,vel_x,vel_y"
    back = np.loadtxt(p, delimiter=",", skiprows=1)
    assert np.array_equal(back[:, :2], pos) and np.array_equal(back[:, 2], rho)


def test_rejects_mismatched_rows(tmp_path):
    import pytest
    with pytest.raises(ValueError):
        output.write_vtk(str(tmp_path / "d.vtk"), np.zeros((4, 3)), {"rho": np.zeros(5)})


def _read_msh(path):
    lines = open(path).read().split("\n")
    assert lines[0] == "$MeshFormat" and lines[1] == "2.2 0 8"
    i = lines.index("$Nodes")
    n = int(lines[i + 1])
    nodes = np.array([[float(v) for v in l.split()] for l in lines[i + 2:i + 2 + n]])
    assert lines[i + 2 + n] == "$EndNodes"
    j = lines.index("$Elements")
    assert int(lines[j + 1]) == n
    el = np.array([[int(v) for v in l.split()] for l in lines[j + 2:j + 2 + n]])
    assert (el[:, 1] == 15).all() and (el[:, 5] == np.arange(1, n + 1)).all()
    out = {"ids": nodes[:, 0], "points": nodes[:, 1:]}
    k = j + 2 + n
    while True:
        try:
            k = lines.index("$NodeData", k)
        except ValueError:
            break
        name = lines[k + 2].strip('"')
        comps, count = int(lines[k + 7]), int(lines[k + 8])
        out[name] = np.array([[float(v) for v in l.split()[1:]] for l in lines[k + 9:k + 9 + count]])
        if comps == 1:
            out[name] = out[name][:, 0]
        assert lines[k + 9 + count] == "$EndNodeData"
        k += 9 + count
    return out


def test_msh_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    pos = rng.normal(size=(23, 3))
    vel = rng.normal(size=(23, 3))
    rho = rng.uniform(990, 1010, size=23)
    p = str(tmp_path / "c.msh")
    output.write_msh(p, pos, {"vel": vel, "rho": rho}, time=0.5, step=7)
    back = _read_msh(p)
    assert np.array_equal(back["ids"], np.arange(1, 24))
    assert np.array_equal(back["points"], pos)
    assert np.array_equal(back["vel"], vel)
    assert np.array_equal(back["rho"], rho)


def test_msh_2d_pads_z(tmp_path):
    pos = np.arange(12.0).reshape(6, 2)
    p = str(tmp_path / "d.msh")
    output.write_msh(p, pos, {"v": pos})
    back = _read_msh(p)
    assert np.array_equal(back["points"][:, :2], pos) and np.all(back["points"][:, 2] == 0)
    assert np.array_equal(back["v"][:, :2], pos) and np.all(back["v"][:, 2] == 0)
