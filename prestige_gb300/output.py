"""Particle-state output: legacy VTK polydata, Gmsh MSH and CSV, written on the host.

The reference anticipates these formats (its .gitignore lists *.vtk, *.msh and *.csv) but has
no writer.  The functions take named arrays in particle-id order (a ParticleSystem's `get`
results, or any arrays of the same shape), so no device code is involved.

  write_vtk(path, pos, fields)   legacy VTK 3.0, binary (big-endian float64), POLYDATA with one
                                 vertex per particle; scalars as SCALARS, n x dim arrays as
                                 VECTORS (2D vectors padded with z = 0)
  write_msh(path, pos, fields)   Gmsh MSH 2.2 (ASCII): one node and one point element (type 15)
                                 per particle, each field as a $NodeData block (1 or 3
                                 components, 2D vectors padded with z = 0), values in %.17g
  write_csv(path, pos, fields)   header x,y[,z],<field>[_x,_y,_z]...; one row per particle
  snapshot(system, names)        positions and the named slices of a ParticleSystem
"""
import numpy as np


def _columns(n, fields):
    out = []
    for name, a in fields.items():
        a = np.asarray(a, np.float64)
        if a.shape[0] != n:
            raise ValueError("field %r has %d rows, positions have %d" % (name, a.shape[0], n))
        out.append((name, a))
    return out


def _points3(pos):
    pos = np.asarray(pos, np.float64)
    if pos.ndim != 2 or pos.shape[1] not in (2, 3):
        raise ValueError("positions must be n x 2 or n x 3")
    if pos.shape[1] == 2:
        pos = np.concatenate([pos, np.zeros((pos.shape[0], 1))], axis=1)
    return pos


def write_vtk(path, pos, fields=None, title="prestige particles"):
    pts = _points3(pos)
    n = pts.shape[0]
    cols = _columns(n, fields or {})
    with open(path, "wb") as f:
        f.write(b"# vtk DataFile Version 3.0\n")
        f.write(title.replace("\n", " ")[:255].encode() + b"\n")
        f.write(b"BINARY\nDATASET POLYDATA\n")
        f.write(b"POINTS %d double\n" % n)
        f.write(pts.astype(">f8").tobytes())
        f.write(b"\nVERTICES %d %d\n" % (n, 2 * n))
        cells = np.empty((n, 2), ">i4")
        cells[:, 0] = 1
        cells[:, 1] = np.arange(n)
        f.write(cells.tobytes())
        if cols:
            f.write(b"\nPOINT_DATA %d\n" % n)
        for name, a in cols:
            tag = name.replace(" ", "_").encode()
            if a.ndim == 1:
                f.write(b"SCALARS %s double 1\nLOOKUP_TABLE default\n" % tag)
                f.write(a.astype(">f8").tobytes())
            elif a.ndim == 2 and a.shape[1] in (2, 3):
                f.write(b"VECTORS %s double\n" % tag)
                f.write(_points3(a).astype(">f8").tobytes())
            else:
                raise ValueError("field %r must be n or n x 2/3" % name)
            f.write(b"\n")


def write_msh(path, pos, fields=None, time=0.0, step=0):
    pts = _points3(pos)
    n = pts.shape[0]
    cols = _columns(n, fields or {})
    ids = np.arange(1, n + 1)
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n")
        f.write("$Nodes\n%d\n" % n)
        np.savetxt(f, np.column_stack([ids, pts]), fmt=["%d", "%.17g", "%.17g", "%.17g"])
        f.write("$EndNodes\n$Elements\n%d\n" % n)
        np.savetxt(f, np.column_stack([ids, np.full(n, 15), np.full(n, 2), np.zeros(n, int), np.ones(n, int), ids]),
                   fmt="%d")
        f.write("$EndElements\n")
        for name, a in cols:
            if a.ndim == 1:
                vals = a[:, None]
            elif a.ndim == 2 and a.shape[1] in (2, 3):
                vals = _points3(a)
            else:
                raise ValueError("field %r must be n or n x 2/3" % name)
            f.write('$NodeData\n1\n"%s"\n1\n%.17g\n3\n%d\n%d\n%d\n' % (name.replace('"', "'"), time, step,
                                                                        vals.shape[1], n))
            np.savetxt(f, np.column_stack([ids, vals]), fmt=["%d"] + ["%.17g"] * vals.shape[1])
            f.write("$EndNodeData\n")


def write_csv(path, pos, fields=None):
    pos = np.asarray(pos, np.float64)
    n, dim = pos.shape
    cols = [pos]
    head = ["x", "y", "z"][:dim]
    for name, a in _columns(n, fields or {}):
        if a.ndim == 1:
            cols.append(a[:, None])
            head.append(name)
        else:
            cols.append(a)
            head += ["%s_%s" % (name, c) for c in "xyz"[:a.shape[1]]]
    np.savetxt(path, np.concatenate(cols, axis=1), delimiter=",", header=",".join(head), comments="", fmt="%.17g")


def snapshot(system, names=("vel", "rho")):
    """(positions, {name: array}) of a ParticleSystem, in particle-id order."""
    return system.get("pos"), {nm: system.get(nm) for nm in names}
