"""Mesh files of the reference's drivers (host side, numpy only).

Restates the readers and writers of ``Library/Utils/MESHIO.h`` that the
tet and shell scripts use, so their input files load unchanged:

* ``read_tri_obj``  — Read_TriMesh_Obj (MESHIO.h:17-80): ``v`` lines give
  positions; an ``f`` line gives the first integer of each of its first three
  vertex tokens (``7``, ``7/3`` and ``7/3/2`` all mean vertex 7), and a fourth
  token makes it a quad split into (0, 1, 2) and (0, 2, 3).
* ``read_tet_vtk``  — Read_TetMesh_Vtk (MESHIO.h:277-339): legacy ASCII VTK,
  the ``POINTS`` block then the ``CELLS`` block (``4 a b c d`` per line),
  reading stops at ``CELL_TYPES``.
* ``write_tri_obj`` — Write_TriMesh_Obj (MESHIO.h:184-213), ``%le`` positions.
* ``write_tet_vtk`` — Write_TetMesh_Vtk (MESHIO.h:403-452), cell type 10; positions
  are written as shortest round-trip decimals (the reference's stream keeps six
  significant digits), so a written mesh reads back bit for bit.
* ``transform_points`` — Transform_Points (MESHIO.h:836-870): scale about a
  centre, rotate about an axis through it, translate.

Like the reference, the readers append to existing arrays and return the
counters (first vertex, first element, vertex count, element count).
"""
from __future__ import annotations

import math

import numpy as np


def _face_indices(line):
    """The reference's scan of an ``f`` line: skip to a digit, read the
    number, skip to the next space; three times, then a possible fourth."""
    n = len(line)
    pos = 0
    out = []
    for _ in range(3):
        while pos < n and not line[pos].isdigit():
            pos += 1
        val = 0
        while pos < n and line[pos].isdigit():
            val = val * 10 + ord(line[pos]) - 48
            pos += 1
        out.append(val - 1)
        while pos < n and line[pos] != " ":
            pos += 1
    while pos < n and not line[pos].isdigit():
        pos += 1
    quad = None
    if pos < n:
        val = 0
        while pos < n and line[pos].isdigit():
            val = val * 10 + ord(line[pos]) - 48
            pos += 1
        quad = val - 1
    return out, quad


def read_tri_obj(path, X=None, faces=None):
    """(X, faces, counter): X (V,3) float64 and faces (F,3) int32 with the
    file's vertices and faces appended to the given arrays (indices offset
    by the vertices already present)."""
    X0 = np.zeros((0, 3)) if X is None else np.asarray(X, dtype=np.float64).reshape(-1, 3)
    F0 = np.zeros((0, 3), np.int32) if faces is None else np.asarray(faces, dtype=np.int32).reshape(-1, 3)
    base_v, base_f = X0.shape[0], F0.shape[0]
    with open(path) as f:
        lines = f.read().splitlines()
    # v lines: the first three numbers after "v " (correctly rounded, as float())
    vt = [line.split()[1:4] for line in lines if line.startswith("v ")]
    pts = np.array(vt, dtype=np.float64).reshape(-1, 3)
    flines = [line for line in lines if line.startswith("f")]
    tris = _plain_triangles(flines)
    if tris is None:  # slashes, quads or other forms: the reference's scan, line by line
        out = []
        for line in flines:
            tri, quad = _face_indices(line)
            out.append(tri)
            if quad is not None:
                out.append([tri[0], tri[2], quad])
        tris = np.asarray(out, dtype=np.int64).reshape(-1, 3)
    Xn = np.vstack([X0, pts])
    Fn = np.vstack([F0, (tris + base_v).astype(np.int32)])
    return Xn, Fn, (base_v, base_f, Xn.shape[0], Fn.shape[0])


def _plain_triangles(flines):
    """Zero-based indices of face lines that are all "f i j k", single
    spaces, positive integers (what _face_indices gives for them), else None."""
    ft = [line.split() for line in flines]
    if not all(len(t) == 4 and " ".join(t) == line for t, line in zip(ft, flines)):
        return None
    try:
        tris = np.array([t[1:] for t in ft], dtype=np.int64).reshape(-1, 3)
    except ValueError:
        return None
    if tris.size and tris.min() < 1:
        return None
    return tris - 1


def read_tet_vtk(path, X=None, tets=None):
    """(X, tets, counter) from a legacy ASCII VTK tet mesh."""
    X0 = np.zeros((0, 3)) if X is None else np.asarray(X, dtype=np.float64).reshape(-1, 3)
    T0 = np.zeros((0, 4), np.int32) if tets is None else np.asarray(tets, dtype=np.int32).reshape(-1, 4)
    base_v, base_t = X0.shape[0], T0.shape[0]
    pts, cells = [], []
    reading_points = reading_cells = False
    n_points = n_cells = 0
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line:
                continue
            if line.startswith("POINTS"):
                reading_points, reading_cells = True, False
                n_points = int(line.split()[1])
            elif line.startswith("CELLS"):
                reading_points, reading_cells = False, True
                n_cells = int(line.split()[1])
            elif line.startswith("CELL_TYPES"):
                reading_points = reading_cells = False
            elif reading_points:
                v = line.split()
                pts.append([float(v[0]), float(v[1]), float(v[2])])
            elif reading_cells:
                v = line.split()
                cells.append([int(v[1]) + base_v, int(v[2]) + base_v, int(v[3]) + base_v, int(v[4]) + base_v])
    if len(pts) != n_points or len(cells) != n_cells:
        raise ValueError(f"{path}: {len(pts)} points / {len(cells)} cells read, header says {n_points} / {n_cells}")
    Xn = np.vstack([X0, np.asarray(pts, dtype=np.float64).reshape(-1, 3)])
    Tn = np.vstack([T0, np.asarray(cells, dtype=np.int32).reshape(-1, 4)])
    return Xn, Tn, (base_v, base_t, Xn.shape[0], Tn.shape[0])


def write_tri_obj(path, X, faces):
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    faces = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    with open(path, "w") as f:
        for x in X:
            f.write("v %e %e %e\n" % (x[0], x[1], x[2]))
        for t in faces:
            f.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))


def write_tet_vtk(path, X, tets):
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    tets = np.asarray(tets, dtype=np.int64).reshape(-1, 4)
    if X.shape[0] == 0 or tets.shape[0] == 0:
        raise ValueError("empty tet mesh")
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 2.0\nUnstructured Grid\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write(f"POINTS {X.shape[0]} double\n")
        for x in X.tolist():  # shortest round-trip decimal of each double
            f.write(f"{x[0]!r} {x[1]!r} {x[2]!r}\n")
        f.write(f"\nCELLS {tets.shape[0]} {5 * tets.shape[0]}\n")
        for t in tets:
            f.write(f"4 {t[0]} {t[1]} {t[2]} {t[3]}\n")
        f.write(f"\nCELL_TYPES {tets.shape[0]}\n")
        f.write("10\n" * tets.shape[0])


def transform_points(X, translate, rot_center, rot_axis, rot_deg, scale, counter=None):
    """Transform_Points: x <- R(axis, deg) (scale * (x - c)) + c + t on the
    rows [counter[0], counter[2]) (all rows when counter is None), in place."""
    X = np.asarray(X)
    lo, hi = (0, X.shape[0]) if counter is None else (counter[0], counter[2])
    a = np.asarray(rot_axis, dtype=np.float64)
    nrm = float(np.linalg.norm(a))
    a = a / nrm if nrm > 0 else np.array([1.0, 0.0, 0.0])
    th = rot_deg / 180.0 * math.pi
    K = np.array([[0.0, -a[2], a[1]], [a[2], 0.0, -a[0]], [-a[1], a[0], 0.0]])
    R = np.eye(3) + math.sin(th) * K + (1.0 - math.cos(th)) * (K @ K)  # Rodrigues
    c = np.asarray(rot_center, dtype=np.float64)
    x = (X[lo:hi] - c) * np.asarray(scale, dtype=np.float64)
    X[lo:hi] = x @ R.T + c + np.asarray(translate, dtype=np.float64)
    return X
