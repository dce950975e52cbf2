"""Dirichlet conditions as the drivers set them up and move them
(FEM/BOUNDARY_CONDITION.h): the DBC storage holds rows (vertex index, x, y, z)
(the reference's VECTOR_STORAGE<T, dim + 1>), the DBC motion one record per
selected group (row range, velocity, rotation centre, rotation axis, angular
velocity in degrees per second). These are host-side bookkeeping; the rows go
to the Newton step as DBC targets (``Context.set_dbc_targets`` or the Hinge
shim's ``DBC`` argument), where targets away from the vertices' positions are
reached through the augmented Lagrangian on the device.
"""
from __future__ import annotations

import math

import numpy as np

INT_MAX = 2 ** 31 - 1


class DBCStorage:
    """Rows (vertex index, x, y, z) in insertion order."""

    def __init__(self, rows=None):
        self.rows = np.zeros((0, 4)) if rows is None else np.asarray(rows, dtype=np.float64).reshape(-1, 4).copy()

    def __len__(self):
        return self.rows.shape[0]

    def __array__(self, dtype=None, copy=None):
        return self.rows if dtype is None else self.rows.astype(dtype)

    def append(self, vI, x):
        self.rows = np.concatenate([self.rows, [[float(vI), x[0], x[1], x[2]]]])

    @property
    def indices(self):
        return self.rows[:, 0].astype(np.int32)

    @property
    def targets(self):
        return self.rows[:, 1:4]


class DBCMotion(list):
    """Records [range (first row, end row), v, rotCenter, rotAxis, angVelDeg]."""


def init_dirichlet(X, relBoxMin, relBoxMax, v, rotCenter, rotAxis, angVelDeg, DBC, motion,
                   vIndRange=(0, 0, INT_MAX, -1)):
    """Init_Dirichlet (BOUNDARY_CONDITION.h:21-107): the vertices with ids in
    [vIndRange[0], vIndRange[2]) inside the box relBoxMin..relBoxMax, relative
    to those vertices' bounding box, become DBC rows at their positions (in
    vertex order), and one motion record covers them."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    if X.shape[0] == 0:
        raise ValueError("no nodes in the model")
    lo_i, hi_i = int(vIndRange[0]), min(int(vIndRange[2]), X.shape[0])
    sel = X[lo_i:hi_i]
    bmin, bmax = sel.min(0), sel.max(0)
    rmin = np.asarray(relBoxMin, float) * (bmax - bmin) + bmin
    rmax = np.asarray(relBoxMax, float) * (bmax - bmin) + bmin
    first = len(DBC)
    inside = np.all((sel >= rmin) & (sel <= rmax), axis=1)
    for k in np.nonzero(inside)[0]:
        DBC.append(lo_i + int(k), sel[k])
    motion.append([(first, len(DBC)), np.asarray(v, float).copy(), np.asarray(rotCenter, float).copy(),
                   np.asarray(rotAxis, float).copy(), float(angVelDeg)])


def rotation_matrix(angle, axis):
    """Rotation by `angle` about `axis` (taken as a unit vector, as Eigen's
    AngleAxis does): R = c I + (1 - c) a a^T + s [a]_x (Rodrigues)."""
    a = np.asarray(axis, dtype=np.float64)
    c, s = math.cos(angle), math.sin(angle)
    sa, ca = s * a, (1.0 - c) * a
    R = np.empty((3, 3))
    R[0, 1], R[1, 0] = ca[0] * a[1] - sa[2], ca[0] * a[1] + sa[2]
    R[0, 2], R[2, 0] = ca[0] * a[2] + sa[1], ca[0] * a[2] - sa[1]
    R[1, 2], R[2, 1] = ca[1] * a[2] - sa[0], ca[1] * a[2] + sa[0]
    for d in range(3):
        R[d, d] = ca[d] * a[d] + c
    return R


def step_dirichlet(motion, h, DBC):
    """Step_Dirichlet (BOUNDARY_CONDITION.h:110-158): every row of a motion
    record is rotated by angVelDeg * h degrees about (rotCenter, rotAxis), then
    translated by v h."""
    for (r0, r1), v, c, axis, deg in motion:
        if r1 <= r0:
            continue
        t = DBC.rows[r0:r1, 1:4]
        if deg:
            R = rotation_matrix(deg / 180.0 * math.pi * h, axis)
            t[:] = (t - c) @ R.T + c
        t += np.asarray(v) * h


def turn_dirichlet(motion):
    """Turn_Dirichlet (BOUNDARY_CONDITION.h:215-223): every velocity reversed."""
    for rec in motion:
        rec[1] = -rec[1]


def reset_dirichlet(X, DBC):
    """Reset_Dirichlet (BOUNDARY_CONDITION.h:160-173): targets = current positions."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    DBC.rows[:, 1:4] = X[DBC.indices]


def load_dirichlet(filePath, vIndOffset, translate, DBC):
    """Load_Dirichlet (BOUNDARY_CONDITION.h:175-197): targets from the vertices
    of an OBJ file (row vertex - vIndOffset), translated; a file that cannot be
    read leaves the targets unchanged."""
    from . import meshio

    try:
        Y, _, _ = meshio.read_tri_obj(filePath, np.zeros((0, 3)), np.zeros((0, 3), np.int32))
    except OSError:
        return
    targets_from_points(Y, vIndOffset, translate, DBC)


def targets_from_points(Y, vIndOffset, translate, DBC):
    """What Load_Dirichlet does with the vertices it read: row target =
    Y[row vertex - vIndOffset] + translate."""
    DBC.rows[:, 1:4] = np.asarray(Y, float)[DBC.indices - int(vIndOffset)] + np.asarray(translate, float)


def pop_back_dirichlet(motion, DBC):
    """Pop_Back_Dirichlet (BOUNDARY_CONDITION.h:249-265): the last motion
    record and its rows are removed."""
    if not motion:
        return
    (r0, r1) = motion[-1][0]
    DBC.rows = np.concatenate([DBC.rows[:r0], DBC.rows[r1:]])
    motion.pop()


def boundary_nodes(V, tris):
    """Find_Boundary_Edge_And_Node (Utils/MESHIO.h:696-726): vertices of the
    edges whose reverse is in no triangle, ascending."""
    tris = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
    e = tris[:, [[0, 1], [1, 2], [2, 0]]].reshape(-1, 2)
    key = e[:, 0] * V + e[:, 1]
    rev = e[:, 1] * V + e[:, 0]
    bnd = ~np.isin(rev, key)
    mark = np.zeros(V, bool)
    mark[e[bnd].reshape(-1)] = True
    return np.nonzero(mark)[0]


def boundary_dirichlet(X, tris, DBC):
    """Boundary_Dirichlet (BOUNDARY_CONDITION.h:199-213): the open boundary's
    vertices of a triangle mesh become DBC rows at their positions."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    for vI in boundary_nodes(X.shape[0], tris):
        DBC.append(int(vI), X[vI])


def magnify_body_force(X, relBoxMin, relBoxMax, factor, b):
    """Magnify_Body_Force (BOUNDARY_CONDITION.h:225-247): the body force of the
    vertices in the relative box scaled by `factor` (b: V x 3, in place)."""
    rows, motion = DBCStorage(), DBCMotion()
    init_dirichlet(X, relBoxMin, relBoxMax, (0, 0, 0), (0, 0, 0), (0, 0, 0), 0.0, rows, motion)
    b = np.asarray(b).reshape(-1, 3)
    b[rows.indices] *= factor
