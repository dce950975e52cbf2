"""Driver-side Dirichlet bookkeeping (FEM/BOUNDARY_CONDITION.h) restated in
idp_gb300.dirichlet: box selection, motion steps (rotation about an axis then
translation), reversal, reset, OBJ sequences, removal of the last group,
open-boundary vertices and body-force magnification."""
import math

import numpy as np
import pytest

from idp_gb300 import dirichlet, meshio


def grid_points():
    g = np.stack(np.meshgrid(np.arange(3.0), np.arange(3.0), np.arange(5.0), indexing="ij"), -1).reshape(-1, 3)
    return g


def test_init_selects_the_relative_box_in_vertex_order():
    X = grid_points()
    D, M = dirichlet.DBCStorage(), dirichlet.DBCMotion()
    dirichlet.init_dirichlet(X, (0, 0, 0.9), (1, 1, 1), (0, 0, 1), (0, 0, 0), (0, 0, 1), 0.0, D, M)
    top = np.nonzero(X[:, 2] >= 4.0)[0]
    assert np.array_equal(D.indices, top) and np.array_equal(D.targets, X[top])
    assert M[0][0] == (0, len(top))
    # a second group appends rows and a record; an index window restricts the box's reference
    dirichlet.init_dirichlet(X, (0, 0, 0), (1, 1, 0.1), (0, 0, 0), (0, 0, 0), (0, 0, 1), 0.0, D, M,
                             vIndRange=(0, 0, 20, -1))
    sel = X[:20]
    lo, hi = sel.min(0), sel.max(0)
    exp = [k for k in range(20) if sel[k, 2] <= lo[2] + 0.1 * (hi[2] - lo[2])]
    assert list(D.indices[len(top):]) == exp and M[1][0] == (len(top), len(top) + len(exp))


def test_step_rotates_then_translates():
    X = grid_points()
    D, M = dirichlet.DBCStorage(), dirichlet.DBCMotion()
    dirichlet.init_dirichlet(X, (0, 0, 0.9), (1, 1, 1), (0.5, 0, 0), (1, 1, 4), (0, 0, 1), 90.0, D, M)
    t0 = D.targets.copy()
    dirichlet.step_dirichlet(M, 0.5, D)  # 45 degrees about z through (1, 1), then +0.25 in x
    c, s = math.cos(math.pi / 4), math.sin(math.pi / 4)
    R = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])
    exp = (t0 - [1, 1, 4]) @ R.T + [1, 1, 4] + [0.25, 0, 0]
    assert np.allclose(D.targets, exp, rtol=0, atol=1e-14)
    dirichlet.turn_dirichlet(M)
    assert np.array_equal(M[0][1], [-0.5, 0, 0])
    dirichlet.reset_dirichlet(X, D)
    assert np.array_equal(D.targets, X[D.indices])


def test_rotation_matrix_is_orthonormal_about_its_axis():
    a = np.array([1.0, 2.0, 2.0]) / 3.0
    R = dirichlet.rotation_matrix(0.7, a)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-15) and np.allclose(R @ a, a, atol=1e-15)
    assert np.linalg.det(R) == pytest.approx(1.0, abs=1e-14)


def test_load_pop_and_boundary(tmp_path):
    X = grid_points()
    D, M = dirichlet.DBCStorage(), dirichlet.DBCMotion()
    dirichlet.init_dirichlet(X, (0, 0, 0.9), (1, 1, 1), (0, 0, 0), (0, 0, 0), (0, 0, 1), 0.0, D, M)
    dirichlet.init_dirichlet(X, (0, 0, 0), (1, 1, 0.1), (0, 0, 0), (0, 0, 0), (0, 0, 1), 0.0, D, M)
    n_top = M[0][0][1]
    # targets from an OBJ whose vertices are the grid shifted by 2 in z
    tris = np.array([[0, 1, 2]], np.int32)
    p = tmp_path / "shell3.obj"
    meshio.write_tri_obj(p, X + [0, 0, 2.0], tris)
    dirichlet.load_dirichlet(str(p), 0, (0.0, -0.75, 0.0), D)
    assert np.allclose(D.targets, X[D.indices] + [0, -0.75, 2.0])
    dirichlet.load_dirichlet(str(tmp_path / "missing.obj"), 0, (0, 0, 0), D)  # unreadable: unchanged
    dirichlet.pop_back_dirichlet(M, D)
    assert len(D) == n_top and len(M) == 1
    # open boundary of a two-triangle square: every vertex
    F = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    assert list(dirichlet.boundary_nodes(5, F)) == [0, 1, 2, 3]
    B = dirichlet.DBCStorage()
    dirichlet.boundary_dirichlet(np.zeros((5, 3)), F, B)
    assert list(B.indices) == [0, 1, 2, 3]
    b = np.ones((X.shape[0], 3))
    dirichlet.magnify_body_force(X, (0, 0, 0.9), (1, 1, 1), 3.0, b)
    assert np.array_equal(b[:, 0] == 3.0, X[:, 2] >= 4.0)
