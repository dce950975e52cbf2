"""The driver methods of FEMDiscreteShellBase that prepare a step on the host
(Python/Drivers/FEMDiscreteShellBase.py:142-299): the tets' gravity body
force, Adjust_Material, Magnify_Body_Force, the DBC pop-back and second
motion list, load_frame, load_velocity and add_mannequin, each against the
reference's formula written out here."""
import numpy as np
import pytest

import cases


def two_bars():
    from idp_gb300 import meshgen
    from idp_gb300.api import TetIPCSim

    sim = TetIPCSim()
    Xa, Ta = meshgen.bar(2, 2, 4, size=(1.0, 1.0, 2.0), seed=0)
    c0 = sim.add_object_3D(Xa, Ta)
    c1 = sim.add_object_3D(Xa + [2.0, 0.0, 0.0], Ta)
    return sim, c0, c1


def test_tet_gravity_body_force_and_material_scaling():
    sim, c0, c1 = two_bars()
    sim.initialize_added_objects((0.0, 0.0, 0.0), 1000.0, 1e4, 0.3)
    # Augment_Mass_Matrix_And_Body_Force: b[v] += vol * rho / 4 * g per tet corner, tets in order
    b = np.zeros_like(sim.X)
    for t in sim.tet:
        d = sim.X[t[1:]] - sim.X[t[0]]
        each = np.dot(d[0], np.cross(d[1], d[2])) / 6.0 * 1000.0 / 4.0
        for v in t:
            b[v] += each * np.array([0.0, -9.81, 0.0])
    assert np.allclose(sim.bodyForce, b, rtol=1e-14, atol=0)
    assert np.allclose(sim.bodyForce[:, 1], -9.81 * sim.nodeAttr["m"], rtol=1e-13)
    m0, b0 = sim.nodeAttr["m"].copy(), sim.bodyForce.copy()
    lam0, mu0 = sim.tetElasticity["lambda"].copy(), sim.tetElasticity["mu"].copy()
    sim.adjust_material(c1, 2.0, 5.0)
    v0, t0, v1, t1 = c1
    assert np.array_equal(sim.nodeAttr["m"][:v0], m0[:v0]) and np.array_equal(sim.nodeAttr["m"][v0:v1], 2 * m0[v0:v1])
    assert np.array_equal(sim.bodyForce[v0:v1], 2 * b0[v0:v1]) and np.array_equal(sim.bodyForce[:v0], b0[:v0])
    assert np.array_equal(sim.tetElasticity["lambda"][t0:t1], 5 * lam0[t0:t1])
    assert np.array_equal(sim.tetElasticity["mu"][:t0], mu0[:t0])
    # Magnify_Body_Force: the vertices in the relative box (the right bar) scaled
    b1 = sim.bodyForce.copy()
    sim.magnify_body_force((0.6, -0.1, -0.1), (1.1, 1.1, 1.1), 3.0)
    right = sim.X[:, 0] >= 0.6 * 3.0
    assert np.array_equal(sim.bodyForce[right], 3 * b1[right]) and np.array_equal(sim.bodyForce[~right], b1[~right])
    sim2, _, _ = two_bars()
    sim2.gravity = (0.0, 0.0, 0.0)
    sim2.initialize_added_objects((0.0, 0.0, 0.0), 1000.0, 1e4, 0.3)
    assert not np.any(sim2.bodyForce)


def test_pop_back_and_second_motion():
    """Pop_Back_Dirichlet removes the last motion's rows while the window is
    open; the second motion list steps its own rows in its own window."""
    sim, c0, c1 = two_bars()
    sim.set_DBC((-0.1, -0.1, -0.1), (0.4, 1.1, 0.1), (0, 0, 0), (0, 0, 0), (1, 0, 0), 0)  # left bar's bottom
    n_fixed = len(sim.DBC)
    sim.set_DBC((0.6, -0.1, 0.9), (1.1, 1.1, 1.1), (0, 1.0, 0), (0, 0, 0), (1, 0, 0), 0)  # right bar's top
    n_top = len(sim.DBC) - n_fixed
    sim.set_DBC2_with_range((-0.1, -0.1, 0.9), (1.1, 1.1, 1.1), (0, 0, -2.0), (0, 0, 0), (1, 0, 0), 0,
                            (0, 0, c0[2], -1))  # the left bar's top, second list
    assert n_fixed > 0 and n_top > 0 and len(sim.DBCMotion2) == 1
    r2 = sim.DBCMotion2[0][0]
    start = sim.DBC.rows.copy()
    sim.MDBC_tmin2, sim.MDBC_tmax2 = -1.0, 10.0
    sim._step_dbc(0.1)  # t = 0: both lists step, no pop-back yet (window closed)
    assert np.allclose(sim.DBC.rows[n_fixed:n_fixed + n_top, 2], start[n_fixed:n_fixed + n_top, 2] + 0.1)
    assert np.allclose(sim.DBC.rows[r2[0]:r2[1], 3], start[r2[0]:r2[1], 3] - 0.2)
    assert np.array_equal(sim.DBC.rows[:n_fixed], start[:n_fixed])
    # pop the last motion of the first list (the right bar's top) once
    sim.DBCPopBackAmt, sim.DBCPopBackTStart, sim.DBCPopBackTEnd = 1, -1.0, 10.0
    sim.MDBC_tmax2 = -2.0  # second list's window closed from here on
    before = sim.DBC.rows.copy()
    sim._step_dbc(0.1)
    assert len(sim.DBCMotion) == 1 and sim.DBCPopBackCounter == 1
    assert len(sim.DBC) == n_fixed + (r2[1] - r2[0])
    assert np.array_equal(sim.DBC.rows[:n_fixed], before[:n_fixed])
    sim._step_dbc(0.1)  # the amount is reached: nothing more is removed
    assert len(sim.DBCMotion) == 1 and sim.DBCPopBackFrameCounter == 1


def test_load_frame_velocity_and_mannequin(tmp_path):
    from idp_gb300 import meshio
    from idp_gb300.api import ShellFlowSim

    X, F = cases.sphere_shell(1)
    meshio.write_tri_obj(tmp_path / "s.obj", X, F)
    sim = ShellFlowSim("double", 3)
    sim.add_shell_3D(str(tmp_path / "s.obj"), (0, 0, 0), (0, 0, 0), (1, 0, 0), 0)
    n0 = sim.X.shape[0]
    cnt = sim.add_mannequin(str(tmp_path / "s.obj"), (3.0, 0, 0), (1, 1, 1), (0, 0, 0), (1, 0, 0), 0)
    assert cnt[0] == n0 and cnt[2] == 2 * n0
    assert np.array_equal(sim.DBC.indices, np.arange(n0, 2 * n0))  # every mannequin vertex, nothing else
    assert np.array_equal(sim.DBC.targets, sim.X[n0:])
    assert np.allclose(sim.X[n0:], sim.X[:n0] + [3.0, 0, 0], atol=1e-9)  # moved by 1e6 and back
    sim.initialize(1000, 100, 0.4, 0.01, 0)
    assert np.array_equal(sim.bodyForce, sim._mass()[:, None] * np.array([0.0, -9.81, 0.0])[None, :])
    sim.initialize(1000, 100, 0.4, 0.01, 1)  # caseI != 0: no gravity
    assert not np.any(sim.bodyForce)
    # load_frame: positions from the file, DBC targets reset to them
    Y = sim.X + 0.01
    meshio.write_tri_obj(tmp_path / "f.obj", Y, sim.Elem)
    sim.load_frame(str(tmp_path / "f.obj"))
    Yr, _, _ = meshio.read_tri_obj(tmp_path / "f.obj")
    assert np.array_equal(sim.X, Yr) and np.array_equal(sim.DBC.targets, Yr[sim.DBC.indices])
    # load_velocity: (frame k - frame k-1) / h
    (tmp_path / "seq").mkdir()
    meshio.write_tri_obj(tmp_path / "seq" / "4.obj", Yr, sim.Elem)
    meshio.write_tri_obj(tmp_path / "seq" / "5.obj", Yr * 1.5, sim.Elem)
    sim.load_velocity(str(tmp_path / "seq"), 5, 0.5)
    Y4, _, _ = meshio.read_tri_obj(tmp_path / "seq" / "4.obj")
    Y5, _, _ = meshio.read_tri_obj(tmp_path / "seq" / "5.obj")
    assert np.array_equal(sim._v_next, (Y5 - Y4) / 0.5)
    with pytest.raises(ValueError):
        sim.load_frame(str(tmp_path / "s.obj"))  # another node count
