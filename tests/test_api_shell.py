"""The reference-shaped Hinge call's elastic-shell storages: the material the
shim reads back from what Initialize_Discrete_Shell fills (element volumes,
Lame parameters, the hinge stiffness in elemAttr P, lumped masses), and the
arguments it refuses."""
import numpy as np
import pytest

import cases


def storages(X0, F, pr, k_mult=1.0):
    import oracle

    mem = oracle.membrane_rest(X0, F, pr["thickness"], pr["E"], pr["nu"])
    IB = np.stack([np.linalg.inv(np.array([[m[0], m[1]], [m[1], m[2]]])) for m in mem])
    P = np.zeros_like(IB)
    P[0, 0, 0] = k_mult * oracle.hinge_stiffness(pr["E"], pr["nu"], pr["thickness"])
    nodeAttr = {"x0": X0.copy(), "v": np.zeros_like(X0), "m": pr["mass"].copy()}
    return nodeAttr, {"IB": IB, "P": P}, {"vol": mem[:, 4], "lambda": mem[:, 5], "mu": mem[:, 6]}


def test_shell_material_recovers_the_initializer_inputs():
    from idp_gb300.api import shell_material

    X0, F = cases.sphere_shell(2)
    pr = cases.shell_problem(X0, F, E=3.2e5, nu=0.37, thickness=0.004, density=800.0)
    nodeAttr, elemAttr, ela = storages(X0, F, pr, k_mult=2.0)
    m = shell_material(F, nodeAttr, elemAttr, ela, 1.5)
    assert m["E"] == pytest.approx(3.2e5, rel=1e-13) and m["nu"] == pytest.approx(0.37, rel=1e-13)
    assert m["thickness"] == pytest.approx(0.004, rel=1e-13) and m["density"] == pytest.approx(800.0, rel=1e-12)
    assert m["bending_mult"] == pytest.approx(3.0, rel=1e-12)  # 1.5 x the stored k's factor 2
    assert m["mass"] is not None and np.array_equal(m["mass"], pr["mass"])


def test_shell_material_rejects_mixed_materials():
    from idp_gb300.api import shell_material

    X0, F = cases.sphere_shell(1)
    pr = cases.shell_problem(X0, F)
    nodeAttr, elemAttr, ela = storages(X0, F, pr)
    ela["mu"] = ela["mu"].copy()
    ela["mu"][3] *= 2
    with pytest.raises(NotImplementedError):
        shell_material(F, nodeAttr, elemAttr, ela, 1.0)
    nodeAttr, elemAttr, ela = storages(X0, F, pr)
    ela["vol"] = ela["vol"].copy()
    ela["vol"][2] *= 1.5
    with pytest.raises(NotImplementedError):
        shell_material(F, nodeAttr, elemAttr, ela, 1.0)


def test_hinge_call_refuses_shells_with_tets():
    from idp_gb300.api import FEM

    X0, F = cases.sphere_shell(1)
    pr = cases.shell_problem(X0, F)
    nodeAttr, elemAttr, ela = storages(X0, F, pr)
    args = [F, [], [], {}, [], [], 0.0, 1.0, [], [], [1.0, 0.0], [1.0, 1.0], [0.0, 0.0], None, 0.1, 1e-3, True,
            pr["dHat2"], [1.0, 1.0, 0.0], 0.0, 1e-10, 0, [], [], False, X0.copy(), nodeAttr, None, elemAttr, ela,
            np.array([[0, 1, 2, 3]], np.int32), None, None, [], [], [], [], [], [], 0.0, [], ""]
    with pytest.raises(NotImplementedError):
        FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*args)
    args[29] = None  # shell elements without elasticityAttr
    args[30] = []
    with pytest.raises(ValueError):
        FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*args)


def rotated_frames(X, n, deg=4.0, shift=0.01, stretch=0.01):
    """Frame k of a character sequence: X turned by k*deg about z, stretched
    along x by 1 + k*stretch and moved by k*shift along x."""
    frames = []
    for k in range(1, n + 1):
        a = np.deg2rad(deg * k)
        R = np.array([[np.cos(a), -np.sin(a), 0.0], [np.sin(a), np.cos(a), 0.0], [0.0, 0.0, 1.0]])
        Y = X @ R.T
        Y[:, 0] = Y[:, 0] * (1 + stretch * k) + shift * k
        frames.append(Y)
    return frames


def test_sequence_frame_sets_rest_shape_velocity_and_targets(tmp_path):
    """The lv_fn sequence step of the shell driver, without a GPU: frame
    lv_fn becomes the rest shape, kappa follows its masses with the default
    multiplier, the velocity points from the current positions to it and
    the DBC rows take its positions as targets."""
    from idp_gb300 import meshio
    from idp_gb300.api import ShellFlowSim, initialize_oipc

    X, F = cases.sphere_shell(2)
    meshio.write_tri_obj(tmp_path / "rest.obj", X, F)
    sim = ShellFlowSim("double", 3)
    sim.add_shell_with_scale_3D(str(tmp_path / "rest.obj"), (0, 0.75, 0), (0.5, 0.5, 0.5), (0, 0, 0), (1, 0, 0), -90)
    Xr, _, _ = meshio.read_tri_obj(tmp_path / "rest.obj")
    Xs = Xr * 0.5
    Xs = np.stack([Xs[:, 0], Xs[:, 2], -Xs[:, 1]], 1) + [0, 0.75, 0]  # -90 degrees about x
    assert np.allclose(sim.X, Xs, atol=1e-12)
    sim.set_DBC((-0.1, 0.8, -0.1), (1.1, 1.1, 1.1), (0, 0, 0), (0, 0, 0), (1, 0, 0), 0)
    sim.initialize(1000, 100, 0.4, 0.01, 0)
    sim.initialize_OIPC(1e-2, 0, 3.0)
    k3 = sim.kappa[0]
    (tmp_path / "seq").mkdir()
    for k, Y in enumerate(rotated_frames(sim.X, 2), 1):
        meshio.write_tri_obj(tmp_path / "seq" / f"{k}.obj", Y, F)
    sim.lv_fn, sim.seqDBCPath, h = 1, str(tmp_path / "seq"), 0.04
    Xc = sim.X.copy()
    v = sim._next_frame_rest_shape(h)
    Y1, _, _ = meshio.read_tri_obj(tmp_path / "seq" / "1.obj")
    assert sim.lv_fn == 2 and np.array_equal(sim._X0, Y1)
    assert np.array_equal(v, (Y1 - Xc) / h)
    rows = sim.DBC.indices
    assert rows.size > 0 and np.array_equal(sim.DBC.targets, Y1[rows])
    k1, km1 = initialize_oipc(float(sim._mass(Y1).mean()), sim.dHat2, 1.0)
    assert sim.kappa[:2] == [k1, km1] and k1 != k3  # the multiplier 3 is not carried over
    bad = tmp_path / "bad"
    bad.mkdir()
    meshio.write_tri_obj(bad / "2.obj", Y1[:-1], F[:1])
    sim.seqDBCPath = str(bad)
    with pytest.raises(ValueError):
        sim._next_frame_rest_shape(h)
