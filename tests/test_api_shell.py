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
