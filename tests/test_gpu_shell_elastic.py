"""Elastic triangle shells of the Hinge path (neo-Hookean membrane + hinge
bending, with offset-IPC self-contact) on the GB300 against the oracle,
through the C ABI: energy and gradient within 1e-9 relative, assembled
Hessian times a vector within 1e-9 (FP64) / 2e-4 (mixed), constraint sets
bit for bit, whole steps (two spheres expanding into each other) to the
oracle's energy within 1e-6, and a buckling sphere pressed flat through
itself to a converged oracle solution; the reference-shaped Hinge call with
shell elements gives the direct C-ABI calls' results bit for bit; a character
sequence (each frame the next rest shape and DBC target) against the oracle."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def shell_ctx(idp, X0, F, pr, mode, v=None, X=None, dbc=None, **kw):
    ctx = idp.Context(h=0.1, mode=mode, **kw)
    ctx.add_elastic_shell_instance(X0 if X is None else X, F, pr["density"], pr["E"], pr["nu"], pr["thickness"],
                                   pr["dHat2"], pr["kappa"], pr["kappa_max"], X0=X0, dbc_idx=dbc)
    if v is not None:
        ctx.set_velocity(0, v)
    ctx.commit()
    return ctx


def shell_oracle(O, X0, F, pr, v, X=None, dbc=None, tol=1e-3):
    surf = O.shell_surface(X0.shape[0], F)
    hin, info = O.shell_hinges(X0, F, surf["edges"])
    k = O.hinge_stiffness(pr["E"], pr["nu"], pr["thickness"])
    hinfo = info.copy()
    mask = np.zeros(X0.shape[0], np.uint8)
    if dbc is not None:
        mask[dbc] = 1
    pb = O.Problem(X=(X0 if X is None else X).copy(), X0=X0, tets=np.zeros((0, 4), np.int32), mass=pr["mass"],
                   lam=np.zeros(0), mu=np.zeros(0), h=0.1, dHat2=pr["dHat2"], kappa=[pr["kappa"], pr["kappa_max"], 0.0],
                   v=v.copy(), faces=F, mem=O.membrane_rest(X0, F, pr["thickness"], pr["E"], pr["nu"]), hinges=hin,
                   hinfo=hinfo, kbend=k, dbc=mask, tol=tol)
    pb.surf = surf
    return pb


def two_spheres(levels=3, gap=0.01, grow=1.08):
    """Two spheres 0.01 apart (inside d-hat 0.02) whose predictor expands each
    by 8 % about its centre: they flatten against each other (about 50
    constraints at the end). The step has one minimum: a perturbed start
    reaches it too."""
    Xa, F = cases.sphere_shell(levels, seed=0, noise=0.01)
    Xb, _ = cases.sphere_shell(levels, seed=1, noise=0.01)
    Xb = Xb + np.array([2.0 + gap, 0.0, 0.0])
    X0 = np.concatenate([Xa, Xb])
    FF = np.concatenate([F, F + Xa.shape[0]]).astype(np.int32)
    c = np.concatenate([np.zeros_like(Xa), np.tile([2.0 + gap, 0.0, 0.0], (Xb.shape[0], 1))])
    pr = cases.shell_problem(X0, FF, dHat=0.02)
    return X0, FF, pr, (c + grow * (X0 - c) - X0) / 0.1


def pressed_sphere():
    X0, F = cases.sphere_shell(3)
    pr = cases.shell_problem(X0, F, dHat=0.02)
    tgt = X0 * np.array([1.0, 1.0, 0.05])  # flattened through itself
    return X0, F, pr, (tgt - X0) / 0.1


def test_mass_and_surface_match(oracle, gpu_lib):
    import idp_gb300 as idp

    X0, F, pr, v = pressed_sphere()
    ctx = shell_ctx(idp, X0, F, pr, idp.MODE_FP64, v=v)
    s = ctx.surface(0)
    o = oracle.shell_surface(X0.shape[0], F)
    assert np.array_equal(s["edges"], o["edges"]) and np.array_equal(s["tris"], o["tris"])
    ctx.close()


@pytest.mark.parametrize("mode,tol", [(0, 1e-9), (1, 2e-4)], ids=["fp64", "mixed"])
def test_energy_gradient_hessian_parity(oracle, gpu_lib, mode, tol):
    import idp_gb300 as idp

    X0, F, pr, v = pressed_sphere()
    # flattened to 1 % of its height: the caps are within d-hat, no edge
    # crosses a face
    rng = np.random.default_rng(4)
    X = X0 * np.array([1.0, 1.0, 0.01]) + 5e-4 * rng.normal(size=X0.shape)
    dbc = np.arange(0, X0.shape[0], 11, dtype=np.int32)
    ctx = shell_ctx(idp, X0, F, pr, mode, v=v, dbc=dbc)
    pb = shell_oracle(oracle, X0, F, pr, v, X=X, dbc=dbc)
    assert len(oracle.edge_tri_intersections(X, pb.surf)) == 0
    xt = X0 + 0.1 * v
    cons, info = oracle.constraint_set(X, X0, pb.surf, pb.dbc, pr["dHat2"])
    assert len(cons) > 1000
    gc = ctx.constraint_set(0, X)
    assert sorted(map(tuple, gc.tolist())) == sorted(map(tuple, cons.tolist()))
    Ee, Ei, Eb = ctx.energy(0, X)
    E_or = oracle._energy(pb, X, xt, False, cons, info) - 0.5 * float(np.sum(pr["mass"][:, None] * (X - xt) ** 2))
    assert Ee == pytest.approx(E_or, rel=1e-9) and E_or > 0
    Eb_or = oracle.barrier_energy(cons, info, X, X0, pr["dHat2"], pr["kappa"])
    assert Eb == pytest.approx(Eb_or, rel=1e-9) and Eb_or > 0
    g = ctx.gradient(0, X)
    go = oracle._gradient(pb, X, xt, cons, info)
    go.reshape(-1, 3)[dbc] = 0
    assert np.linalg.norm(g - go) <= 1e-9 * np.linalg.norm(go)
    H = oracle._hessian(pb, X, cons, info)
    for _ in range(2):
        x = rng.normal(size=X.size)
        y, yo = ctx.hessian_apply(0, X, x), H @ x
        assert np.linalg.norm(y - yo) <= tol * np.linalg.norm(yo)
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_sphere_contact_step_matches_oracle(oracle, gpu_lib, mode):
    """Two expanding spheres pressed against each other: the step ends with
    contact constraints active, injective, at the oracle's energy within 1e-6
    relative and at the oracle's positions within 1e-5."""
    import idp_gb300 as idp

    X0, F, pr, v = two_spheres()
    ctx = shell_ctx(idp, X0, F, pr, mode, v=v, newton_tol=1e-5, max_newton=500)
    rc, res = ctx.advance(check=False)
    assert rc in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP), res
    Xg, _, _ = ctx.state(0)
    assert len(ctx.intersections(0)) == 0
    pb = shell_oracle(oracle, X0, F, pr, v, tol=1e-5)
    pb.max_iters = 500
    its = oracle.advance_one_step(pb)
    rel = abs(res[0]["energy"] - pb.last_energy) / abs(pb.last_energy)
    print(f"two spheres: GPU {res[0]['newton_iters']} iterations E {res[0]['energy']:.12e} C "
          f"{res[0]['num_constraints']}; oracle {its} iterations E {pb.last_energy:.12e} C {pb.log[-1]['ncons']}; "
          f"rel {rel:.2e}; max |dX| {np.abs(Xg - pb.X).max():.2e}")
    assert res[0]["num_constraints"] > 0
    assert len(oracle.edge_tri_intersections(Xg, pb.surf)) == 0
    assert rel <= 1e-6
    assert np.abs(Xg - pb.X).max() <= 1e-5
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_pressed_sphere_is_a_converged_oracle_solution(oracle, gpu_lib, mode):
    """A sphere whose predictor flattens it through itself buckles: the step
    has many nearby minima and which one a trajectory reaches depends on
    last-bit rounding. The GPU's result is a converged, injective solution
    with its caps in contact: the oracle's Newton loop started from it stops
    within a few iterations at its energy within 1e-6."""
    import idp_gb300 as idp

    X0, F, pr, v = pressed_sphere()
    ctx = shell_ctx(idp, X0, F, pr, mode, v=v, newton_tol=1e-5, max_newton=1000)
    rc, res = ctx.advance(check=False)
    assert rc in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP), res
    Xg, _, _ = ctx.state(0)
    assert len(ctx.intersections(0)) == 0 and res[0]["num_constraints"] > 0
    pb = shell_oracle(oracle, X0, F, pr, v, X=Xg, tol=1e-5)
    pb.max_iters = 50
    its = oracle.advance_one_step(pb, Xtilde=X0 + 0.1 * v)
    rel = abs(res[0]["energy"] - pb.last_energy) / abs(pb.last_energy)
    print(f"pressed sphere: GPU {res[0]['newton_iters']} iterations E {res[0]['energy']:.12e}; oracle from the GPU "
          f"result {its} iterations E {pb.last_energy:.12e}; rel {rel:.2e}")
    assert its <= 10 and rel <= 1e-6
    assert len(oracle.edge_tri_intersections(Xg, pb.surf)) == 0
    ctx.close()


def test_hinge_call_with_shell_elements_matches_c_abi(oracle, gpu_lib):
    """Advance_One_Step_IE_Hinge with the shell's elements, element attributes
    and hinge stencils as Initialize_Discrete_Shell prepares them."""
    import idp_gb300 as idp
    from idp_gb300.api import FEM, shell_material

    X0, F, pr, v = two_spheres()
    surf = oracle.shell_surface(X0.shape[0], F)
    hin, info = oracle.shell_hinges(X0, F, surf["edges"])
    mem = oracle.membrane_rest(X0, F, pr["thickness"], pr["E"], pr["nu"])
    k = oracle.hinge_stiffness(pr["E"], pr["nu"], pr["thickness"])
    # the reference's storages: rest first fundamental form per face (IB), its
    # P slot of face 0 holding the hinge stiffness, (F, vol, lambda, mu) per face
    IB = np.stack([np.linalg.inv(np.array([[m[0], m[1]], [m[1], m[2]]])) for m in mem])
    elemAttr = {"IB": IB, "P": np.zeros_like(IB)}
    elemAttr["P"][0, 0, 0] = k
    elasticityAttr = {"vol": mem[:, 4], "lambda": mem[:, 5], "mu": mem[:, 6]}
    nodeAttr = {"x0": X0.copy(), "v": v.copy(), "g": np.zeros_like(X0), "m": pr["mass"].copy()}
    kappaVec = [pr["kappa"], pr["kappa_max"], 0.0]
    X = X0.copy()
    args = [F, [], [], {}, hin, info, 0.0, 1.0, [], [], [1.0, 0.0], [1.0, 1.0], [0.0, 0.0], None, 0.1, 1e-3,
            True, pr["dHat2"], kappaVec, 0.0, 1e-10, 0, [], [], False, X, nodeAttr, None, elemAttr, elasticityAttr,
            np.zeros((0, 4), np.int32), None, None, [], [], [], [], [], [], 0.0, [], ""]
    its = FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*args)
    mat = shell_material(F, nodeAttr, elemAttr, elasticityAttr, 1.0)
    ctx = idp.Context(h=0.1, mode=idp.MODE_MIXED, newton_tol=1e-3)
    ctx.add_elastic_shell_instance(X0, F, mat["density"], mat["E"], mat["nu"], mat["thickness"], pr["dHat2"],
                                   pr["kappa"], pr["kappa_max"], bending_mult=mat["bending_mult"], mass=mat["mass"])
    ctx.set_velocity(0, v)
    ctx.commit()
    _, r = ctx.advance(check=False)
    Xd, vd, kd = ctx.state(0)
    assert its == r[0]["newton_iters"]
    assert np.array_equal(X, Xd) and np.array_equal(nodeAttr["v"], vd) and kappaVec[0] == kd[0]
    assert r[0]["num_constraints"] > 0
    ctx.close()


@pytest.mark.parametrize("mode,tol", [(0, 1e-5), (1, 2e-4)], ids=["fp64", "mixed"])
def test_character_sequence_matches_oracle(oracle, gpu_lib, tmp_path, mode, tol):
    """The shell driver over a three-frame sequence (lv_fn / seqDBCPath, as
    the mannequin script drives it): each step takes frame k as the rest
    shape, points the velocity at it and moves the top cap's DBC rows onto
    it, under gravity; the oracle is fed the same rest shape, velocity,
    kappa, body force and targets, step by step."""
    from idp_gb300 import meshio
    from idp_gb300.api import ShellFlowSim, initialize_oipc
    from test_api_shell import rotated_frames

    X, F = cases.sphere_shell(2)
    meshio.write_tri_obj(tmp_path / "rest.obj", X, F)
    sim = ShellFlowSim("double", 3, mode=mode)
    sim.add_shell_with_scale_3D(str(tmp_path / "rest.obj"), (0, 0.75, 0), (0.5, 0.5, 0.5), (0, 0, 0), (1, 0, 0), -90)
    sim.set_DBC((-0.1, 0.8, -0.1), (1.1, 1.1, 1.1), (0, 0, 0), (0, 0, 0), (1, 0, 0), 0)
    h, g = 0.1, np.array([0.0, -1.0, 0.0])
    sim.dt = sim.frame_dt = h
    sim.gravity = tuple(g)
    sim.PNTol = 1e-5
    sim.initialize(1000, 1e4, 0.4, 0.01, 0)
    sim.initialize_OIPC(1e-3, 0)
    (tmp_path / "seq").mkdir()
    for k, Y in enumerate(rotated_frames(sim.X, 3), 1):
        meshio.write_tri_obj(tmp_path / "seq" / f"{k}.obj", Y, F)
    sim.lv_fn, sim.seqDBCPath, sim.output_folder = 1, str(tmp_path / "seq"), str(tmp_path / "out")
    rows = sim.DBC.indices.copy()
    assert rows.size > 4
    for f in range(1, 4):
        Y, _, _ = meshio.read_tri_obj(tmp_path / "seq" / f"{f}.obj")
        pr = cases.shell_problem(Y, F, density=1000.0, E=1e4, nu=0.4, thickness=0.01, dHat=1e-3)
        k, km = initialize_oipc(float(pr["mass"].mean()), 1e-6, 1.0)
        pr["kappa"], pr["kappa_max"] = k, km
        pb = shell_oracle(oracle, Y, F, pr, (Y - sim.X) / h, X=sim.X, dbc=rows, tol=1e-5)
        pb.h, pb.b = h, pr["mass"][:, None] * g[None, :]
        pb.dbc_rows, pb.dbc_target = rows, Y[rows]
        sim.advance_one_frame(f)
        sim.write(f)
        oracle.advance_one_step(pb)
        assert sim.lv_fn == f + 1
        assert np.array_equal(sim.X[rows], Y[rows])  # nothing in the way: the rows reach their targets
        assert np.max(np.abs(sim.X - pb.X)) <= tol
        Xw, Fw, _ = meshio.read_tri_obj(tmp_path / "out" / f"shell{f}.obj")
        assert np.array_equal(Fw, F) and np.allclose(Xw, sim.X, rtol=1e-5, atol=1e-6)
    assert np.max(np.linalg.norm(sim.X - Y, axis=1)) > 1e-3  # gravity pulled the free part off the frame
