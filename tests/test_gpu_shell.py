"""Triangle shells in flow mode (idp_add_shell_instance; Advance_One_Step_IE_Flow,
FEM/Shell/DISCRETE_SHELL.h:1113) on the GB300 against the oracle: surface
primitives and constraint sets bit-exact (index work), flow energy and
gradient within 1e-9 relative (FP64, different summation order and the
edge form of the energy), Hessian products within 1e-9 (FP64 mode), and
whole flow steps: one Newton step without contacts, contact-resolving steps
with the energy within 1e-5 relative of the oracle's direct solve (both stop
at the same Newton tolerance, not at the same iterate)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 0.5  # the normal-flow scripts' dt with smoothIntensity 0.5


def shell(n=12, seed=1, shift=(0.0, 0.0, 0.0), scale=1.0):
    from idp_gb300 import meshgen

    X, T, _ = meshgen.blob(n=n, lmax=4, seed=seed)
    Xs, F = meshgen.shell_from_tets(X, T)
    return Xs * scale + np.asarray(shift), F


def setup(oracle, parts, thickness=0.01, density=1000.0):
    """One shell made of the given (X, F) parts (disjoint components)."""
    Xs, Fs, off = [], [], 0
    for X, F in parts:
        Xs.append(X)
        Fs.append(F + off)
        off += X.shape[0]
    X, F = np.vstack(Xs), np.vstack(Fs).astype(np.int32)
    keep, mass, vol = oracle.shell_init(X, F, density, thickness)
    assert keep.all()
    diag = float(np.linalg.norm(X.max(0) - X.min(0)))
    dHat2 = (1e-3 * diag) ** 2
    k, km = oracle.kappa_init(float(mass.mean()), dHat2)
    return dict(X=X, F=F, mass=mass, vol=vol, dHat2=dHat2, kappa=k, kappa_max=km, thickness=thickness,
                density=density)


def gpu_ctx(idp, s, mode, **kw):
    ctx = idp.Context(h=H, mode=mode, **kw)
    ctx.add_shell_instance(s["X"], s["F"], s["density"], s["thickness"], s["dHat2"], s["kappa"], s["kappa_max"])
    ctx.commit()
    return ctx


def oracle_pb(oracle, s, X=None):
    X0 = s["X"]
    return oracle.Problem(X=(X0 if X is None else X).copy(), X0=X0.copy(), tets=None, mass=s["mass"], lam=None,
                          mu=None, h=H, dHat2=s["dHat2"], kappa=[s["kappa"], s["kappa_max"], 0.0],
                          v=np.zeros_like(X0), faces=s["F"], fvol=s["vol"])


def test_shell_surface_matches_oracle(oracle, gpu_lib):
    import idp_gb300 as idp

    s = setup(oracle, [shell()])
    ctx = gpu_ctx(idp, s, idp.MODE_MIXED)
    g = ctx.surface(0)
    o = oracle.shell_surface(s["X"].shape[0], s["F"])
    for k in ("tris", "edges", "nodes"):
        assert np.array_equal(g[k], o[k]), k
    ctx.close()


def test_flow_energy_gradient_hessian(oracle, gpu_lib):
    import idp_gb300 as idp

    s = setup(oracle, [shell()])
    rng = np.random.default_rng(0)
    X = s["X"] + 0.002 * rng.normal(size=s["X"].shape)
    ctx = gpu_ctx(idp, s, idp.MODE_FP64)
    Ee, Ei, Eb = ctx.energy(0, X)
    # x_tilde = x^n (zero velocity): inertia measured from the current state
    Eo = oracle.flow_energy(X, s["F"], s["vol"], H)
    assert Ee == pytest.approx(Eo, rel=1e-9)
    g = ctx.gradient(0, X)
    go = oracle.flow_gradient(X, s["F"], s["vol"], H) + (s["mass"][:, None] * (X - s["X"])).reshape(-1)
    assert np.linalg.norm(g - go) <= 1e-9 * np.linalg.norm(go)
    x = rng.normal(size=X.size)
    y = ctx.hessian_apply(0, X, x)
    Ho = oracle.flow_hessian(X.size, s["F"], s["vol"], H)
    yo = Ho @ x + np.repeat(s["mass"], 3) * x
    assert np.linalg.norm(y - yo) <= 1e-9 * np.linalg.norm(yo)
    ctx.close()


def test_two_shells_constraint_set_bitexact(oracle, gpu_lib):
    import idp_gb300 as idp

    a = shell(seed=1)
    b = shell(seed=2, shift=(0.0, 0.0, 0.0))
    # place the second shell just beyond the first along x
    b = (b[0] + np.array([a[0][:, 0].max() - b[0][:, 0].min() + 2e-3, 0.0, 0.0]), b[1])
    s = setup(oracle, [a, b])
    s["dHat2"] = (5e-3) ** 2
    ctx = gpu_ctx(idp, s, idp.MODE_MIXED)
    g = ctx.constraint_set(0, s["X"])
    surf = oracle.shell_surface(s["X"].shape[0], s["F"])
    o, _ = oracle.constraint_set(s["X"], s["X"], surf, np.zeros(s["X"].shape[0], np.uint8), s["dHat2"])
    assert len(o) > 0
    assert sorted(map(tuple, g.tolist())) == sorted(map(tuple, o.tolist()))
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_flow_step_contact_free(oracle, gpu_lib, mode):
    import idp_gb300 as idp

    s = setup(oracle, [shell()])
    ctx = gpu_ctx(idp, s, mode, pcg_rel_tol=1e-10)
    ctx.set_normal_flow(0, 0.005)
    rc, res = ctx.advance(check=False)
    assert res[0]["status"] == idp.IDP_OK
    assert res[0]["newton_iters"] == 1  # quadratic, no contacts: one step
    Xg, vg, _ = ctx.state(0)
    pb = oracle_pb(oracle, s)
    Xt = s["X"] + oracle.normal_flow_velocity(s["X"], s["F"], 0.005, H) * H
    assert oracle.advance_one_step(pb, Xtilde=Xt) == 1
    assert res[0]["energy"] == pytest.approx(pb.last_energy, rel=1e-6)
    assert np.abs(Xg - pb.X).max() <= 1e-6 * np.abs(pb.X).max()
    # next step without a predictor: the velocity is zeroed (x_tilde = x) and
    # only the Laplacian smoothing moves the shell, as in the oracle
    rc, res = ctx.advance(check=False)
    X2, _, _ = ctx.state(0)
    assert oracle.advance_one_step(pb, Xtilde=pb.X.copy()) == 1
    assert res[0]["energy"] == pytest.approx(pb.last_energy, rel=1e-6)
    assert np.abs(X2 - pb.X).max() <= 1e-3 * np.abs(X2 - Xg).max()
    ctx.close()


def test_flow_steps_with_contact(oracle, gpu_lib):
    """Two shells flowing outward into each other: the barrier activates, the
    result stays intersection-free and its energy matches the oracle's."""
    import idp_gb300 as idp

    a = shell(seed=1)
    b = shell(seed=2)
    b = (b[0] + np.array([a[0][:, 0].max() - b[0][:, 0].min() + 4e-3, 0.0, 0.0]), b[1])
    s = setup(oracle, [a, b])
    ctx = gpu_ctx(idp, s, idp.MODE_FP64, max_newton=200, verify_iterates=1, pcg_rel_tol=1e-10)
    pb = oracle_pb(oracle, s)
    pb.max_iters = 200
    for step in range(3):
        ctx.set_normal_flow(0, 0.004)
        rc, res = ctx.advance(check=False)
        assert res[0]["status"] in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP), res
        Xt = pb.X + oracle.normal_flow_velocity(pb.X, s["F"], 0.004, H) * H
        oracle.advance_one_step(pb, Xtilde=Xt)
        assert res[0]["energy"] == pytest.approx(pb.last_energy, rel=1e-5), step
    assert res[0]["num_constraints"] > 0
    assert ctx.stats()["verify_failures"] == 0
    Xg, _, _ = ctx.state(0)
    assert len(oracle.edge_tri_intersections(Xg, oracle.shell_surface(Xg.shape[0], s["F"]))) == 0
    ctx.close()


def test_reference_shaped_flow_call(oracle, gpu_lib):
    """FEM.DiscreteShell.Advance_One_Step_IE_Flow with the reference's
    positional arguments (body force b = magnitude * M_ii * n from
    Update_Normal_Flow_Neumann) gives the same step as the C-ABI calls."""
    import idp_gb300 as idp
    from idp_gb300.api import FEM

    s = setup(oracle, [shell()])
    X = s["X"].copy()
    mag = 0.02
    n = oracle.normal_flow_velocity(X, s["F"], 1.0, 1.0)  # unit normals
    b = (mag * s["mass"][:, None] * n).reshape(-1)
    nodeAttr = {"x0": s["X"].copy(), "v": np.zeros_like(X), "m": s["mass"].copy()}
    elasticityAttr = {"vol": s["vol"].copy()}
    kappaVec = [s["kappa"], s["kappa_max"], 0.0]
    it = FEM.DiscreteShell.Advance_One_Step_IE_Flow(
        s["F"], [], [], None, None, None, 0.0, 0.0, None, None, None, None, None, b, H, 1e-3, True, s["dHat2"],
        kappaVec, 0.0, 0.0, 0, None, None, False, X, nodeAttr, None, None, elasticityAttr, [], None, None, [], None,
        [], None, [], None, 0.0, [], "")
    assert it == 1
    ctx = gpu_ctx(idp, s, idp.MODE_MIXED)
    ctx.set_normal_flow(0, H * H * mag)
    ctx.advance(check=False)
    Xg, _, _ = ctx.state(0)
    assert np.allclose(X, Xg, rtol=0, atol=1e-12 * np.abs(Xg).max())
    ctx.close()


def test_normal_flow_script_driver(oracle, gpu_lib, tmp_path):
    """The normal-flow script's calls (12-14_normal_flow.py) through
    ShellFlowSim, on a shell read from an OBJ file, give the same states as
    the C-ABI calls they stand for."""
    import idp_gb300 as idp
    from idp_gb300 import meshio
    from idp_gb300.api import ShellFlowSim

    X, F = shell()
    p = tmp_path / "blob.obj"
    meshio.write_tri_obj(p, X, F)
    sim = ShellFlowSim("double", 3)
    smooth = 0.5
    sim.normalFlowMag = 0.005
    sim.frame_num = 2
    sim.add_shell_3D(str(p), (0, 0, 0), (0, 0, 0), (0, 0, 0), 0)
    sim.dt = 1.0 * smooth
    sim.frame_dt = 1.0 * smooth
    sim.flow = True
    sim.normalFlowMag /= smooth * smooth
    sim.initialize(1, 0, 0, 1, 0)
    sim.initialize_OIPC(1e-3, 0)
    X0 = sim.X.copy()
    sim.run()
    assert len(sim.DBC) == 0  # closed surface: nothing fixed
    ctx = idp.Context(h=0.5, mode=idp.MODE_MIXED)
    k0, km0 = idp.api.initialize_oipc(float(sim._mass().mean()), 1e-6)
    ctx.add_shell_instance(X0, F, 1.0, 1.0, 1e-6, k0, km0)
    ctx.commit()
    for _ in range(2):
        ctx.set_normal_flow(0, 0.25 * 0.005 / 0.25)
        ctx.advance(check=False)
    Xg, _, _ = ctx.state(0)
    assert np.array_equal(sim.X, Xg)
    assert not np.array_equal(Xg, X0)
    ctx.close()
