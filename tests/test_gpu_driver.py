"""The reference-shaped driver call and the inputs around the Newton loop on
the GB300: FEM.DiscreteShell.Advance_One_Step_IE_Hinge with the reference's
positional arguments gives the direct C-ABI calls' results bit for bit
(positions, velocity, kappa; fixed DBC and a body force included, and a
kappa the driver resets between calls is read again); the body-force
predictor, the adaptive kappa and DBC-projected Newton directions match the
oracle."""
import math

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def bar_case(seed=0, ang=1.2):
    from idp_gb300 import meshgen

    X, tets = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 2.6), seed=seed)
    tgt = meshgen.bend_target(X, angle=ang * math.pi, radius=0.45, size=(1.0, 1.0, 2.6))
    return X, tets, tgt, cases.problem(X, tets)


def reference_args(X, tets, pr, v, kappaVec, DBC, b, h=0.1, tol=1e-3):
    """The positional argument list of Advance_One_Step_IE_Hinge
    (FEM/Shell/DISCRETE_SHELL.h:1110) for a tet mesh with offset IPC."""
    T = tets.shape[0]
    nodeAttr = {"x0": X.copy(), "v": v.copy(), "g": np.zeros_like(X), "m": pr["mass"].copy()}
    tetEl = {"lambda": np.full(T, pr["lam"]), "mu": np.full(T, pr["mu"])}
    return dict(Elem=[], segs=[], DBC=DBC, edge2tri={}, edgeStencil=[], edgeInfo=[], thickness=0.0,
                bendingStiffMult=1.0, fiberStiffMult=[], fiberLimit=[], s=[1.0, 0.0], sHat=[1.0, 1.0],
                kappa_s=[0.0, 0.0], b=b, h=h, NewtonTol=tol, withCollision=True, dHat2=pr["dHat2"],
                kappaVec=kappaVec, mu=0.0, epsv2=1e-10, fricIterAmt=0, compNodeRange=[], muComp=[],
                staticSolve=False, X=X.copy(), nodeAttr=nodeAttr, M=None, elemAttr=None, elasticityAttr=None,
                tet=tets, tetAttr=None, tetElasticityAttr=tetEl, rod=[], rodInfo=[], rodHinge=[], rodHingeInfo=[],
                stitchInfo=[], stitchRatio=[], k_stitch=0.0, particle=[], outputFolder="")


def test_hinge_call_matches_the_c_abi(gpu_lib):
    import idp_gb300 as idp
    from idp_gb300 import api
    from idp_gb300.api import FEM

    # a cantilever: the base fixed, the bar swung sideways and pulled down
    # by gravity (no self-contact, a few Newton iterations per step)
    X, tets, tgt, pr = bar_case(ang=0.3)
    V = X.shape[0]
    h = 0.1
    v = np.zeros_like(X)
    v[:, 0] = 0.5 * X[:, 2]
    fixed = np.nonzero(X[:, 2] < 1e-12)[0].astype(np.int32)
    DBC = np.concatenate([fixed[:, None].astype(np.float64), X[fixed]], axis=1)  # (index, target)
    b = np.zeros_like(X)
    b[:, 1] = -9.8 * pr["mass"]  # gravity
    kappaVec = [pr["kappa"], pr["kappa_max"], 0.0]
    a = reference_args(X, tets, pr, v, kappaVec, DBC, b)
    order = list(a)
    its = [FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*[a[k] for k in order]) for _ in range(2)]
    # the same two steps through the C ABI directly
    ctx = idp.Context(h=h, mode=idp.MODE_MIXED, newton_tol=1e-3)
    ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"],
                     dbc_idx=fixed)
    ctx.set_velocity(0, v)
    ctx.set_body_force(0, b)
    ctx.commit()
    r1 = ctx.advance(check=False)[1][0]
    r2 = ctx.advance(check=False)[1][0]
    Xd, vd, kd = ctx.state(0)
    assert its == [r1["newton_iters"], r2["newton_iters"]]
    assert np.array_equal(a["X"], Xd) and np.array_equal(a["nodeAttr"]["v"], vd)
    assert kappaVec[0] == kd[0]
    assert np.array_equal(a["X"][fixed], X[fixed])  # fixed DBC vertices stay
    # a driver that resets kappa (initialize_OIPC) between calls
    kappaVec[0] = pr["kappa"]
    FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*[a[k] for k in order])
    ctx.set_kappa(0, [pr["kappa"], pr["kappa_max"], 0.0])
    ctx.advance(check=False)
    Xd, vd, kd = ctx.state(0)
    assert np.array_equal(a["X"], Xd) and kappaVec[0] == kd[0]
    # a new tet array with the same content reuses the context; different
    # content (a moved rest shape) builds a new one
    key, c0 = api._Cache.key, api._Cache.ctx
    a2 = dict(a, tet=tets.copy())
    assert api._context_for(np.asarray(a2["tet"]), a2["X"], a2["nodeAttr"], a2["tetElasticityAttr"], a2["dHat2"],
                            kappaVec, DBC, h, 1e-3, 0.0, api.DiscreteShell.mode) is c0
    a3 = dict(a, nodeAttr=dict(a["nodeAttr"], x0=X * 1.01))
    api._context_for(np.asarray(a3["tet"]), a3["X"], a3["nodeAttr"], a3["tetElasticityAttr"], a3["dHat2"], kappaVec,
                     DBC, h, 1e-3, 0.0, api.DiscreteShell.mode)
    assert api._Cache.key != key
    ctx.close()


def test_body_force_step_matches_oracle(oracle, gpu_lib):
    import idp_gb300 as idp

    X, tets, tgt, pr = bar_case(ang=0.6)
    h = 0.1
    v = (tgt - X) / h
    b = np.zeros_like(X)
    b[:, 2] = -30.0 * pr["mass"]
    ctx = idp.Context(h=h, mode=idp.MODE_FP64, newton_tol=1e-5)
    ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    ctx.set_velocity(0, v)
    ctx.set_body_force(0, b)
    ctx.commit()
    # the predictor enters the inertia energy: check it at a test configuration
    Xt = X + 0.01 * np.sin(X)
    Ee, Ei, Eb = ctx.energy(0, Xt)
    xt = X + (h * v + (h * h) * (b / pr["mass"][:, None]))
    assert Ei == pytest.approx(0.5 * float(np.sum(pr["mass"][:, None] * (Xt - xt) ** 2)), rel=1e-12)
    rc, res = ctx.advance(check=False)
    assert rc == idp.IDP_OK, res
    T = tets.shape[0]
    po = oracle.Problem(X=X.copy(), X0=X, tets=tets, mass=pr["mass"], lam=np.full(T, pr["lam"]),
                        mu=np.full(T, pr["mu"]), h=h, dHat2=pr["dHat2"], kappa=[pr["kappa"], pr["kappa_max"], 0.0],
                        v=v.copy(), b=b, tol=1e-5, max_iters=300)
    oracle.advance_one_step(po)
    assert abs(res[0]["energy"] - po.last_energy) <= 1e-6 * abs(po.last_energy)
    Xg, vg, _ = ctx.state(0)
    assert np.max(np.abs(Xg - po.X)) <= 1e-4 * np.max(np.abs(po.X))
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_kappa_adapts_like_the_oracle(oracle, gpu_lib, mode):
    """Two bars pressed together with a barrier a millionth of its usual
    stiffness: the bars close below 1e-9 and kappa doubles
    (IMPLICIT_EULER.h:566-595) on the GPU as in the oracle. How often it
    doubles depends on which iterate first brings a pair below 1e-18, a
    last-bit matter along the trajectory, so the counts agree within a few
    doublings; the GPU's result is a converged solution of the step at the
    GPU's kappa: the oracle, started from it with that kappa, stops within a
    few iterations at the GPU's energy within 1e-5 (the barrier this soft
    leaves the energy flat near the solution)."""
    import idp_gb300 as idp

    X, tets = cases.two_bars(gap=2e-3, seed=0)
    pr = cases.problem(X, tets, dHat=5e-3)
    V, T = X.shape[0], tets.shape[0]
    v = np.zeros_like(X)
    v[V // 2:, 0] = -0.02 / 0.1
    k0 = pr["kappa"] * 1e-6
    ctx = idp.Context(h=0.1, mode=mode, newton_tol=1e-5, max_newton=500)
    ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], k0, pr["kappa_max"])
    ctx.set_velocity(0, v)
    ctx.commit()
    rc, res = ctx.advance(check=False)
    assert rc == idp.IDP_OK, res
    Xg, _, kap = ctx.state(0)

    def problem(X1, kappa):
        return oracle.Problem(X=X1.copy(), X0=X, tets=tets, mass=pr["mass"], lam=np.full(T, pr["lam"]),
                              mu=np.full(T, pr["mu"]), h=0.1, dHat2=pr["dHat2"], kappa=kappa, v=v.copy(), tol=1e-5,
                              max_iters=500)

    po = problem(X, [k0, pr["kappa_max"], 0.0])
    oracle.advance_one_step(po)
    dg, do = math.log2(res[0]["kappa"] / k0), math.log2(po.kappa[0] / k0)
    # from the GPU's result, kappa held at the GPU's value
    pw = problem(Xg, [kap[0], kap[0], 0.0])
    its = oracle.advance_one_step(pw, Xtilde=X + 0.1 * v)
    rel = abs(res[0]["energy"] - pw.last_energy) / abs(pw.last_energy)
    print(f"kappa doublings: GPU {dg:.0f}, oracle {do:.0f}; iterations GPU {res[0]['newton_iters']}, oracle "
          f"{len(po.log)}; oracle from the GPU result {its} iterations, rel energy {rel:.2e}")
    assert dg >= 6 and do >= 6 and abs(dg - do) <= 4
    assert its <= 10 and rel <= 1e-5
    ctx.close()


@pytest.mark.parametrize("mode,tol", [(0, 1e-6), (1, 2e-3)], ids=["fp64", "mixed"])
def test_dbc_projected_newton_direction(oracle, gpu_lib, mode, tol):
    """Newton direction with fixed DBC vertices (rows and columns projected to
    the identity, Math/CSR_MATRIX.h:130-141; gradient rows zeroed,
    IMPLICIT_EULER.h:476-480) against the oracle's direct solve, at a contact
    configuration."""
    import scipy.sparse.linalg as spla

    import idp_gb300 as idp

    X0, tets, Xd = cases.folded_bar(seed=1, n=(2, 2, 8), frac=0.97, radius=1.0)
    pr = cases.problem(X0, tets, dHat=0.05)
    V = X0.shape[0]
    fixed = np.arange(0, V, 5, dtype=np.int32)
    rng = np.random.default_rng(2)
    v = rng.normal(size=X0.shape)
    ctx = idp.Context(h=0.1, mode=mode, pcg_rel_tol=1e-8)
    ctx.add_instance(X0, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"],
                     dbc_idx=fixed)
    ctx.set_velocity(0, v)
    ctx.commit()
    p, its, rel = ctx.newton_direction(0, Xd)
    T = tets.shape[0]
    dbc = np.zeros(V, np.uint8)
    dbc[fixed] = 1
    pb = oracle.Problem(X=Xd.copy(), X0=X0, tets=tets, mass=pr["mass"], lam=np.full(T, pr["lam"]),
                        mu=np.full(T, pr["mu"]), h=0.1, dHat2=pr["dHat2"], kappa=[pr["kappa"], pr["kappa_max"], 0.0],
                        v=np.zeros_like(X0), dbc=dbc)
    cons, info = oracle.constraint_set(Xd, X0, oracle.surface(X0, tets), dbc, pr["dHat2"])
    assert len(cons) > 0
    H = oracle._hessian(pb, Xd, cons, info)
    g = oracle._gradient(pb, Xd, X0 + 0.1 * v, cons, info)
    g.reshape(-1, 3)[fixed] = 0
    po = spla.spsolve(H.tocsc(), -g)
    assert np.all(p.reshape(-1, 3)[fixed] == 0) and np.all(po.reshape(-1, 3)[fixed] == 0)
    assert np.linalg.norm(p - po) <= tol * np.linalg.norm(po)
    ctx.close()
