"""GB300 parity of every sub-step against the CPU oracle, through the C ABI.

Bars: constraint sets and surface primitives bit-exact (index work); CCD
step bit-exact (same FP64 operations, same voxel grid, fixed-order means);
energy and gradient within 1e-9 relative (FP64, different summation order);
assembled Hessian times a vector within 1e-9 (FP64 mode) / 2e-4 (mixed mode,
FP32 element Hessians) relative to |H x|.
"""
import math

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def ctx_for(idp, X, tets, pr, mode, h=0.1, X0=None, v=None, dbc=None, **kw):
    ctx = idp.Context(h=h, mode=mode, **kw)
    ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"],
                     X0=X0, dbc_idx=dbc)
    if v is not None:
        ctx.set_velocity(0, v)
    ctx.commit()
    return ctx


def oracle_problem(O, X, tets, pr, h=0.1, X0=None):
    T = tets.shape[0]
    return O.Problem(X=X.copy(), X0=X if X0 is None else X0, tets=tets, mass=pr["mass"], lam=np.full(T, pr["lam"]),
                     mu=np.full(T, pr["mu"]), h=h, dHat2=pr["dHat2"], kappa=[pr["kappa"], pr["kappa_max"], 0.0],
                     v=np.zeros_like(X))


def contact_configs():
    out = []
    for seed in range(3):
        X, tets = cases.two_bars(gap=2e-3, seed=seed)
        out.append((f"two_bars_{seed}", X, tets, X, 5e-3))
    X0, tets, Xd = cases.folded_bar(seed=0, frac=1.0)
    out.append(("folded_overlap_far", X0, tets, Xd, 0.08))
    X0, tets, Xd = cases.folded_bar(seed=1, n=(2, 2, 8), frac=0.97, radius=1.0)
    out.append(("folded_near", X0, tets, Xd, 0.05))
    return out


def sort_rows(a):
    return sorted(map(tuple, np.asarray(a).tolist()))


def test_surface_matches_oracle(oracle, gpu_lib):
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    for X, tets in [meshgen.bar(3, 2, 5, seed=0)[:2], meshgen.blob(n=12, lmax=4, seed=1)[:2]]:
        pr = cases.problem(X, tets)
        ctx = ctx_for(idp, X, tets, pr, idp.MODE_MIXED)
        g = ctx.surface(0)
        o = oracle.surface(X, tets)
        assert np.array_equal(g["tris"], o["tris"])
        assert np.array_equal(g["edges"], o["edges"])
        assert np.array_equal(g["nodes"], o["nodes"])
        ctx.close()


@pytest.mark.parametrize("name,X0,tets,X,dhat", contact_configs(), ids=lambda v: v if isinstance(v, str) else "")
def test_constraint_set_bitexact(oracle, gpu_lib, name, X0, tets, X, dhat):
    import idp_gb300 as idp

    pr = cases.problem(X0, tets, dHat=dhat)
    ctx = ctx_for(idp, X0, tets, pr, idp.MODE_MIXED)
    g = ctx.constraint_set(0, X)
    surf = oracle.surface(X0, tets)
    o, _ = oracle.constraint_set(X, X0, surf, np.zeros(X0.shape[0], np.uint8), pr["dHat2"])
    assert len(o) > 0, name
    assert sort_rows(g) == sort_rows(o), name
    ctx.close()


def test_constraint_set_empty_and_dbc(oracle, gpu_lib):
    import idp_gb300 as idp

    X, tets = cases.two_bars(gap=0.5)
    pr = cases.problem(X, tets, dHat=5e-3)
    ctx = ctx_for(idp, X, tets, pr, idp.MODE_MIXED)
    assert len(ctx.constraint_set(0, X)) == 0
    ctx.close()
    # all-DBC stencils are excluded (IPC.h:171-172, 384-385)
    X, tets = cases.two_bars(gap=2e-3, seed=1)
    dbc = np.arange(X.shape[0] // 2, X.shape[0], dtype=np.int32)
    pr = cases.problem(X, tets, dHat=5e-3)
    ctx = ctx_for(idp, X, tets, pr, idp.MODE_MIXED, dbc=dbc)
    mask = np.zeros(X.shape[0], np.uint8)
    mask[dbc] = 1
    o, _ = oracle.constraint_set(X, X, oracle.surface(X, tets), mask, pr["dHat2"])
    assert sort_rows(ctx.constraint_set(0, X)) == sort_rows(o)
    ctx.close()


def test_repeated_builds_match_oracle(oracle, gpu_lib):
    """Later constraint-set and CCD builds of a context reuse the table
    capacities of the first one without a host round trip; they must give the
    same results as a fresh build."""
    import idp_gb300 as idp

    X0, tets, Xd = cases.folded_bar(seed=1, n=(2, 2, 8), frac=0.97, radius=1.0)
    pr = cases.problem(X0, tets, dHat=0.05)
    ctx = ctx_for(idp, X0, tets, pr, idp.MODE_MIXED)
    surf = oracle.surface(X0, tets)
    z = np.zeros(X0.shape[0], np.uint8)
    rng = np.random.default_rng(9)
    for k, frac in enumerate((0.0, 0.5, 1.0, 0.8, 1.0)):
        X = X0 + frac * (Xd - X0)
        g = ctx.constraint_set(0, X)
        o, _ = oracle.constraint_set(X, X0, surf, z, pr["dHat2"])
        assert sort_rows(g) == sort_rows(o), k
        d = 0.05 * rng.normal(size=X.shape)
        ag, _ = ctx.ccd_stepsize(0, X, d.reshape(-1), 1.0)
        ao, rc = oracle.ccd_stepsize(X, d.reshape(-1), surf, z, 1.0)
        assert ag == ao, (k, ag, ao)
    ctx.close()


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_ccd_stepsize_bitexact(oracle, gpu_lib, seed):
    import idp_gb300 as idp

    X, tets = cases.two_bars(gap=0.02, seed=seed)
    pr = cases.problem(X, tets, dHat=5e-3)
    rng = np.random.default_rng(seed)
    V = X.shape[0]
    d = 0.05 * rng.normal(size=(V, 3))
    d[V // 2:, 0] -= 0.15
    ctx = ctx_for(idp, X, tets, pr, idp.MODE_MIXED)
    for a0 in (1.0, 0.37):
        ag, _ = ctx.ccd_stepsize(0, X, d.reshape(-1), a0)
        ao, rc = oracle.ccd_stepsize(X, d.reshape(-1), oracle.surface(X, tets), np.zeros(V, np.uint8), a0)
        assert rc == 0
        assert ag == ao, (a0, ag, ao)
        assert 0 < ag <= a0
    ctx.close()


@pytest.mark.parametrize("name,X0,tets,X,dhat", [contact_configs()[k] for k in (0, 1, 2, 4)], ids=lambda v: v if isinstance(v, str) else "")
def test_energy_gradient_parity(oracle, gpu_lib, name, X0, tets, X, dhat):
    import idp_gb300 as idp

    h = 0.1
    pr = cases.problem(X0, tets, dHat=dhat)
    rng = np.random.default_rng(5)
    v = rng.normal(size=X.shape)
    # x_tilde = x + h v is formed from the context's current positions (X0)
    ctx = ctx_for(idp, X0, tets, pr, idp.MODE_FP64, h=h, v=v)
    Ee, Ei, Eb = ctx.energy(0, X)
    g = ctx.gradient(0, X)
    pb = oracle_problem(oracle, X, tets, pr, h=h, X0=X0)
    xt = X0 + h * v
    cons, info = oracle.constraint_set(X, X0, oracle.surface(X0, tets), np.zeros(X0.shape[0], np.uint8), pr["dHat2"])
    E_el = oracle.tet_energy(X, tets, pb.IB, pb.vol, pb.lam, pb.mu, h * h)
    E_in = 0.5 * float(np.sum(pr["mass"][:, None] * (X - xt) ** 2))
    E_b = oracle.barrier_energy(cons, info, X, X0, pr["dHat2"], pr["kappa"])
    assert Ee == pytest.approx(E_el, rel=1e-9)
    assert Ei == pytest.approx(E_in, rel=1e-9)
    assert Eb == pytest.approx(E_b, rel=1e-9, abs=1e-12)
    go = oracle._gradient(pb, X, xt, cons, info)
    assert np.linalg.norm(g - go) <= 1e-9 * np.linalg.norm(go)
    ctx.close()


@pytest.mark.parametrize("mode,tol", [(0, 1e-9), (1, 2e-4)])
def test_hessian_apply_parity(oracle, gpu_lib, mode, tol):
    name, X0, tets, X, dhat = contact_configs()[0]
    import idp_gb300 as idp

    pr = cases.problem(X0, tets, dHat=dhat)
    ctx = ctx_for(idp, X0, tets, pr, mode)
    pb = oracle_problem(oracle, X, tets, pr, X0=X0)
    cons, info = oracle.constraint_set(X, X0, oracle.surface(X0, tets), np.zeros(X0.shape[0], np.uint8), pr["dHat2"])
    assert len(cons) > 0
    H = oracle._hessian(pb, X, cons, info)
    rng = np.random.default_rng(0)
    for _ in range(3):
        x = rng.normal(size=X.size)
        y = ctx.hessian_apply(0, X, x)
        yo = H @ x
        assert np.linalg.norm(y - yo) <= tol * np.linalg.norm(yo)
    ctx.close()


# PCG paths: one thread-block cluster per instance (default at these sizes),
# or the grid-wide cooperative PCG forced down to small instances
PCG_PATHS = {"cluster": {}, "grid": {"pcg_grid_min_vertices": 1, "pcg_grid_cta_vertices": 16}}


@pytest.mark.parametrize("path", sorted(PCG_PATHS))
@pytest.mark.parametrize("mode", [0, 1])
def test_newton_direction_solves_system(oracle, gpu_lib, mode, path):
    import idp_gb300 as idp
    import scipy.sparse.linalg as spla

    name, X0, tets, X, dhat = contact_configs()[1]
    pr = cases.problem(X0, tets, dHat=dhat)
    rng = np.random.default_rng(1)
    v = rng.normal(size=X.shape)
    ctx = ctx_for(idp, X0, tets, pr, mode, v=v, pcg_rel_tol=1e-8, **PCG_PATHS[path])
    p, its, rel = ctx.newton_direction(0, X)
    assert rel <= 1e-7 and its > 0
    pb = oracle_problem(oracle, X, tets, pr, X0=X0)
    cons, info = oracle.constraint_set(X, X0, oracle.surface(X0, tets), np.zeros(X0.shape[0], np.uint8), pr["dHat2"])
    H = oracle._hessian(pb, X, cons, info)
    g = oracle._gradient(pb, X, X0 + 0.1 * v, cons, info)
    po = spla.spsolve(H.tocsc(), -g)
    tol = 1e-6 if mode == 0 else 2e-3  # mixed: FP32 element Hessians
    assert np.linalg.norm(p - po) <= tol * np.linalg.norm(po)
    ctx.close()


@pytest.mark.parametrize("path", sorted(PCG_PATHS))
@pytest.mark.parametrize("mode", [0, 1])
def test_newton_direction_contact_free(oracle, gpu_lib, mode, path):
    """A direction without contact constraints (the grid PCG takes its
    pipelined branch there) against a direct solve."""
    import idp_gb300 as idp
    import scipy.sparse.linalg as spla
    from idp_gb300 import meshgen

    X0, tets, _ = meshgen.blob(n=12, lmax=6, seed=4)
    pr = cases.problem(X0, tets)
    rng = np.random.default_rng(5)
    X = X0 + rng.uniform(-0.01, 0.01, X0.shape)
    v = rng.normal(size=X0.shape)
    ctx = ctx_for(idp, X0, tets, pr, mode, v=v, pcg_rel_tol=1e-8, **PCG_PATHS[path])
    p, its, rel = ctx.newton_direction(0, X)
    assert rel <= 1e-7 and its > 0
    pb = oracle_problem(oracle, X, tets, pr, X0=X0)
    cons, info = oracle.constraint_set(X, X0, oracle.surface(X0, tets), np.zeros(X0.shape[0], np.uint8), pr["dHat2"])
    assert len(cons) == 0
    H = oracle._hessian(pb, X, cons, info)
    g = oracle._gradient(pb, X, X0 + 0.1 * v, cons, info)
    po = spla.spsolve(H.tocsc(), -g)
    tol = 1e-6 if mode == 0 else 2e-3
    assert np.linalg.norm(p - po) <= tol * np.linalg.norm(po)
    ctx.close()


def small_bar_problem():
    from idp_gb300 import meshgen

    X, tets = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 2.6), seed=0)
    target = meshgen.bend_target(X, angle=2.2 * math.pi, radius=0.45, size=(1.0, 1.0, 2.6))
    pr = cases.problem(X, tets)
    return X, tets, target, pr


@pytest.mark.parametrize("path", sorted(PCG_PATHS))
@pytest.mark.parametrize("mode", [0, 1])
def test_full_step_injective_and_close_to_oracle(oracle, gpu_lib, mode, path):
    import idp_gb300 as idp

    X, tets, target, pr = small_bar_problem()
    h = 0.1
    v = (target - X) / h
    ctx = ctx_for(idp, X, tets, pr, mode, h=h, v=v, newton_tol=1e-3, max_newton=600, **PCG_PATHS[path])
    rc, res = ctx.advance(check=False)
    assert rc in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP), res
    Xg, vg, kap = ctx.state(0)
    # injective: positive volumes and positive distances at the result
    pb = oracle_problem(oracle, X, tets, pr)
    surf = oracle.surface(X, tets)
    assert oracle.tet_energy(Xg, tets, pb.IB, pb.vol, pb.lam, pb.mu, 1.0) is not None
    cons, info = oracle.constraint_set(Xg, X, surf, np.zeros(X.shape[0], np.uint8), pr["dHat2"])
    if len(cons):
        assert oracle.min_dist2(cons, Xg)[0] > 0
    # the same step on the oracle (direct solve)
    po = oracle_problem(oracle, X, tets, pr)
    po.v = v.copy()
    po.max_iters = 600
    oracle.advance_one_step(po)
    rel = abs(res[0]["energy"] - po.last_energy) / abs(po.last_energy)
    assert rel <= 1e-3, (res[0]["energy"], po.last_energy)
    assert np.allclose(vg, (Xg - X) / h)
    ctx.close()


@pytest.mark.parametrize("path", sorted(PCG_PATHS))
def test_batch_is_bitwise_identical_to_alone(oracle, gpu_lib, path):
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    h = 0.1
    probs = []
    for seed, (nx, nz, ang) in enumerate([(2, 6, 2.1 * math.pi), (3, 7, 2.2 * math.pi), (2, 5, 1.9 * math.pi)]):
        X, tets = meshgen.bar(nx, nx, nz, size=(1.0, 1.0, 2.0), seed=seed)
        tgt = meshgen.bend_target(X, angle=ang, radius=0.4, size=(1.0, 1.0, 2.0))
        probs.append((X, tets, tgt, cases.problem(X, tets)))
    batch = idp.Context(h=h, mode=idp.MODE_MIXED, max_newton=40, **PCG_PATHS[path])
    for i, (X, tets, tgt, pr) in enumerate(probs):
        batch.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
        batch.set_velocity(i, (tgt - X) / h)
    batch.commit()
    _, rb = batch.advance(check=False)
    for i, (X, tets, tgt, pr) in enumerate(probs):
        alone = ctx_for(idp, X, tets, pr, idp.MODE_MIXED, h=h, v=(tgt - X) / h, max_newton=40, **PCG_PATHS[path])
        _, ra = alone.advance(check=False)
        Xa, _, _ = alone.state(0)
        Xb, _, _ = batch.state(i)
        assert np.array_equal(Xa, Xb), i
        assert ra[0]["newton_iters"] == rb[i]["newton_iters"]
        assert ra[0]["energy"] == rb[i]["energy"]
        alone.close()
    batch.close()


def test_inverted_input_is_rejected(gpu_lib):
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    X, tets = meshgen.bar(2, 2, 2, seed=0)
    bad = tets.copy()
    bad[0, [1, 2]] = bad[0, [2, 1]]
    pr = cases.problem(X, tets)
    ctx = idp.Context()
    ctx.add_instance(X, bad, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    with pytest.raises(idp.IDPError) as e:
        ctx.commit()
    assert e.value.code == idp.IDP_ERR_INVERTED
    ctx.close()


def test_normal_flow_velocity_bitexact(oracle, gpu_lib):
    """Device normal-flow predictor equals the oracle's bit for bit, per
    instance and for all instances at once."""
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    h = 0.1
    meshes = [meshgen.bar(3, 2, 5, seed=0)[:2], meshgen.blob(n=12, lmax=4, seed=1)[:2]]
    ctx = idp.Context(h=h, mode=idp.MODE_MIXED)
    rng = np.random.default_rng(3)
    moved = []
    for X, tets in meshes:
        pr = cases.problem(X, tets)
        ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    ctx.commit()
    for i, (X, tets) in enumerate(meshes):
        Xm = X + rng.uniform(-0.01, 0.01, X.shape)
        ctx.set_positions(i, Xm)
        moved.append(Xm)
    ctx.set_normal_flow(-1, 0.05)
    for i, (X, tets) in enumerate(meshes):
        _, v, _ = ctx.state(i)
        o = oracle.normal_flow_velocity(moved[i], oracle.surface(X, tets)["tris"], 0.05, h)
        assert np.array_equal(v, o), i
    ctx.set_normal_flow(1, -0.02)
    _, v0, _ = ctx.state(0)
    _, v1, _ = ctx.state(1)
    assert np.array_equal(v0, oracle.normal_flow_velocity(moved[0], oracle.surface(*meshes[0])["tris"], 0.05, h))
    assert np.array_equal(v1, oracle.normal_flow_velocity(moved[1], oracle.surface(*meshes[1])["tris"], -0.02, h))
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_normal_flow_step_close_to_oracle(oracle, gpu_lib, mode):
    """One normal-flow solve on a small blob: injective, and the final
    incremental potential within 1e-3 relative of the oracle's direct-solve
    Newton step on the same predictor."""
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    X, tets, _ = meshgen.blob(n=10, lmax=6, seed=2)
    pr = cases.problem(X, tets)
    h = 0.1
    ctx = ctx_for(idp, X, tets, pr, mode, h=h, newton_tol=1e-3, max_newton=200)
    ctx.set_normal_flow(0, 0.05)
    _, v0, _ = ctx.state(0)
    rc, res = ctx.advance(check=False)
    assert rc == idp.IDP_OK, res
    Xg, _, _ = ctx.state(0)
    pb = oracle_problem(oracle, X, tets, pr)
    assert oracle.tet_energy(Xg, tets, pb.IB, pb.vol, pb.lam, pb.mu, 1.0) is not None
    po = oracle_problem(oracle, X, tets, pr)
    po.v = oracle.normal_flow_velocity(X, oracle.surface(X, tets)["tris"], 0.05, h)
    assert np.array_equal(po.v, v0)
    po.max_iters = 200
    oracle.advance_one_step(po)
    rel = abs(res[0]["energy"] - po.last_energy) / abs(po.last_energy)
    assert rel <= 1e-3, (res[0]["energy"], po.last_energy)
    ctx.close()
