"""CPU checks of the oracle: analytic known answers, finite differences of
every derivative, and structural properties of its constraint set and CCD.

The reference ships no tests or golden vectors for this path (its Tests/
directory is absent), so these analytic cases and the disabled finite-
difference routines' method (forward differences, relative error; e.g.
Physics/NEOHOOKEAN.h:357-401) are what pins the oracle.
"""
import math

import numpy as np
import pytest


def fd_grad(f, x, eps=1e-7):
    g = np.zeros_like(x)
    for i in range(x.size):
        xp, xm = x.copy(), x.copy()
        xp.flat[i] += eps
        xm.flat[i] -= eps
        g.flat[i] = (f(xp) - f(xm)) / (2 * eps)
    return g


# ---------------------------------------------------------------- distances
def test_point_triangle_types_known_answers(oracle):
    t0, t1, t2 = np.array([0.0, 0, 0]), np.array([1.0, 0, 0]), np.array([0.0, 1, 0])
    cases = {  # point -> (type, squared distance)
        (0.2, 0.2, 0.5): (6, 0.25),
        (-1.0, -1.0, 0.0): (0, 2.0),
        (2.0, -0.5, 0.0): (1, 1.25),
        (-0.5, 2.0, 1.0): (2, 2.25),
        (0.5, -1.0, 0.0): (3, 1.0),
        (1.0, 1.0, 0.0): (4, 0.5),
        (-1.0, 0.5, 0.0): (5, 1.0),
    }
    for p, (ty, d2) in cases.items():
        p = np.array(p)
        assert oracle.lib().ora_type_pt(*[oracle._d(oracle.f64(a)) for a in (p, t0, t1, t2)]) == ty, p
        d = oracle.lib().ora_dist_pt_unclassified(*[oracle._d(oracle.f64(a)) for a in (p, t0, t1, t2)])
        assert d == pytest.approx(d2, rel=1e-14), p


def test_edge_edge_types_known_answers(oracle):
    a0, a1 = np.array([0.0, 0, 0]), np.array([1.0, 0, 0])
    cases = {  # (b0, b1) -> (type, squared distance)
        ((0.5, -1, 1), (0.5, 1, 1)): (8, 1.0),   # skew edges crossing in projection
        ((-1, -1, 1), (-1, 1, 1)): (2, 2.0),     # ea0 closest to the interior of eb
        ((2, -1, 1), (2, 1, 1)): (5, 2.0),       # ea1 closest to the interior of eb
        ((-1, 0, 1), (-2, 0, 2)): (0, 2.0),      # ea0 - eb0
        ((2, 0, 1), (3, 0, 1)): (3, 2.0),        # ea1 - eb0
        ((-2, 0, 1), (-1, 0, 1)): (1, 2.0),      # ea0 - eb1
        ((3, 0, 1), (2, 0, 1)): (4, 2.0),        # ea1 - eb1
        ((0.5, 0, 1), (0.5, 0, 3)): (6, 1.0),    # eb0 closest to the interior of ea
        ((0.5, 0, 3), (0.5, 0, 1)): (7, 1.0),    # eb1 closest to the interior of ea
    }
    for (b0, b1), (ty, d2) in cases.items():
        b0, b1 = np.array(b0, float), np.array(b1, float)
        d = oracle.lib().ora_dist_ee_unclassified(*[oracle._d(oracle.f64(a)) for a in (a0, a1, b0, b1)])
        assert d == pytest.approx(d2, rel=1e-14), (b0, b1)
        assert oracle.lib().ora_type_ee(*[oracle._d(oracle.f64(a)) for a in (a0, a1, b0, b1)]) == ty, (b0, b1)
    # parallel edges are never classified as the degenerate line-line case
    b0, b1 = np.array([0.2, 0.0, 1.0]), np.array([0.8, 0.0, 1.0])
    ty = oracle.lib().ora_type_ee(*[oracle._d(oracle.f64(a)) for a in (a0, a1, b0, b1)])
    assert ty != 8
    d = oracle.lib().ora_dist_ee_unclassified(*[oracle._d(oracle.f64(a)) for a in (a0, a1, b0, b1)])
    assert d == pytest.approx(1.0, rel=1e-14)


@pytest.mark.parametrize("kind,n", [(0, 2), (1, 3), (2, 4), (3, 4), (4, 4)])
def test_distance_derivatives_fd(oracle, kind, n):
    rng = np.random.default_rng(kind + 11)
    for _ in range(5):
        x = rng.normal(size=3 * n)
        d, g, H = oracle.dist_derivs(kind, x)
        f = lambda y: oracle.dist_derivs(kind, y)[0]  # noqa: E731
        gf = fd_grad(f, x)
        assert np.allclose(g, gf, rtol=1e-6, atol=1e-7 * max(1.0, np.abs(g).max()))
        Hf = np.stack([fd_grad(lambda y: oracle.dist_derivs(kind, y)[1][j], x) for j in range(3 * n)])
        assert np.allclose(H, Hf, rtol=1e-5, atol=1e-6 * max(1.0, np.abs(H).max()))
        assert np.allclose(H, H.T, atol=1e-12 * max(1.0, np.abs(H).max()))


def test_make_pd(oracle):
    rng = np.random.default_rng(3)
    A = rng.normal(size=(12, 12))
    A = A + A.T
    P = oracle.make_pd(A)
    w = np.linalg.eigvalsh(P)
    assert w.min() > -1e-10 * np.abs(w).max()
    wa, Va = np.linalg.eigh(A)
    ref = (Va * np.maximum(wa, 0)) @ Va.T
    assert np.allclose(P, ref, atol=1e-10 * np.abs(A).max())
    B = A @ A.T + np.eye(12)  # already positive definite: returned unchanged
    assert np.array_equal(oracle.make_pd(B), B)


def test_barrier_known_answers(oracle):
    k, km = oracle.kappa_init(2.0, 1e-4)
    # b''(1e-16) with kappa=1 and dHat2=1e-4
    d, dh = 1e-16, 1e-4
    Hb = (math.log(d / dh) * -2.0 - (d - dh) * 4.0 / d) + 1.0 / (d * d) * (d - dh) ** 2
    assert k == pytest.approx(1e11 * 2.0 * 3 / (4e-16 * Hb), rel=1e-14)
    assert km == pytest.approx(100 * k, rel=1e-15)


# ---------------------------------------------------------------- elasticity
def _tiny_mesh():
    import idp_gb300.meshgen as mg
    X, tets = mg.bar(2, 2, 3, size=(1.0, 1.0, 1.5), jitter=0.05, seed=1)
    return X, tets


def test_tet_energy_gradient_hessian_fd(oracle):
    X, tets = _tiny_mesh()
    IB, vol = oracle.tet_rest(X, tets)
    T = tets.shape[0]
    lam, mu = np.full(T, 5.0), np.full(T, 2.0)
    rng = np.random.default_rng(0)
    Y = X + 0.05 * rng.normal(size=X.shape)
    f = lambda y: oracle.tet_energy(y.reshape(-1, 3), tets, IB, vol, lam, mu, 0.3)  # noqa: E731
    g = oracle.tet_gradient(Y, tets, IB, vol, lam, mu, 0.3)
    assert np.allclose(g, fd_grad(f, Y.reshape(-1)), rtol=1e-6, atol=1e-8)
    # unprojected element Hessians match finite differences of the gradient
    He = oracle.tet_hessian(Y, tets, IB, vol, lam, mu, 0.3, project=False)
    n = Y.size
    H = np.zeros((n, n))
    for t in range(T):
        dof = (3 * tets[t][:, None] + np.arange(3)).reshape(-1)
        H[np.ix_(dof, dof)] += He[t]
    Hf = np.stack([fd_grad(lambda y: oracle.tet_gradient(y.reshape(-1, 3), tets, IB, vol, lam, mu, 0.3)[j],
                           Y.reshape(-1)) for j in range(n)])
    assert np.allclose(H, Hf, rtol=1e-5, atol=1e-7 * np.abs(H).max())
    # projected element Hessians are PSD
    Hp = oracle.tet_hessian(Y, tets, IB, vol, lam, mu, 0.3, project=True)
    for t in range(T):
        assert np.linalg.eigvalsh(Hp[t]).min() > -1e-9 * np.abs(Hp[t]).max()
    # inversion is rejected (INC_POTENTIAL.h:98-108)
    Z = X.copy()
    Z[tets[0][0]] = X[tets[0][1:]].mean(0) * 2 - X[tets[0][0]]
    assert oracle.tet_energy(Z, tets, IB, vol, lam, mu, 0.3) is None


# ---------------------------------------------------------------- surface
def test_surface_of_bar(oracle):
    import idp_gb300.meshgen as mg
    X, tets = mg.bar(3, 2, 4, seed=0)
    s = oracle.surface(X, tets)
    nN, nE, nT = len(s["nodes"]), len(s["edges"]), len(s["tris"])
    assert nN - nE + nT == 2          # closed genus-0 surface
    assert 2 * nE == 3 * nT           # closed manifold
    # reference ordering: triangles lexicographic, edges lexicographic
    t = [tuple(x) for x in s["tris"]]
    e = [tuple(x) for x in s["edges"]]
    assert t == sorted(t) and e == sorted(e)
    assert np.all(np.diff(s["nodes"]) > 0)
    # outward orientation: signed volume of the surface is positive
    P = X[s["tris"]]
    vol = np.einsum("ti,ti->t", P[:, 0], np.cross(P[:, 1], P[:, 2])).sum() / 6
    assert vol > 0


# ---------------------------------------------------------------- contact
def _two_bars(gap, seed=0, n=(2, 2, 4)):
    """Two jittered bars side by side with a small gap in x."""
    import idp_gb300.meshgen as mg
    X, tets = mg.bar(*n, size=(1.0, 1.0, 2.0), jitter=0.05, seed=seed)
    Y = X.copy()
    Y[:, 0] += 1.0 + gap
    rng = np.random.default_rng(seed + 100)
    Y[:, 1] += rng.uniform(-0.3, 0.3)
    Y[:, 2] += rng.uniform(-0.3, 0.3)
    return np.concatenate([X, Y]), np.concatenate([tets, tets + X.shape[0]]).astype(np.int32)


def test_constraint_set_properties(oracle):
    X, tets = _two_bars(gap=2e-3)
    s = oracle.surface(X, tets)
    dbc = np.zeros(X.shape[0], np.uint8)
    dHat2 = (5e-3) ** 2
    cons, info = oracle.constraint_set(X, X, s, dbc, dHat2)
    assert cons.shape[0] > 0
    # every constraint is closer than dHat and positive
    md, d2 = oracle.min_dist2(cons, X)
    assert md > 0 and np.all(d2 < dHat2)
    # no duplicates; multiplicity only on regular PP/PE records
    assert len({tuple(c) for c in cons}) == cons.shape[0]
    mult = cons[:, 3] < -1
    assert np.all(cons[mult, 0] < 0)
    assert np.all(info[:, 0] == 1.0)
    # far apart: empty set
    X2, tets2 = _two_bars(gap=0.5)
    s2 = oracle.surface(X2, tets2)
    c2, _ = oracle.constraint_set(X2, X2, s2, np.zeros(X2.shape[0], np.uint8), dHat2)
    assert c2.shape[0] == 0


def test_barrier_gradient_fd(oracle):
    X, tets = _two_bars(gap=2e-3, seed=4)
    s = oracle.surface(X, tets)
    dbc = np.zeros(X.shape[0], np.uint8)
    dHat2 = (5e-3) ** 2
    cons, info = oracle.constraint_set(X, X, s, dbc, dHat2)
    assert cons.shape[0] > 0
    kappa = 10.0
    g = oracle.barrier_gradient(cons, info, X, X, dHat2, kappa)
    idx = np.unique(np.abs(np.where(np.abs(g) > 0)[0]))[:30]
    x = X.reshape(-1).copy()
    for i in idx:
        h = 1e-9
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fp = oracle.barrier_energy(cons, info, xp.reshape(-1, 3), X, dHat2, kappa)
        fm = oracle.barrier_energy(cons, info, xm.reshape(-1, 3), X, dHat2, kappa)
        assert (fp - fm) / (2 * h) == pytest.approx(g[i], rel=2e-4, abs=1e-6 * np.abs(g).max())


def test_ccd_step_is_conservative(oracle):
    X, tets = _two_bars(gap=0.05, seed=2)
    s = oracle.surface(X, tets)
    dbc = np.zeros(X.shape[0], np.uint8)
    V = X.shape[0]
    d = np.zeros((V, 3))
    d[V // 2:, 0] = -0.2   # second bar moves into the first
    a, rc = oracle.ccd_stepsize(X, d.reshape(-1), s, dbc, 1.0)
    assert rc == 0
    assert 0 < a < 0.25 / 0.9 + 1e-12
    # at alpha the bars are still separated
    Xa = X + a * d
    cons, _ = oracle.constraint_set(Xa, X, s, dbc, 1e-2)
    md, _ = oracle.min_dist2(cons, Xa)
    assert md > 0
    # no motion toward each other: full step
    d2 = np.zeros((V, 3))
    d2[V // 2:, 0] = 0.2
    a2, _ = oracle.ccd_stepsize(X, d2.reshape(-1), s, dbc, 1.0)
    assert a2 == pytest.approx(1.0) or a2 > 0.5


def test_normal_flow_outward_unit(oracle):
    """Oracle normal-flow shift has length |step| on surface vertices, points
    out of a star-shaped blob, and is zero inside."""
    from idp_gb300 import meshgen

    X, tets, _ = meshgen.blob(n=10, lmax=6, seed=2)
    surf = oracle.surface(X, tets)
    h = 0.1
    v = oracle.normal_flow_velocity(X, surf["tris"], 0.05, h)
    on = np.zeros(X.shape[0], bool)
    on[surf["nodes"]] = True
    assert np.allclose(np.linalg.norm(v[on], axis=1) * h, 0.05)
    assert np.all(v[~on] == 0)
    assert np.all(np.einsum("ij,ij->i", v[on], X[on] - X.mean(0)) > 0)


# ---------------------------------------------------------------- shells, flow mode
def _shell(n=12, seed=1):
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from idp_gb300 import meshgen

    X, T, _ = meshgen.blob(n=n, lmax=4, seed=seed)
    return meshgen.shell_from_tets(X, T)


def test_flow_energy_forms_agree(oracle):
    """-h/2 x^T L x (INC_POTENTIAL.h:53-73) equals the edge form
    h/12 sum vol (|x0-x1|^2 + |x1-x2|^2 + |x2-x0|^2); its gradient is -h L x."""
    X, F = _shell()
    keep, mass, vol = oracle.shell_init(X, F, 1000.0, 0.01)
    assert keep.all()
    rng = np.random.default_rng(0)
    Y = X + 0.01 * rng.normal(size=X.shape)
    h = 0.5
    e_ref = oracle.flow_energy(Y, F, vol, h)
    d = lambda a, b: ((Y[F[:, a]] - Y[F[:, b]]) ** 2).sum(1)
    e_edge = float((h / 12 * vol * (d(0, 1) + d(1, 2) + d(2, 0))).sum())
    assert e_ref == pytest.approx(e_edge, rel=1e-12)
    g = oracle.flow_gradient(Y, F, vol, h)
    f = lambda z: oracle.flow_energy(z.reshape(-1, 3), F, vol, h)
    idx = rng.choice(Y.size, 12, replace=False)
    gfd = np.array([(f(Y.reshape(-1) + 1e-6 * np.eye(Y.size)[i]) - f(Y.reshape(-1) - 1e-6 * np.eye(Y.size)[i])) / 2e-6
                    for i in idx])
    assert np.allclose(gfd, g[idx], rtol=1e-5, atol=1e-10)


def test_shell_surface_and_mass(oracle):
    X, F = _shell()
    s = oracle.shell_surface(X.shape[0], F)
    assert X.shape[0] - len(s["edges"]) + F.shape[0] == 2  # closed genus-0 surface
    assert np.array_equal(s["tris"], F)
    assert np.array_equal(s["nodes"], np.arange(X.shape[0]))
    assert sorted(map(tuple, s["edges"].tolist())) == list(map(tuple, s["edges"].tolist()))
    keep, mass, vol = oracle.shell_init(X, F, 1000.0, 0.01)
    assert mass.sum() == pytest.approx(1000.0 * vol.sum(), rel=1e-12)


def test_flow_step_contact_free_is_one_newton_step(oracle):
    """Flow mode without contacts: one Newton step solves the quadratic
    exactly (IMPLICIT_EULER.h:850-854)."""
    X, F = _shell()
    keep, mass, vol = oracle.shell_init(X, F, 1000.0, 0.01)
    h = 0.5
    diag = float(np.linalg.norm(X.max(0) - X.min(0)))
    dHat2 = (1e-3 * diag) ** 2
    k, km = oracle.kappa_init(float(mass.mean()), dHat2)
    pb = oracle.Problem(X=X.copy(), X0=X.copy(), tets=None, mass=mass, lam=None, mu=None, h=h, dHat2=dHat2,
                        kappa=[k, km, 0.0], v=np.zeros_like(X), faces=F, fvol=vol)
    Xt = X + oracle.normal_flow_velocity(X, F, 0.005, h) * h
    it = oracle.advance_one_step(pb, Xtilde=Xt)
    assert it == 1
    # the result minimises E: gradient vanishes
    g = oracle.flow_gradient(pb.X, F, vol, h) + (mass[:, None] * (pb.X - Xt)).reshape(-1)
    assert np.linalg.norm(g) < 1e-8 * np.linalg.norm((mass[:, None] * (X - Xt)).reshape(-1))
