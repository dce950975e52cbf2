"""GB300 exact intersection check (idp_check_intersection /
idp_check_intersection_all, restating Check_Edge_Tri_Intersect,
FEM/IPC.h:2444-2517) against the oracle: the intersecting (triangle, edge)
pairs are index work, so the lists must be identical. Also: the optional
per-iterate verification inside idp_advance runs on every accepted step and
finds nothing on a converging self-contact solve.
"""
import math

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _two_bars(offset, n=(2, 2, 4)):
    from idp_gb300 import meshgen

    X1, T1 = meshgen.bar(*n, size=(1.0, 1.0, 2.0), seed=0)
    X2, T2 = meshgen.bar(*n, size=(1.0, 1.0, 2.0), seed=1)
    return np.vstack([X1, X2 + np.asarray(offset)]), np.vstack([T1, T2 + X1.shape[0]])


def intersection_configs():
    from idp_gb300 import meshgen

    out = []
    X, tets = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 4.0), seed=0)
    out.append(("bar_rest", X, tets, X))
    out.append(("bar_bend_target", X, tets, meshgen.bend_target(X, angle=2.2 * math.pi)))
    out.append(("bar_bend_target_twist", X, tets, meshgen.bend_target(X, angle=2.4 * math.pi, twist=1.0)))
    Xb, tb = _two_bars((0.4, 0.3, 0.5))
    out.append(("two_bars_overlap", Xb, tb, Xb))
    Xc, tc = _two_bars((1.0, 0.0, 0.0))  # faces touching exactly: coplanar contact, not a crossing
    out.append(("two_bars_touching", Xc, tc, Xc))
    X0, tf, Xd = cases.folded_bar(seed=0, frac=1.0)
    out.append(("folded_overlap", X0, tf, Xd))
    Xs, ts = meshgen.blob(n=14, lmax=4, seed=2)[:2]
    out.append(("blob_rest", Xs, ts, Xs))
    return out


@pytest.mark.parametrize("name,X0,tets,X", intersection_configs(), ids=lambda v: v if isinstance(v, str) else "")
def test_intersections_match_oracle(oracle, gpu_lib, name, X0, tets, X):
    import idp_gb300 as idp

    pr = cases.problem(X0, tets)
    ctx = idp.Context(mode=idp.MODE_MIXED)
    ctx.add_instance(X0, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    ctx.commit()
    g = ctx.intersections(0, X)
    surf = oracle.surface(X0, tets)
    o = oracle.edge_tri_intersections(X, surf)
    assert np.array_equal(g, o), (name, len(g), len(o))
    if name in ("bar_bend_target", "bar_bend_target_twist", "two_bars_overlap", "folded_overlap"):
        assert len(o) > 0, name
    else:
        assert len(o) == 0, name
    # current state (the rest shape) is intersection-free when the rest shape is
    assert len(ctx.intersections(0)) == len(oracle.edge_tri_intersections(X0, surf))
    ctx.close()


def test_intersection_counts_per_instance(oracle, gpu_lib):
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    X, tets = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 4.0), seed=0)
    Xt = meshgen.bend_target(X, angle=2.2 * math.pi)
    Xb, tb = _two_bars((0.4, 0.3, 0.5))
    items = [(X, tets, X), (X, tets, Xt), (Xb, tb, Xb), (X, tets, meshgen.bend_target(X, angle=1.2 * math.pi))]
    ctx = idp.Context(mode=idp.MODE_MIXED)
    for X0, T, _ in items:
        pr = cases.problem(X0, T)
        ctx.add_instance(X0, T, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    ctx.commit()
    for i, (_, _, Xs) in enumerate(items):
        ctx.set_positions(i, Xs)
    counts = ctx.intersection_counts()
    want = [len(oracle.edge_tri_intersections(Xs, oracle.surface(X0, T))) for X0, T, Xs in items]
    assert list(counts) == want
    assert want[0] == 0 and want[1] > 0 and want[2] > 0
    ctx.close()


def test_verify_every_accepted_iterate(oracle, gpu_lib):
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    X, tets = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 2.6), seed=0)
    target = meshgen.bend_target(X, angle=2.2 * math.pi, radius=0.45, size=(1.0, 1.0, 2.6))
    pr = cases.problem(X, tets)
    h = 0.1
    ctx = idp.Context(h=h, mode=idp.MODE_MIXED, max_newton=80, verify_iterates=1)
    ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    ctx.set_velocity(0, (target - X) / h)
    ctx.commit()
    rc, res = ctx.advance(check=False)
    assert res[0]["status"] in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP, idp.IDP_ERR_NOT_CONVERGED), res
    st = ctx.stats()
    assert st["verify_checks"] == res[0]["newton_iters"] > 0
    assert st["verify_failures"] == 0
    Xg, _, _ = ctx.state(0)
    assert len(oracle.edge_tri_intersections(Xg, oracle.surface(X, tets))) == 0
    # the target itself would not pass
    assert len(oracle.edge_tri_intersections(target, oracle.surface(X, tets))) > 0
    ctx.close()
