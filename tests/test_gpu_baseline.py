"""The GPU path against the oracle on two benchmark configurations, at full
size, through the C ABI.

* bar: 6x6x24 cubes x 5 tets (4,320 tets) bent onto a self-intersecting
  2.2 pi circle. At three contact-heavy iterates of the oracle's own Newton
  trajectory (committed in tests/golden/baseline_configs.npz): constraint
  set as a set (bit-exact), CCD step along the oracle's Newton direction
  (bit-exact), energy and gradient (1e-9 relative), Hessian times a vector
  (1e-9 FP64 / 2e-4 mixed, FP32 element Hessians). The whole solve to
  PNTol 1e-5: a converged solution for the oracle too (its Newton loop
  started from the GPU's result stops at once, within 1e-6 relative).
* blob: the 220,515-tet spherical-harmonic blob. Energy and gradient at a
  perturbed flow iterate (1e-9 relative), and the first normal-flow step
  solved to PNTol 1e-5: final energy within 1e-6 relative of the oracle's.

Every accepted result is also checked injective: positive tet volumes and
no edge-triangle intersection (exact predicates, on the device and in the
oracle).
"""
import math
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = np.load(os.path.join(HERE, "golden", "baseline_configs.npz"))
PNTOL = float(FIX["pntol"][0])


def sort_rows(a):
    return sorted(map(tuple, np.asarray(a).tolist()))


def bar_problem(O):
    pb = O.make_bar_problem(6, 6, 24, angle=2.2 * math.pi, seed=0, tol=PNTOL)
    T = pb.tets.shape[0]
    pr = dict(mass=pb.mass, lam=float(pb.lam[0]), mu=float(pb.mu[0]), dHat2=pb.dHat2, kappa=pb.kappa[0],
              kappa_max=pb.kappa[1])
    assert T == 4320 and pb.X.shape[0] == 1225
    return pb, pr


def bar_ctx(idp, pb, pr, mode, **kw):
    ctx = idp.Context(h=pb.h, mode=mode, **kw)
    ctx.add_instance(pb.X0, pb.tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    ctx.set_velocity(0, pb.v)
    ctx.commit()
    return ctx


def injective(O, ctx, X, X0, tets, IB, vol, lam, mu, surf):
    assert O.tet_energy(X, tets, IB, vol, lam, mu, 1.0) is not None
    assert len(ctx.intersections(0)) == 0
    assert len(O.edge_tri_intersections(X, surf)) == 0


@pytest.mark.parametrize("k", [0, 1, 2])
def test_bar_iterate_constraint_set_and_ccd_bitexact(oracle, gpu_lib, k):
    import idp_gb300 as idp

    pb, pr = bar_problem(oracle)
    X = FIX["bar_X"][k]
    d = FIX["bar_dir"][k]
    ctx = bar_ctx(idp, pb, pr, idp.MODE_FP64)
    surf = oracle.surface(pb.X0, pb.tets)
    z = np.zeros(X.shape[0], np.uint8)
    g = ctx.constraint_set(0, X)
    o, _ = oracle.constraint_set(X, pb.X0, surf, z, pr["dHat2"])
    assert len(o) == int(FIX["bar_ncons"][k]) and len(o) > 500
    assert sort_rows(g) == sort_rows(o)
    for a0 in (1.0, 0.5, 0.0625):
        ag, _ = ctx.ccd_stepsize(0, X, d, a0)
        ao, rc = oracle.ccd_stepsize(X, d, surf, z, a0)
        assert rc == 0 and 0 < ag <= a0
        assert ag == ao, (k, a0, ag, ao)
    ctx.close()


@pytest.mark.parametrize("k", [0, 1, 2])
@pytest.mark.parametrize("mode,tol", [(0, 1e-9), (1, 2e-4)], ids=["fp64", "mixed"])
def test_bar_iterate_energy_gradient_hessian(oracle, gpu_lib, k, mode, tol):
    import idp_gb300 as idp

    pb, pr = bar_problem(oracle)
    X = FIX["bar_X"][k]
    ctx = bar_ctx(idp, pb, pr, mode)
    xt = pb.X0 + pb.h * pb.v
    surf = oracle.surface(pb.X0, pb.tets)
    cons, info = oracle.constraint_set(X, pb.X0, surf, np.zeros(X.shape[0], np.uint8), pr["dHat2"])
    Ee, Ei, Eb = ctx.energy(0, X)
    h2 = pb.h * pb.h
    E_el = oracle.tet_energy(X, pb.tets, pb.IB, pb.vol, pb.lam, pb.mu, h2)
    E_in = 0.5 * float(np.sum(pr["mass"][:, None] * (X - xt) ** 2))
    E_b = oracle.barrier_energy(cons, info, X, pb.X0, pr["dHat2"], pr["kappa"])
    assert Ee == pytest.approx(E_el, rel=1e-9)
    assert Ei == pytest.approx(E_in, rel=1e-9)
    assert Eb == pytest.approx(E_b, rel=1e-9) and E_b > 0
    g = ctx.gradient(0, X)
    go = oracle._gradient(pb, X, xt, cons, info)
    assert np.linalg.norm(g - go) <= 1e-9 * np.linalg.norm(go)
    H = oracle._hessian(pb, X, cons, info)
    rng = np.random.default_rng(k)
    for _ in range(2):
        x = rng.normal(size=X.size)
        y, yo = ctx.hessian_apply(0, X, x), H @ x
        assert np.linalg.norm(y - yo) <= tol * np.linalg.norm(yo)
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_bar_solve_is_a_converged_oracle_solution(oracle, gpu_lib, mode):
    """The self-intersecting bar solved to PNTol 1e-5 on the GPU. Its final
    configuration is a converged solution of the same step for the oracle:
    the oracle's Newton loop, started from it (same predictor and kappa),
    stops within a few iterations and ends within 1e-6 relative of the GPU's
    incremental potential; the result is injective.

    The step has several nearby local minima (the target folds the bar
    through itself), and which one a trajectory reaches depends on last-bit
    rounding along ~900 contact-heavy iterations: from the rest state the
    oracle stops at the energy recorded in the fixture, reported here, not
    asserted."""
    import idp_gb300 as idp

    pb, pr = bar_problem(oracle)
    ctx = bar_ctx(idp, pb, pr, mode, newton_tol=PNTOL, max_newton=6000)
    rc, res = ctx.advance(check=False)
    assert rc in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP), res
    Xg, _, kap = ctx.state(0)
    injective(oracle, ctx, Xg, pb.X0, pb.tets, pb.IB, pb.vol, pb.lam, pb.mu, oracle.surface(pb.X0, pb.tets))
    # the oracle's Newton loop from the GPU's result
    po, _ = bar_problem(oracle)
    xt = po.X0 + po.h * po.v
    po.X = Xg.copy()
    po.kappa = [kap[0], kap[1], 0.0]
    po.max_iters = 50
    its = oracle.advance_one_step(po, Xtilde=xt)
    rel = abs(res[0]["energy"] - po.last_energy) / abs(po.last_energy)
    E_rest = float(FIX["bar_energy"][0])
    print(f"bar: GPU {res[0]['newton_iters']} iterations E {res[0]['energy']:.12e}; oracle from the GPU result "
          f"{its} iterations E {po.last_energy:.12e} (rel {rel:.2e}); oracle from rest "
          f"{int(FIX['bar_newton_iters'][0])} iterations E {E_rest:.12e}")
    assert its <= 10, its
    assert rel <= 1e-6, (res[0]["energy"], po.last_energy)
    ctx.close()


@pytest.fixture(scope="module")
def blob():
    sys.path.insert(0, os.path.dirname(HERE))
    import bench

    p = bench.blob_problem(64)
    assert p["tets"].shape[0] == int(FIX["blob_tets"][0])
    return p


def blob_ctx(idp, p, mode, **kw):
    ctx = idp.Context(h=0.1, mode=mode, **kw)
    ctx.add_instance(p["X"], p["tets"], p["mass"], p["lam"], p["mu"], p["dHat2"], p["kappa"], p["kappa_max"])
    ctx.commit()
    ctx.set_normal_flow(0, 0.05)
    return ctx


def blob_oracle(O, p, v):
    T = p["tets"].shape[0]
    return O.Problem(X=p["X"].copy(), X0=p["X"], tets=p["tets"], mass=p["mass"], lam=np.full(T, p["lam"]),
                     mu=np.full(T, p["mu"]), h=0.1, dHat2=p["dHat2"], kappa=[p["kappa"], p["kappa_max"], 0.0], v=v,
                     tol=PNTOL)


def test_blob_full_size_energy_gradient(oracle, gpu_lib, blob):
    import idp_gb300 as idp

    p = blob
    ctx = blob_ctx(idp, p, idp.MODE_FP64)
    _, v, _ = ctx.state(0)
    surf = oracle.surface(p["X"], p["tets"])
    vo = oracle.normal_flow_velocity(p["X"], surf["tris"], 0.05, 0.1)
    assert np.array_equal(v, vo)
    rng = np.random.default_rng(7)
    X = p["X"] + 0.1 * v * 0.5 + rng.uniform(-2e-3, 2e-3, p["X"].shape)
    pb = blob_oracle(oracle, p, vo)
    xt = p["X"] + 0.1 * vo
    cons, info = oracle.constraint_set(X, p["X"], surf, np.zeros(X.shape[0], np.uint8), p["dHat2"])
    Ee, Ei, Eb = ctx.energy(0, X)
    assert Ee == pytest.approx(oracle.tet_energy(X, pb.tets, pb.IB, pb.vol, pb.lam, pb.mu, 0.01), rel=1e-9)
    assert Ei == pytest.approx(0.5 * float(np.sum(p["mass"][:, None] * (X - xt) ** 2)), rel=1e-9)
    assert Eb == pytest.approx(oracle.barrier_energy(cons, info, X, p["X"], p["dHat2"], p["kappa"]), rel=1e-9,
                               abs=1e-12)
    g = ctx.gradient(0, X)
    go = oracle._gradient(pb, X, xt, cons, info)
    assert np.linalg.norm(g - go) <= 1e-9 * np.linalg.norm(go)
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_blob_flow_step_matches_the_oracle_energy(oracle, gpu_lib, blob, mode):
    import idp_gb300 as idp

    p = blob
    ctx = blob_ctx(idp, p, mode, newton_tol=PNTOL, max_newton=500)
    rc, res = ctx.advance(check=False)
    assert rc == idp.IDP_OK, res
    E_or = float(FIX["blob_energy"][0])
    rel = abs(res[0]["energy"] - E_or) / abs(E_or)
    print(f"blob: GPU {res[0]['newton_iters']} iterations E {res[0]['energy']:.15e}; oracle "
          f"{int(FIX['blob_newton_iters'][0])} iterations E {E_or:.15e}; rel {rel:.2e}")
    assert rel <= 1e-6
    Xg, _, _ = ctx.state(0)
    pb = blob_oracle(oracle, p, np.zeros_like(p["X"]))
    assert oracle.tet_energy(Xg, pb.tets, pb.IB, pb.vol, pb.lam, pb.mu, 1.0) is not None
    assert len(ctx.intersections(0)) == 0
    ctx.close()
