"""Golden fixtures (tests/golden/oracle_golden.npz, made by
tests/golden/make_golden.py from the oracle on seeded inputs).

CPU: the oracle still reproduces them (integer outputs exactly, floating
point to 1e-12 relative: libm's log may differ in the last bit between
platforms). GPU: the CUDA path reproduces them through the C ABI (index sets
and CCD step sizes exactly, energies and gradients to the parity tolerance).
"""
import math
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import cases  # noqa: E402
import make_golden as mg  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "oracle_golden.npz"))


def close(a, b, rtol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.allclose(a, b, rtol=rtol, atol=rtol * max(1.0, float(np.abs(b).max(initial=0.0))))


def sort_rows(a):
    a = np.asarray(a)
    return a[np.lexsort(a.T[::-1])] if a.size else a


def test_oracle_reproduces_golden(oracle):
    for seed in range(2):
        X, tets = mg.contact_case(seed)
        surf = oracle.surface(X, tets)
        assert np.array_equal(surf["tris"], GOLD[f"contact{seed}_surf_tris"])
        assert np.array_equal(surf["edges"], GOLD[f"contact{seed}_surf_edges"])
        assert np.array_equal(surf["nodes"], GOLD[f"contact{seed}_surf_nodes"])
        dHat2 = float(GOLD[f"contact{seed}_dhat2"][0])
        kappa = float(GOLD[f"contact{seed}_kappa"][0])
        cons, info = oracle.constraint_set(X, X, surf, np.zeros(X.shape[0], np.uint8), dHat2)
        assert np.array_equal(sort_rows(cons), GOLD[f"contact{seed}_cons"])
        assert close(oracle.barrier_energy(cons, info, X, X, dHat2, kappa), GOLD[f"contact{seed}_barrier_E"][0], 1e-12)
        assert close(oracle.barrier_gradient(cons, info, X, X, dHat2, kappa), GOLD[f"contact{seed}_barrier_g"], 1e-12)
    for seed in range(2):
        X, tets, d = mg.ccd_case(seed)
        for k in range(2):
            a_exp, a0 = GOLD[f"ccd{seed}_{k}_alpha"]
            a, rc = oracle.ccd_stepsize(X, d.reshape(-1), oracle.surface(X, tets), np.zeros(X.shape[0], np.uint8), a0)
            assert rc == 0 and a == a_exp
    for seed in range(2):
        X, tets = mg.flow_case(seed)
        v = oracle.normal_flow_velocity(X, oracle.surface(X, tets)["tris"], 0.05, 0.1)
        assert np.array_equal(v, GOLD[f"flow{seed}_v"])


def test_oracle_reproduces_golden_isect_and_shells(oracle):
    for seed in range(2):
        X, tets, Xt = mg.isect_case(seed)
        pairs = oracle.edge_tri_intersections(Xt, oracle.surface(X, tets))
        assert len(pairs) > 0 and np.array_equal(pairs, GOLD[f"isect{seed}_pairs"])
    for seed in range(2):
        Xs, F, Xd = mg.shell_case(seed)
        keep, mass, vol = oracle.shell_init(Xs, F, 1000.0, 0.01)
        assert keep.all()
        assert np.array_equal(oracle.shell_surface(Xs.shape[0], F)["edges"], GOLD[f"shell{seed}_edges"])
        assert close(mass, GOLD[f"shell{seed}_mass"], 1e-12)
        assert close(oracle.flow_energy(Xd, F, vol, 0.5), GOLD[f"shell{seed}_flowE"][0], 1e-12)
        assert close(oracle.flow_gradient(Xd, F, vol, 0.5), GOLD[f"shell{seed}_flowg"], 1e-12)


def test_oracle_step_reproduces_golden(oracle):
    X, tets, target = mg.step_case()
    pr = cases.problem(X, tets)
    T = tets.shape[0]
    pb = oracle.Problem(X=X.copy(), X0=X, tets=tets, mass=pr["mass"], lam=np.full(T, pr["lam"]),
                        mu=np.full(T, pr["mu"]), h=0.1, dHat2=pr["dHat2"], kappa=[pr["kappa"], pr["kappa_max"], 0.0],
                        v=(target - X) / 0.1, tol=1e-3, max_iters=400)
    it = oracle.advance_one_step(pb)
    assert it == int(GOLD["step_newton_iters"][0])
    assert close(pb.last_energy, GOLD["step_energy"][0], 1e-9)


@pytest.mark.gpu
def test_gpu_reproduces_golden(gpu_lib):
    import idp_gb300 as idp

    for seed in range(2):
        X, tets = mg.contact_case(seed)
        pr = cases.problem(X, tets, dHat=5e-3)
        ctx = idp.Context(h=0.1, mode=idp.MODE_FP64)
        ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
        ctx.commit()
        surf = ctx.surface(0)
        assert np.array_equal(surf["tris"], GOLD[f"contact{seed}_surf_tris"])
        assert np.array_equal(surf["edges"], GOLD[f"contact{seed}_surf_edges"])
        assert np.array_equal(sort_rows(ctx.constraint_set(0, X)), GOLD[f"contact{seed}_cons"])
        ctx.close()
    for seed in range(2):
        X, tets, d = mg.ccd_case(seed)
        pr = cases.problem(X, tets, dHat=5e-3)
        ctx = idp.Context(h=0.1, mode=idp.MODE_MIXED)
        ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
        ctx.commit()
        for k in range(2):
            a_exp, a0 = GOLD[f"ccd{seed}_{k}_alpha"]
            a, _ = ctx.ccd_stepsize(0, X, d.reshape(-1), float(a0))
            assert a == a_exp
        ctx.close()
    for seed in range(2):
        X0, tets, Xd = mg.energy_case(seed)
        pr = cases.problem(X0, tets)
        ctx = idp.Context(h=0.1, mode=idp.MODE_FP64)
        ctx.add_instance(X0, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
        ctx.commit()
        Ee, _, _ = ctx.energy(0, Xd)
        assert close(Ee, GOLD[f"tet{seed}_E"][0], 1e-9)
        ctx.close()
    for seed in range(2):
        X, tets = mg.flow_case(seed)
        pr = cases.problem(X, tets)
        ctx = idp.Context(h=0.1, mode=idp.MODE_MIXED)
        ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
        ctx.commit()
        ctx.set_normal_flow(0, 0.05)
        _, v, _ = ctx.state(0)
        assert np.array_equal(v, GOLD[f"flow{seed}_v"])
        ctx.close()
    for seed in range(2):
        X, tets, Xt = mg.isect_case(seed)
        pr = cases.problem(X, tets)
        ctx = idp.Context(h=0.1, mode=idp.MODE_MIXED)
        ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
        ctx.commit()
        assert np.array_equal(ctx.intersections(0, Xt), GOLD[f"isect{seed}_pairs"])
        ctx.close()
    for seed in range(2):
        Xs, F, Xd = mg.shell_case(seed)
        ctx = idp.Context(h=0.5, mode=idp.MODE_FP64)
        ctx.add_shell_instance(Xs, F, 1000.0, 0.01, 1e-6, 1.0, 100.0)
        ctx.commit()
        assert np.array_equal(ctx.surface(0)["edges"], GOLD[f"shell{seed}_edges"])
        Ee, _, _ = ctx.energy(0, Xd)
        assert close(Ee, GOLD[f"shell{seed}_flowE"][0], 1e-9)
        ctx.close()
    X, tets, target = mg.step_case()
    pr = cases.problem(X, tets)
    for mode in (idp.MODE_FP64, idp.MODE_MIXED):
        ctx = idp.Context(h=0.1, mode=mode, newton_tol=1e-3, max_newton=400)
        ctx.add_instance(X, tets, pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
        ctx.set_velocity(0, (target - X) / 0.1)
        ctx.commit()
        rc, res = ctx.advance(check=False)
        assert rc in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP), res
        rel = abs(res[0]["energy"] - GOLD["step_energy"][0]) / abs(GOLD["step_energy"][0])
        assert rel <= 1e-3, (res[0]["energy"], GOLD["step_energy"][0])
        ctx.close()
