"""Moving Dirichlet conditions on the GB300 against the oracle
(IMPLICIT_EULER.h:305-401, 701-757; FEM/Shell/DIRICHLET.h): targets reached at
once when nothing is in the way, through the penalty (with its stiffness
doubling) when contact blocks it; the reference-shaped Hinge call with DBC
rows (index, x, y, z) gives the direct C-ABI calls' results bit for bit."""
import numpy as np
import pytest

from test_dbc_oracle import two_bar_problem

pytestmark = pytest.mark.gpu


def gpu_two_bars(idp, pb, mode, tol=1e-3):
    ctx = idp.Context(h=pb.h, mode=mode, newton_tol=tol, max_newton=pb.max_iters)
    rows = np.asarray(pb.dbc_rows, np.int32)
    ctx.add_instance(pb.X, pb.tets, pb.mass, pb.lam, pb.mu, pb.dHat2, pb.kappa[0], pb.kappa[1], X0=pb.X0,
                     dbc_idx=rows)
    ctx.set_dbc_targets(0, pb.dbc_target)
    ctx.commit()
    return ctx


def run_both(oracle, idp, pb, mode):
    ctx = gpu_two_bars(idp, pb, mode, tol=pb.tol)
    rc, res = ctx.advance(check=False)
    Xg, vg, _ = ctx.state(0)
    its = oracle.advance_one_step(pb)
    return ctx, res[0], Xg, its


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_unobstructed_targets(oracle, gpu_lib, mode):
    import idp_gb300 as idp

    pb, X, rows, tgt = two_bar_problem(oracle, +0.05)
    ctx, r, Xg, its = run_both(oracle, idp, pb, mode)
    assert r["status"] == idp.IDP_OK
    assert np.array_equal(Xg[rows], tgt)
    assert abs(r["energy"] - pb.last_energy) <= 1e-6 * abs(pb.last_energy)
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "mixed"])
def test_blocked_targets_through_the_penalty(oracle, gpu_lib, mode):
    import idp_gb300 as idp

    pb, X, rows, tgt = two_bar_problem(oracle, -0.01, tol=1e-5)
    ctx, r, Xg, its = run_both(oracle, idp, pb, mode)
    print(f"penalty step: GPU {r['newton_iters']} iterations E {r['energy']:.12e}; oracle {its} iterations "
          f"E {pb.last_energy:.12e}; progress {pb.last_stats['dbc_progress']}")
    assert r["status"] == idp.IDP_OK
    d0 = np.linalg.norm(tgt - X[rows])
    assert np.linalg.norm(tgt - Xg[rows]) <= 0.01 * d0
    assert len(ctx.intersections(0)) == 0 and r["num_constraints"] > 0
    assert abs(r["energy"] - pb.last_energy) <= 1e-6 * abs(pb.last_energy)
    assert np.max(np.abs(Xg - pb.X)) <= 1e-4
    ctx.close()


def test_penalty_stiffness_doubling_ends_at_an_oracle_solution(oracle, gpu_lib):
    """A stiff first bar fixed at its far side blocks the second bar's way:
    the penalty has to double before the DBC vertices cover 99 % of it (the
    oracle doubles it twice). Where the penalty lets go (between 99 % and
    100 % of the way) depends on the trajectory, so the GPU's result is
    checked as a converged solution: the DBC vertices are at least 99 % of
    the way, the fixed ones did not move, and the oracle started from it with
    every DBC vertex held where it is stops within a few iterations at its
    energy within 1e-6."""
    import idp_gb300 as idp

    pb, X, rows, tgt = two_bar_problem(oracle, -0.01, tol=1e-5)
    far = np.where(X[: rows[0], 0] < 0.05)[0]
    pb.dbc = pb.dbc.copy()
    pb.dbc[far] = 1
    pb.dbc_rows = np.concatenate([far.astype(np.int32), rows])
    pb.dbc_target = np.concatenate([X[far], tgt])
    pb.lam, pb.mu = pb.lam * 1e5, pb.mu * 1e5
    pb.max_iters = 100
    X0, kap0 = pb.X.copy(), list(pb.kappa)
    ctx, r, Xg, its = run_both(oracle, idp, pb, idp.MODE_FP64)
    prog = pb.last_stats["dbc_progress"]
    assert max(s for _, _, s in prog) >= 2e6  # the oracle did double
    assert r["status"] in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP)  # converged (a capped ACCD loop stays safe)
    assert np.array_equal(Xg[far], X[far])  # fixed rows stay
    d0 = np.linalg.norm(tgt - X[rows])
    assert np.linalg.norm(tgt - Xg[rows]) <= 0.01 * d0 + 1e-15
    pw = oracle.Problem(X=Xg.copy(), X0=X0, tets=pb.tets, mass=pb.mass, lam=pb.lam, mu=pb.mu, h=pb.h, dHat2=pb.dHat2,
                        kappa=[r["kappa"], r["kappa"], 0.0], v=np.zeros_like(X0), dbc=pb.dbc, tol=1e-5, max_iters=50)
    its_w = oracle.advance_one_step(pw, Xtilde=X0)
    rel = abs(r["energy"] - pw.last_energy) / abs(pw.last_energy)
    print(f"doubling: GPU {r['newton_iters']} iterations, oracle {its} (stiffness {[s for _, _, s in prog]}); "
          f"oracle from the GPU result {its_w} iterations, rel energy {rel:.2e}")
    assert its_w <= 10 and rel <= 1e-6
    ctx.close()


def test_targets_validated(gpu_lib):
    import idp_gb300 as idp
    from idp_gb300 import meshgen

    X, tets = meshgen.bar(1, 1, 2, size=(1.0, 1.0, 2.0), seed=0)
    m = meshgen.lumped_mass(X, tets, 1000.0)
    ctx = idp.Context()
    ctx.add_instance(X, tets, m, 1.0, 1.0, 1e-4, 1.0, 10.0)
    ctx.add_instance(X, tets, m, 1.0, 1.0, 1e-4, 1.0, 10.0, dbc_idx=[0, 1, 0])
    with pytest.raises(ValueError):
        ctx.set_dbc_targets(0, np.zeros((1, 3)))  # no DBC vertices
    with pytest.raises(idp.IDPError):
        ctx.set_dbc_targets(1, np.zeros((3, 3)))  # vertex 0 listed twice
    with pytest.raises(ValueError):
        ctx.set_dbc_targets(1, np.zeros((2, 3)))
    ctx.set_dbc_targets(1, None)
    ctx.close()


def test_hinge_call_with_moving_dbc_rows_matches_c_abi(oracle, gpu_lib):
    import idp_gb300 as idp
    from idp_gb300.api import FEM

    from test_gpu_driver import reference_args

    pb, X, rows, tgt = two_bar_problem(oracle, -0.01)
    pr = dict(mass=pb.mass, lam=pb.lam[0], mu=pb.mu[0], dHat2=pb.dHat2)
    DBC = np.concatenate([rows[:, None].astype(np.float64), tgt], axis=1)
    kappaVec = [pb.kappa[0], pb.kappa[1], 0.0]
    a = reference_args(X, pb.tets, pr, np.zeros_like(X), kappaVec, DBC, None)
    its = FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*list(a.values()))
    ctx = gpu_two_bars(idp, pb, idp.MODE_MIXED)
    _, r = ctx.advance(check=False)
    Xd, vd, kd = ctx.state(0)
    assert its == r[0]["newton_iters"]
    assert np.array_equal(a["X"], Xd) and np.array_equal(a["nodeAttr"]["v"], vd) and kappaVec[0] == kd[0]
    # the next call with the targets where the bar now is: every row fixed
    DBC2 = np.concatenate([rows[:, None].astype(np.float64), a["X"][rows]], axis=1)
    a["DBC"] = DBC2
    FEM.DiscreteShell.Advance_One_Step_IE_Hinge(*list(a.values()))
    assert np.array_equal(a["X"][rows], DBC2[:, 1:])
    ctx.close()


def test_twisting_bar_driver_matches_oracle(oracle, gpu_lib):
    """TetIPCSim with its bottom fixed (set_DBC, zero motion) and its top
    turning at 90 degrees per second (set_DBC with an angular velocity):
    Step_Dirichlet moves the top rows before each step and the Newton step
    puts the top vertices on them; three steps against the oracle fed the
    same rows."""
    import idp_gb300 as idp
    from idp_gb300 import dirichlet, meshgen
    from idp_gb300.api import TetIPCSim

    X, tets = meshgen.bar(2, 2, 6, size=(1.0, 1.0, 3.0), seed=0)
    sim = TetIPCSim(dt=0.1, PNTol=1e-5, mode=idp.MODE_FP64)
    sim.gravity = (0.0, 0.0, 0.0)  # Dirichlet motion only
    sim.add_object_3D(X, tets)
    sim.initialize_added_objects((0.0, 0.0, 0.0), 1000.0, 1e4, 0.3)
    sim.initialize_OIPC(1e-3 * float(np.linalg.norm(X.max(0) - X.min(0))), 0.0)
    sim.set_DBC((-0.1, -0.1, -0.1), (1.1, 1.1, 0.01), (0, 0, 0), (0, 0, 0), (0, 0, 1), 0.0)
    sim.set_DBC((-0.1, -0.1, 0.99), (1.1, 1.1, 1.1), (0, 0, 0), (0.5, 0.5, 3.0), (0, 0, 1), 90.0)
    rows = sim.DBC.indices.copy()
    assert len(sim.DBCMotion) == 2 and rows.size > 8
    # the oracle, fed the same rows step by step
    D, M = dirichlet.DBCStorage(sim.DBC.rows), dirichlet.DBCMotion([list(r) for r in sim.DBCMotion])
    T = tets.shape[0]
    mask = np.zeros(X.shape[0], np.uint8)
    mask[rows] = 1
    pb = oracle.Problem(X=X.copy(), X0=X, tets=tets, mass=sim.nodeAttr["m"], lam=sim.tetElasticity["lambda"],
                        mu=sim.tetElasticity["mu"], h=0.1, dHat2=sim.dHat2, kappa=list(sim.kappa), v=np.zeros_like(X),
                        dbc=mask, dbc_rows=rows, tol=1e-5)
    for _ in range(3):
        sim.advance_one_time_step()
        dirichlet.step_dirichlet(M, 0.1, D)
        pb.dbc_target = D.targets.copy()
        oracle.advance_one_step(pb)
        assert np.array_equal(D.rows, sim.DBC.rows)
        assert np.array_equal(sim.X[rows], D.targets)  # reached at once (nothing in the way)
        assert np.max(np.abs(sim.X - pb.X)) <= 1e-5
    # the top turned by 27 degrees about the bar's axis
    top = rows[(X[rows, 2] > 2.9) & (np.hypot(X[rows, 0] - 0.5, X[rows, 1] - 0.5) > 0.1)]
    ang = np.arctan2(sim.X[top, 1] - 0.5, sim.X[top, 0] - 0.5) - np.arctan2(X[top, 1] - 0.5, X[top, 0] - 0.5)
    assert np.allclose(np.mod(ang, 2 * np.pi), np.deg2rad(27.0), atol=1e-9)
