"""The oracle's moving Dirichlet conditions (IMPLICIT_EULER.h:305-401,
701-757; FEM/Shell/DIRICHLET.h): DBC vertices move onto their targets at once
when the CCD step of their displacement is 1, and through the augmented
Lagrangian's penalty when contact blocks the way."""
import numpy as np

import cases


def two_bar_problem(oracle, shift, tol=1e-3):
    X, tets = cases.two_bars(gap=2e-3, seed=0)
    pr = cases.problem(X, tets, dHat=5e-3)
    V, T = X.shape[0], tets.shape[0]
    rows = np.arange(V // 2, V, dtype=np.int32)  # the second bar, every vertex
    tgt = X[rows].copy()
    tgt[:, 0] += shift
    dbc = np.zeros(V, np.uint8)
    dbc[rows] = 1
    pb = oracle.Problem(X=X.copy(), X0=X, tets=tets, mass=pr["mass"], lam=np.full(T, pr["lam"]),
                        mu=np.full(T, pr["mu"]), h=0.1, dHat2=pr["dHat2"], kappa=[pr["kappa"], pr["kappa_max"], 0.0],
                        v=np.zeros_like(X), dbc=dbc, dbc_rows=rows, dbc_target=tgt, tol=tol, max_iters=400)
    return pb, X, rows, tgt


def test_unobstructed_targets_are_reached_at_once(oracle):
    pb, X, rows, tgt = two_bar_problem(oracle, +0.05)  # away from the first bar
    oracle.advance_one_step(pb)
    assert pb.dbc_alpha == 1.0
    assert np.array_equal(pb.X[rows], tgt)
    assert pb.last_stats["dbc_progress"] == []
    assert np.max(np.abs(pb.X[: rows[0]] - X[: rows[0]])) < 1e-12  # nothing pushed the first bar


def test_blocked_targets_through_the_penalty(oracle):
    """The second bar is moved 1 cm into the first (gap 2 mm): the CCD step of
    the displacement is below 1, the penalty pulls the bar there and the
    first bar is pushed away, with no intersection."""
    pb, X, rows, tgt = two_bar_problem(oracle, -0.01)
    its = oracle.advance_one_step(pb)
    assert 0 < pb.dbc_alpha < 1
    prog = pb.last_stats["dbc_progress"]
    assert prog and prog[0][2] == 1e6 and prog[-1][1] >= 0.99
    d0 = np.linalg.norm(tgt - X[rows])
    assert np.linalg.norm(tgt - pb.X[rows]) <= 0.01 * d0
    assert np.max(X[: rows[0], 0] - pb.X[: rows[0], 0]) > 5e-3  # the first bar gave way
    assert len(oracle.edge_tri_intersections(pb.X, pb.surf)) == 0
    assert pb.log[-1]["dbc_stiff"] == 0 and its >= 2


def test_penalty_stiffness_doubles_when_the_solve_settles(oracle):
    """A stiff first bar fixed at its far side: the penalty alone cannot pull
    the second bar 99 % of the way in one solve, so the stiffness doubles
    (IMPLICIT_EULER.h:722-738) before the conditions are met."""
    pb, X, rows, tgt = two_bar_problem(oracle, -0.01)
    far = np.where(X[: rows[0], 0] < 0.05)[0]
    pb.dbc = pb.dbc.copy()
    pb.dbc[far] = 1
    pb.dbc_rows = np.concatenate([far.astype(np.int32), rows])
    pb.dbc_target = np.concatenate([X[far], tgt])
    pb.lam, pb.mu = pb.lam * 1e5, pb.mu * 1e5
    pb.max_iters = 100
    oracle.advance_one_step(pb)
    prog = pb.last_stats["dbc_progress"]
    stiffs = [s for _, _, s in prog]
    assert stiffs[0] == 1e6 and max(stiffs) >= 2e6 and prog[-1][1] >= 0.99
