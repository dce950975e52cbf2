"""Generate the golden fixtures of this directory from the CPU oracle.

The reference ships no test vectors for this path and cannot be built here,
so these fixtures are produced by the oracle (the restated reference
algorithm) on seeded inputs. They pin the oracle against silent changes and
give the GPU tests fixed expected values. Regenerate with

    python tests/golden/make_golden.py

Every input is regenerated from seeds by the tests, so the fixtures hold only
seeds, sizes and expected outputs. The inputs use only numpy's portable
generator and elementary arithmetic, so they are bit-identical on every host.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402

import cases  # noqa: E402
from idp_gb300 import meshgen  # noqa: E402


def contact_case(seed):
    """Two jittered bars 2e-3 apart (many PT/EE constraints within d-hat 5e-3)."""
    X, tets = cases.two_bars(gap=2e-3, seed=seed)
    return X, tets


def ccd_case(seed):
    X, tets = cases.two_bars(gap=0.02, seed=seed)
    rng = np.random.default_rng(seed)
    V = X.shape[0]
    d = 0.05 * rng.normal(size=(V, 3))
    d[V // 2:, 0] -= 0.15
    return X, tets, d


def energy_case(seed):
    X0, tets = meshgen.bar(3, 3, 6, size=(1.0, 1.0, 2.0), seed=seed)
    Xd = meshgen.bend_target(X0, angle=0.7 * math.pi, radius=1.1, size=(1.0, 1.0, 2.0))
    return X0, tets, Xd


def flow_case(seed):
    """A jittered bar, slightly sheared (inputs built from numpy's portable
    generator and linspace only, so they are bit-identical on every host)."""
    X, tets = meshgen.bar(3, 3, 5, size=(1.0, 1.0, 1.6), jitter=0.05, seed=seed)
    X = X.copy()
    X[:, 0] += 0.1 * X[:, 2]
    return X, tets


def isect_case(seed):
    """A jittered bar and its bend onto 2.2 pi turns (self-intersecting)."""
    X, tets = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 4.0), seed=seed)
    return X, tets, meshgen.bend_target(X, angle=2.2 * math.pi)


def shell_case(seed):
    """The boundary of a jittered bar as a closed shell, sheared (portable
    arithmetic only), and a perturbed state of it."""
    X, tets = meshgen.bar(2, 3, 4, size=(1.0, 1.5, 2.0), seed=seed)
    Xs, F = meshgen.shell_from_tets(X, tets)
    Xs = Xs.copy()
    Xs[:, 0] += 0.1 * Xs[:, 2]
    rng = np.random.default_rng(100 + seed)
    Xd = Xs + 0.01 * rng.uniform(-1.0, 1.0, Xs.shape)
    return Xs, F, Xd


def step_case():
    """A bar bent 1.6 pi into a ring whose ends approach (contact, no overlap)."""
    X, tets = meshgen.bar(2, 2, 6, size=(1.0, 1.0, 2.4), seed=0)
    target = meshgen.bend_target(X, angle=1.6 * math.pi, radius=0.45, size=(1.0, 1.0, 2.4))
    return X, tets, target


def main():
    O.build()
    out = {}
    for seed in range(2):
        X, tets = contact_case(seed)
        surf = O.surface(X, tets)
        pr = cases.problem(X, tets, dHat=5e-3)
        cons, info = O.constraint_set(X, X, surf, np.zeros(X.shape[0], np.uint8), pr["dHat2"])
        order = np.lexsort(cons.T[::-1])
        out[f"contact{seed}_surf_tris"] = surf["tris"]
        out[f"contact{seed}_surf_edges"] = surf["edges"]
        out[f"contact{seed}_surf_nodes"] = surf["nodes"]
        out[f"contact{seed}_cons"] = cons[order]
        out[f"contact{seed}_dhat2"] = np.array([pr["dHat2"]])
        out[f"contact{seed}_kappa"] = np.array([pr["kappa"]])
        out[f"contact{seed}_barrier_E"] = np.array([O.barrier_energy(cons, info, X, X, pr["dHat2"], pr["kappa"])])
        out[f"contact{seed}_barrier_g"] = O.barrier_gradient(cons, info, X, X, pr["dHat2"], pr["kappa"])
    for seed in range(2):
        X, tets, d = ccd_case(seed)
        for k, a0 in enumerate((1.0, 0.37)):
            a, rc = O.ccd_stepsize(X, d.reshape(-1), O.surface(X, tets), np.zeros(X.shape[0], np.uint8), a0)
            out[f"ccd{seed}_{k}_alpha"] = np.array([a, a0])
    for seed in range(2):
        X0, tets, Xd = energy_case(seed)
        IB, vol = O.tet_rest(X0, tets)
        pr = cases.problem(X0, tets)
        lam = np.full(tets.shape[0], pr["lam"])
        mu = np.full(tets.shape[0], pr["mu"])
        out[f"tet{seed}_E"] = np.array([O.tet_energy(Xd, tets, IB, vol, lam, mu, 0.01)])
        out[f"tet{seed}_g"] = O.tet_gradient(Xd, tets, IB, vol, lam, mu, 0.01)
    for seed in range(2):
        X, tets = flow_case(seed)
        out[f"flow{seed}_v"] = O.normal_flow_velocity(X, O.surface(X, tets)["tris"], 0.05, 0.1)
    for seed in range(2):
        X, tets, Xt = isect_case(seed)
        out[f"isect{seed}_pairs"] = O.edge_tri_intersections(Xt, O.surface(X, tets))
    for seed in range(2):
        Xs, F, Xd = shell_case(seed)
        keep, mass, vol = O.shell_init(Xs, F, 1000.0, 0.01)
        surf = O.shell_surface(Xs.shape[0], F)
        out[f"shell{seed}_edges"] = surf["edges"]
        out[f"shell{seed}_mass"] = mass
        out[f"shell{seed}_flowE"] = np.array([O.flow_energy(Xd, F, vol, 0.5)])
        out[f"shell{seed}_flowg"] = O.flow_gradient(Xd, F, vol, 0.5)
    X, tets, target = step_case()
    pr = cases.problem(X, tets)
    T = tets.shape[0]
    pb = O.Problem(X=X.copy(), X0=X, tets=tets, mass=pr["mass"], lam=np.full(T, pr["lam"]), mu=np.full(T, pr["mu"]),
                   h=0.1, dHat2=pr["dHat2"], kappa=[pr["kappa"], pr["kappa_max"], 0.0], v=(target - X) / 0.1,
                   tol=1e-3, max_iters=400)
    it = O.advance_one_step(pb)
    out["step_newton_iters"] = np.array([it])
    out["step_energy"] = np.array([pb.last_energy])
    out["step_X"] = pb.X
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
