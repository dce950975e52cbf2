"""Generate tests/golden/baseline_configs.npz from the CPU oracle: the
oracle's results on two of the benchmark configurations, for the GPU tests
that compare against them at full size.

* bar (6x6x24 cubes x 5 tets = 4,320 tets, jitter 0.05h, seed 0; target =
  the centreline bent onto a circle of radius 0.5 over 2.2 pi, which
  self-intersects; neo-Hookean E = 1e4, nu = 0.3, inertia weight from
  density 1e3 and h = 0.1, d-hat = 1e-3 bbox diagonal, adaptive kappa):
  the oracle's Newton solve to PNTol 1e-5. Kept: three iterates of that
  trajectory (the most contact-heavy of every tenth iterate in each third
  of the trajectory), the Newton directions taken there and the constraint
  counts at them, the final energy and iteration count.
* blob (SH blob r = 1 + 0.3 sum c_lm Y_lm, l <= 8, seed 0, on a 64^3 grid:
  220,515 tets): the oracle's first normal-flow step (surface x_tilde = x +
  0.05 n) to PNTol 1e-5; kept: final energy and iteration count.

The oracle here is the restated reference (FP64, sparse Cholesky); running
it takes several minutes, which is why its outputs are committed. Inputs are
regenerated by the tests from the same seeds. Regenerate with

    python tests/golden/make_baseline_fixtures.py
"""
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

PNTOL = 1e-5


def bar_fixture(out):
    pb = O.make_bar_problem(6, 6, 24, angle=2.2 * math.pi, seed=0, tol=PNTOL)
    pb.max_iters = 5000
    rec = []

    def on_iter(it, Xp, sol, nc):
        if it % 10 == 0:
            rec.append((nc, it, Xp.copy(), sol.copy()))
        if it % 50 == 0:
            print(f"bar it {it} C {nc} E {pb.log[-1]['E']:.12e} res {pb.log[-1]['res']:.3e}", flush=True)

    t0 = time.perf_counter()
    it = O.advance_one_step(pb, on_iter=on_iter)
    print(f"bar converged: {it} iterations, E {pb.last_energy:.15e}, {time.perf_counter() - t0:.0f} s", flush=True)
    # the most contact-heavy recorded iterate in each third of the trajectory
    thirds = [[r for r in rec if k * it <= 3 * r[1] < (k + 1) * it] for k in range(3)]
    picks = [max(t, key=lambda r: (r[0], -r[1])) for t in thirds]
    out["bar_iters"] = np.array([r[1] for r in picks], np.int32)
    out["bar_ncons"] = np.array([r[0] for r in picks], np.int32)
    out["bar_X"] = np.stack([r[2] for r in picks])
    out["bar_dir"] = np.stack([r[3] for r in picks])
    out["bar_energy"] = np.array([pb.last_energy])
    out["bar_newton_iters"] = np.array([it], np.int32)
    out["bar_kappa_final"] = np.array([pb.kappa[0]])


def blob_fixture(out):
    sys.path.insert(0, ROOT)
    import bench

    p = bench.blob_problem(64)
    T = p["tets"].shape[0]
    surf = O.surface(p["X"], p["tets"])
    v = O.normal_flow_velocity(p["X"], surf["tris"], 0.05, 0.1)
    pb = O.Problem(X=p["X"].copy(), X0=p["X"], tets=p["tets"], mass=p["mass"], lam=np.full(T, p["lam"]),
                   mu=np.full(T, p["mu"]), h=0.1, dHat2=p["dHat2"], kappa=[p["kappa"], p["kappa_max"], 0.0],
                   v=v, tol=PNTOL, max_iters=500)
    t0 = time.perf_counter()
    it = O.advance_one_step(pb)
    print(f"blob step: {it} iterations, E {pb.last_energy:.15e}, {time.perf_counter() - t0:.0f} s", flush=True)
    out["blob_tets"] = np.array([T], np.int32)
    out["blob_energy"] = np.array([pb.last_energy])
    out["blob_newton_iters"] = np.array([it], np.int32)


def main():
    out = {}
    blob_fixture(out)
    bar_fixture(out)
    out["pntol"] = np.array([PNTOL])
    np.savez_compressed(os.path.join(HERE, "baseline_configs.npz"), **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()
