"""Benchmark of the injective-deformation Newton step on GB300.

Default workload ``blob`` (single large normal-flow solve): a closed bumpy
blob r(u) = 1 + 0.3 * sum_{l<=8} c_lm Y_lm (c ~ N(0, 1/l^2), seed 0),
tetrahedralised on a 64^3 background grid (220,515 tets, 49,863 vertices).
A step is one normal-flow solve: every surface vertex's predictor moves by
0.05 along its area-weighted outward normal, interior vertices are held
(x_tilde = x), and idp_advance runs Newton to convergence with the IPC
barrier, CCD-filtered line search and the mixed-precision PCG. W warm-up
steps and K timed steps continue one flow sequence (20 steps for K=17, W=3).

* value: solves/s with the state resident in HBM; time = the library's
  CUDA-event time of each step on its own stream, summed over the K steps.
* fp64: the same K steps re-solved in FP64 mode from the identical start
  states (positions, velocity, kappa); its solves/s and the relative energy
  difference mixed vs FP64 are reported per run.
* e2e: the same K steps through the public API with host buffers: pinned
  positions uploaded, normal flow set, solved, positions read back, all in
  the timed region (host wall clock around synchronous calls).
* roofline: the cluster PCG kernel (dominant), algorithmic bytes per launch /
  event time, against MEASURED_PEAKS.json hbm_gbs.
* cpu_baseline and oracle_check: the CPU oracle (FP64, sparse Cholesky)
  solving the first timed step(s) of the same full-size blob from the GPU's
  start states (at least one step, more while --cpu-sample-s lasts): its
  solves/s, and the GPU energies' relative error against it per step.
* constraints_per_step: the constraint-set size at the end of each step.

``--workload batch256`` (256 bars, tet counts log-uniform in [1k, 50k]) and
``--workload bar`` (6x6x24 bar, bend 2.2pi) time one batched solve per step
from a restored device snapshot instead. ``--workload serve`` drives the
request server with Poisson arrivals, ``anim`` the animation-fix cylinder,
``shellflow`` flow mode on a triangle shell, and ``charseq`` the
character-sequence script on an elastic shell (frames/s; the mesh and
frames by path, or a synthetic turning shell).

``--impl reference`` times the reference's CPU path (the oracle port: the
reference does not build in this environment) on the same metric: on the
blob, full-size flow steps from the rest state (at least one, as many as
about 2.5 minutes allow; "steps" is the number that ran).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/sec & p50/p99 latency, mixed vs FP64 GPU at <=1e-6 rel energy err"
UNIT = "solves/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=17)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="blob",
                    choices=["blob", "batch256", "bar", "serve", "anim", "shellflow", "charseq"])
    ap.add_argument("--charseq-mesh", default="", help="charseq: rest shell (OBJ), e.g. the mannequin wm2_15k.obj; "
                    "empty: a synthetic bumpy shell")
    ap.add_argument("--charseq-frames", default="", help="charseq: folder of frame OBJs 1.obj, 2.obj, ... "
                    "(e.g. Rumba_Dancing_unfixed); empty: synthetic frames")
    ap.add_argument("--charseq-n", type=int, default=68, help="charseq: background grid of the synthetic shell")
    ap.add_argument("--shell-n", type=int, default=48, help="shellflow: background grid of the blob whose surface is "
                                                            "the shell")
    ap.add_argument("--frames", type=int, default=120, help="anim: keyframes solved")
    ap.add_argument("--frame-stride", type=int, default=1, help="anim: keyframe step")
    ap.add_argument("--anim-n", type=int, default=22, help="anim: cells across the cylinder's diameter")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: Poisson arrival rate (jobs/s)")
    ap.add_argument("--duration", type=float, default=4.0, help="serve: seconds of arrivals")
    ap.add_argument("--serve-workers", type=int, default=4)
    ap.add_argument("--serve-batch", type=int, default=8)
    ap.add_argument("--hbm-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-newton-cap", type=int, default=30)
    ap.add_argument("--serve-pool", type=int, default=8, help="serve: bars and blobs in the job pool (each)")
    ap.add_argument("--serve-max-bar-tets", type=int, default=50_000)
    ap.add_argument("--serve-max-blob-tets", type=int, default=100_000)
    ap.add_argument("--blob-n", type=int, default=64)
    ap.add_argument("--flow-step", type=float, default=0.05)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--pcg-rel-tol", type=float, default=0.0,
                    help="PCG relative tolerance of the timed arm (0 = library default); the FP64 arm keeps the default")
    ap.add_argument("--pcg-grid-cta-vertices", type=int, default=0,
                    help="vertices per CTA of the grid-wide PCG (0 = library default)")
    ap.add_argument("--pcg-local-degree", type=int, default=-1,
                    help="grid PCG's CTA-local polynomial preconditioner degree (-1 = library default, 0 = block Jacobi)")
    ap.add_argument("--caller-vertex-order", action="store_true",
                    help="keep the caller's vertex order on the device (default: spatial order)")
    ap.add_argument("--progress", action="store_true", help="print progress lines to stderr")
    ap.add_argument("--autotune", action="store_true",
                    help="pick the PCG tile and preconditioner shapes with idp_gb300.autotune before timing "
                         "(untimed; cached per workload kind)")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--max-newton", type=int, default=2000)
    ap.add_argument("--newton-budget", type=int, default=0,
                    help="batch/bar workloads: stop every instance after this many Newton iterations and report "
                         "Newton iterations/s (0 = solve to convergence, report solves/s)")
    ap.add_argument("--fp64-sample", type=int, default=16,
                    help="batch/bar workloads: instances re-solved one at a time on the FP64 path")
    ap.add_argument("--cpu-sample-s", type=float, default=20.0,
                    help="CPU baseline budget (at least one full solve runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def extra_params(args):
    """Library parameters the command line sets for the timed arm."""
    kw = {}
    if args.pcg_local_degree >= 0:
        kw["pcg_local_degree"] = args.pcg_local_degree
    if args.caller_vertex_order:
        kw["caller_vertex_order"] = 1
    return kw


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, world):
    """Max of a per-rank float over all ranks (every rank gets it); the
    ranks' timed regions are reported by their slowest rank."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_workload(args, seed):
    import numpy as np
    from idp_gb300 import meshgen

    if args.workload == "bar":
        X, tets = meshgen.bar(6, 6, 24, seed=seed)
        items = [dict(X=X, tets=tets, target=meshgen.bend_target(X, angle=2.2 * math.pi))]
        desc = "bar: 6x6x24 cubes x 5 tets (4320 tets), bend 2.2pi"
    else:
        items = meshgen.bar_batch(args.instances, 1_000, 50_000, seed=seed)
        desc = (f"batch{args.instances}_bars: tets log-uniform [1k,50k], bend U[1.5pi,2.5pi], jitter 0.05h, "
                "one arena")
    probs = []
    for it in items:
        X, tets = it["X"], it["tets"]
        mass = meshgen.lumped_mass(X, tets, 1000.0)
        lam, mu = meshgen.lame(1e4, 0.3)
        diag = float(np.linalg.norm(X.max(0) - X.min(0)))
        dHat2 = (1e-3 * diag) ** 2
        from idp_gb300.api import initialize_oipc

        k, km = initialize_oipc(float(mass.mean()), dHat2)
        probs.append(dict(X=X, tets=tets, target=it["target"], mass=mass, lam=lam, mu=mu, dHat2=dHat2, kappa=k,
                          kappa_max=km))
    return probs, desc


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.rows = []
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    p = os.path.join(ROOT, "profiles", "pcg_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


def cpu_baseline(probs, budget_s, newton_budget=0):
    """Oracle (FP64, direct solve) on a bounded sample: solves of the
    smallest instances (capped at newton_budget Newton iterations when it is
    set) until the time budget is spent; throughput extrapolated to the
    workload by tet count (solves/s, or Newton iterations/s summed over the
    workload's instances when newton_budget is set)."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    order = sorted(range(len(probs)), key=lambda i: probs[i]["tets"].shape[0])
    t_used, tets_done, solved, iters = 0.0, 0, 0, 0
    for i in order:
        p = probs[i]
        T = p["tets"].shape[0]
        pb = O.Problem(X=p["X"].copy(), X0=p["X"], tets=p["tets"], mass=p["mass"], lam=np.full(T, p["lam"]),
                       mu=np.full(T, p["mu"]), h=0.1, dHat2=p["dHat2"], kappa=[p["kappa"], p["kappa_max"], 0.0],
                       v=(p["target"] - p["X"]) / 0.1, tol=1e-3, max_iters=newton_budget or 2000)
        t0 = time.perf_counter()
        iters += O.advance_one_step(pb)
        t_used += time.perf_counter() - t0
        tets_done += T
        solved += 1
        if t_used >= budget_s:
            break
    mean_tets = sum(p["tets"].shape[0] for p in probs) / len(probs)
    rate = tets_done / t_used / mean_tets  # workload solves per second
    unit = UNIT
    if newton_budget:
        # Newton iterations per second at the mean instance size
        rate = iters / t_used * (tets_done / solved) / mean_tets
        unit = "newton_iters/s"
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": rate, "unit": unit, "cores": cores, "kind": "port",
            "sample": (f"oracle {'solves capped at %d Newton iterations' % newton_budget if newton_budget else 'full solves'}"
                       f" of the {solved} smallest instance(s) ({tets_done} tets, {iters} Newton iterations, "
                       f"{t_used:.1f} s); scaled to the mean instance ({mean_tets:.0f} tets); element and contact "
                       "loops OpenMP on all cores, sparse LU (SciPy SuperLU) on one")}


H = 0.1


def blob_problem(n, seed=0):
    import numpy as np
    from idp_gb300 import meshgen
    from idp_gb300.api import initialize_oipc

    X, tets, _ = meshgen.blob(n=n, lmax=8, amp=0.3, seed=seed)
    mass = meshgen.lumped_mass(X, tets, 1000.0)
    lam, mu = meshgen.lame(1e4, 0.3)
    dHat2 = (1e-3 * float(np.linalg.norm(X.max(0) - X.min(0)))) ** 2
    k, km = initialize_oipc(float(mass.mean()), dHat2)
    return dict(X=X, tets=tets, mass=mass, lam=lam, mu=mu, dHat2=dHat2, kappa=k, kappa_max=km)


def blob_desc(p, n, step):
    return (f"blob_normal_flow: SH blob lmax 8 amp 0.3 seed 0 on {n}^3 grid ({p['tets'].shape[0]} tets, "
            f"{p['X'].shape[0]} verts), surface x_tilde = x + {step} n, interior x_tilde = x, h=0.1, "
            f"E=1e4 nu=0.3 rho=1e3, dhat=1e-3 bbox diag")


def oracle_flow_steps(p, starts, step, budget_s, tol=1e-3):
    """The oracle (FP64, sparse Cholesky) solving normal-flow steps of the
    full blob: step k starts from starts[k] = (X, kappa[3]) (the next start
    is the oracle's own result when starts[k+1] is None), at least one step,
    more while the time budget lasts. Returns per-step results and the
    time spent in the steps."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    T = p["tets"].shape[0]
    surf = O.surface(p["X"], p["tets"])
    out, t_used = [], 0.0
    X, kap = None, None
    for k, st in enumerate(starts):
        if st is not None:
            X, kap = st[0], st[1]
        v = O.normal_flow_velocity(X, surf["tris"], step, H)
        pb = O.Problem(X=X.copy(), X0=p["X"], tets=p["tets"], mass=p["mass"], lam=np.full(T, p["lam"]),
                       mu=np.full(T, p["mu"]), h=H, dHat2=p["dHat2"], kappa=[kap[0], kap[1], 0.0], v=v, tol=tol,
                       max_iters=500)
        pb.surf = surf
        t0 = time.perf_counter()
        it = O.advance_one_step(pb)
        t_used += time.perf_counter() - t0
        out.append(dict(energy=pb.last_energy, newton_iters=it, constraints=int(pb.log[-1]["ncons"])))
        X, kap = pb.X.copy(), [pb.kappa[0], pb.kappa[1], 0.0]
        if t_used >= budget_s:
            break
    return out, t_used


def cpu_cores():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def run_flow(args):
    import numpy as np
    import torch
    import idp_gb300 as idp

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    mode = idp.MODE_MIXED if args.mode == "mixed" else idp.MODE_FP64
    # replicas: every rank runs its own blob (seeded by rank)
    p = blob_problem(args.blob_n, seed=rank)
    desc = blob_desc(p, args.blob_n, args.flow_step)
    V = p["X"].shape[0]

    tuned = None
    if args.autotune:
        from idp_gb300 import autotune

        inst = [dict(p, normal_flow=args.flow_step)]
        tp, rec = autotune.tune(inst, base=dict(h=H, newton_tol=1e-3, mode=mode), device_name=None)
        tuned = {k: tp[k] for k in autotune.DEFAULT_SPACE}
        tuned_rec = {"params": tuned, "step_ms": rec["ms"], "cached": rec["cached"]}

    def make_ctx(m, timed_arm=True):
        kw = {}
        if tuned and timed_arm:
            kw.update(tuned)
        if timed_arm and args.pcg_rel_tol > 0:
            kw["pcg_rel_tol"] = args.pcg_rel_tol
        if args.pcg_local_degree >= 0:
            kw["pcg_local_degree"] = args.pcg_local_degree
        if args.caller_vertex_order:
            kw["caller_vertex_order"] = 1
        kw.setdefault("pcg_grid_cta_vertices", args.pcg_grid_cta_vertices)
        c = idp.Context(h=H, newton_tol=1e-3, max_newton=args.max_newton, mode=m, device=local, **kw)
        c.add_instance(p["X"], p["tets"], p["mass"], p["lam"], p["mu"], p["dHat2"], p["kappa"], p["kappa_max"])
        c.commit()
        return c

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    ctx = make_ctx(mode)
    for _ in range(args.warmup):
        ctx.set_normal_flow(0, args.flow_step)
        ctx.advance(check=False)
    # start states of the timed steps (host copies taken outside the device
    # time of each step; they let the FP64 and e2e passes redo the same work)
    starts = []
    dev_ms, wall, results = [], [], []
    launches = 0
    pcg_ms = pcg_bytes = 0.0
    phase = {k: 0.0 for k in ("pcg_ms", "tet_ms", "contact_ms", "ccd_ms")}
    barrier()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            starts.append(ctx.state(0))
            t0 = time.perf_counter()
            ctx.set_normal_flow(0, args.flow_step)
            rc, res = ctx.advance(check=False)
            wall.append(time.perf_counter() - t0)
            st = ctx.stats()
            dev_ms.append(st["total_ms"])
            pcg_ms += st["pcg_ms"]
            pcg_bytes += st["pcg_bytes"]
            launches += st["kernel_launches"] + 1
            for k in phase:
                phase[k] += st[k]
            results.append(res[0])
    barrier()
    total_ms = max_over_ranks(sum(dev_ms), world)
    value = world * args.steps / (total_ms / 1000.0)

    # ---- FP64 arm from the same start states
    fp64 = None
    if not args.no_fp64 and mode == idp.MODE_MIXED:
        cd = make_ctx(idp.MODE_FP64, timed_arm=False)
        d_ms, rel, energies64 = [], [], []
        for k, (Xs, vs, ks) in enumerate(starts):
            cd.set_positions(0, Xs)
            cd.set_kappa(0, ks)
            cd.set_normal_flow(0, args.flow_step)
            _, rd = cd.advance(check=False)
            d_ms.append(cd.stats()["total_ms"])
            Em, Ed = results[k]["energy"], rd[0]["energy"]
            energies64.append(Ed)
            rel.append(abs(Em - Ed) / max(abs(Ed), 1e-300))
        fp64 = {"solves_per_s": len(d_ms) / (sum(d_ms) / 1000.0), "ms_per_step": statistics.mean(d_ms),
                "energies": energies64,
                "rel_energy_err_max": max(rel), "rel_energy_err_mean": statistics.mean(rel),
                "mixed_speedup": (sum(d_ms) / total_ms) if total_ms > 0 else None}
        cd.close()

    # ---- end to end through the public API with pinned host buffers
    Xh = [torch.from_numpy(np.ascontiguousarray(Xs)).pin_memory() for Xs, _, _ in starts]
    Xo = torch.empty_like(Xh[0]).pin_memory()
    e2e_wall = []
    for k, (Xs, vs, ks) in enumerate(starts):
        ctx.set_kappa(0, ks)
        barrier()
        t0 = time.perf_counter()
        ctx.set_positions_ptr(0, Xh[k].data_ptr())
        ctx.set_normal_flow(0, args.flow_step)
        ctx.advance(check=False)
        ctx.state_ptr(0, Xo.data_ptr())
        e2e_wall.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(sum(e2e_wall), world)
    e2e_val = world * len(e2e_wall) / e2e_s
    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    achieved = (pcg_bytes / (pcg_ms / 1000.0) / 1e9) if pcg_ms > 0 else None
    traffic = ncu_traffic()
    lat = [r["latency_ms"] for r in results]
    newton = [r["newton_iters"] for r in results]
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mode == idp.MODE_MIXED else "f64", "data": "synthetic",
        "config": {"workload": desc, "tets": int(p["tets"].shape[0]), "verts": V, "mode": args.mode,
                   "parallelism": f"replicas{world}",
                   "l2": "working set larger than L2 (BSR + tet data + vectors > 129 MB); no flush"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "newton_iters": {"mean": float(np.mean(newton)), "max": int(np.max(newton)), "total": int(np.sum(newton))},
        "pcg_iters_per_newton": float(sum(r["pcg_iters"] for r in results) / max(1, int(np.sum(newton)))),
        "autotune": tuned_rec if tuned else None,
        "status": sorted({int(r["status"]) for r in results}),
        "phase_ms_per_step": {k: v / args.steps for k, v in phase.items()},
        "fp64": fp64,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 3 * V * 8, "d2h_bytes_per_step": 3 * V * 8},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": traffic.get("bytes_per_launch") if traffic else None,
                     "kernel": "k_pcg_grid (grid-wide cooperative PCG: BSR rows resident in shared memory, "
                               "FP32 SpMV + block-Jacobi, one reduction round per iteration)",
                     "achieved_basis": "algorithmic bytes of the PCG iterations / PCG event time",
                     "traffic_basis": "ncu DRAM read+write bytes of one launch (profiles/pcg_traffic.json)",
                     "peak_source": peak_kind},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "wall_ms_per_step": 1000 * statistics.mean(wall),
    }
    cons = [int(r["num_constraints"]) for r in results]
    out["constraints_per_step"] = {"min": min(cons), "max": max(cons), "mean": float(np.mean(cons)),
                                   "steps_with_contact": sum(1 for c in cons if c > 0)}
    if not args.no_cpu_baseline:
        # the oracle solves the first timed steps from the same start states
        # (full size); its time is the CPU baseline, its energies the
        # error check of those steps
        ores, t_or = oracle_flow_steps(p, [(X, k) for X, _, k in starts], args.flow_step, args.cpu_sample_s)
        n = len(ores)
        rel_m = [abs(results[k]["energy"] - ores[k]["energy"]) / abs(ores[k]["energy"]) for k in range(n)]
        chk = {"steps": n, "first_step": args.warmup + 1, "rel_energy_err_mixed": rel_m,
               "max": max(rel_m), "oracle_newton_iters": [o["newton_iters"] for o in ores],
               "gpu_newton_iters": [results[k]["newton_iters"] for k in range(n)],
               "oracle_constraints": [o["constraints"] for o in ores]}
        if fp64 is not None:
            chk["rel_energy_err_fp64"] = [abs(fp64["energies"][k] - ores[k]["energy"]) / abs(ores[k]["energy"])
                                          for k in range(n)]
        out["oracle_check"] = chk
        out["cpu_baseline"] = {
            "value": n / t_or, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
            "sample": f"oracle (FP64, sparse Cholesky) solving {n} full normal-flow step(s) of the same "
                      f"{int(p['tets'].shape[0])}-tet blob (steps {args.warmup + 1}-{args.warmup + n} of the "
                      f"sequence, from the GPU's start states), {t_or:.1f} s; element, contact and front "
                      "assembly loops OpenMP, dense fronts multithreaded BLAS, on all cores"}
    if fp64 is not None:
        fp64.pop("energies", None)
    print(json.dumps(out), flush=True)


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    if args.workload in ("serve", "anim", "shellflow", "charseq"):
        print(json.dumps({"impl": "reference", "unavailable": f"{args.workload}: the reference's CPU path (the "
                          "oracle port) is timed on the blob and batch workloads only"}))
        return
    vals = []
    bl = None
    if args.workload == "blob":
        # the full blob's flow sequence from its rest state, one full step
        # at least, more while about 2.5 minutes last; no warm-up (nothing
        # to warm on the CPU); steps = the steps that ran
        p = blob_problem(args.blob_n)
        desc = blob_desc(p, args.blob_n, args.flow_step)
        starts = [(p["X"], [p["kappa"], p["kappa_max"], 0.0])] + [None] * max(0, args.steps - 1)
        ores, t_or = oracle_flow_steps(p, starts, args.flow_step, 150.0)
        n = len(ores)
        v = n / t_or
        out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": n,
               "warmup": 0, "ms_per_step": 1000.0 * t_or / n, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": desc, "tets": int(p["tets"].shape[0]), "verts": int(p["X"].shape[0])},
               "newton_iters": [o["newton_iters"] for o in ores], "energies": [o["energy"] for o in ores],
               "constraints": [o["constraints"] for o in ores],
               "cpu_baseline": {"value": v, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
                                "sample": f"oracle (FP64, sparse Cholesky) solving flow steps 1-{n} of the full "
                                          f"{int(p['tets'].shape[0])}-tet blob from its rest state, {t_or:.1f} s; "
                                          "element, contact and front assembly loops OpenMP, dense fronts "
                                          "multithreaded BLAS, on all cores"},
               "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "note": "reference CPU path = oracle port (the reference does not build in this environment: "
                       "Eigen, CHOLMOD, Boost and Kokkos are absent)"}
        print(json.dumps(out))
        return
    metric, unit = METRIC, UNIT
    if args.workload != "blob":
        probs, desc = make_workload(args, seed=0)
        if args.newton_budget > 0:
            desc += f"; first {args.newton_budget} Newton iterations of every instance from the rest state"
            metric = "Newton iterations/s (summed over instances), mixed batched vs FP64 one at a time"
            unit = "newton_iters/s"
        per_step = min(args.cpu_sample_s, 150.0 / max(1, args.warmup + args.steps))
        for _ in range(args.warmup + args.steps):
            bl = cpu_baseline(probs, per_step, args.newton_budget)
            vals.append(bl["value"])
    v = statistics.mean(vals[args.warmup:]) if args.steps else vals[-1]
    out = {"impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v if v else None,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": desc, "instances": len(probs)},
           "cpu_baseline": dict(bl, value=v),
           "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "reference CPU path = oracle port (the reference does not build here: Eigen, CHOLMOD, Boost "
                   "and Kokkos are absent)"}
    print(json.dumps(out))


def run_gpu(args):
    import numpy as np
    import torch
    import idp_gb300 as idp

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    mode = idp.MODE_MIXED if args.mode == "mixed" else idp.MODE_FP64
    torch.cuda.set_device(local)
    # replicas: every rank solves its own copy of the workload (seeded by rank)
    probs, desc = make_workload(args, seed=rank)
    budget = args.newton_budget
    max_newton = budget if budget > 0 else args.max_newton
    if budget > 0:
        desc += f"; first {budget} Newton iterations of every instance from the rest state"
    ctx = idp.Context(h=0.1, newton_tol=1e-3, max_newton=max_newton, mode=mode, device=local, **extra_params(args))
    for i, p in enumerate(probs):
        ctx.add_instance(p["X"], p["tets"], p["mass"], p["lam"], p["mu"], p["dHat2"], p["kappa"], p["kappa_max"])
        ctx.set_velocity(i, (p["target"] - p["X"]) / 0.1)
    ctx.commit()
    ctx.save_state()
    nI = len(probs)
    total_tets = sum(p["tets"].shape[0] for p in probs)
    total_verts = sum(p["X"].shape[0] for p in probs)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def progress(msg):
        if args.progress and rank == 0:
            print(f"[{time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)

    # ---- resident inputs: restore the device snapshot, advance
    for w in range(args.warmup):
        ctx.restore_state()
        t0 = time.perf_counter()
        if args.progress:
            # the warm-up solve in slices of 100 Newton iterations, reporting
            # how many instances are still iterating (same result as advance)
            ctx.step_begin()
            n_active, done = len(probs), 0
            while n_active:
                _, n_active, rw = ctx.step_iterate(100)
                done += 100
                progress(f"warm-up step {w}: {done} iterations, {n_active} instances iterating, "
                         f"{time.perf_counter() - t0:.0f} s")
        else:
            _, rw = ctx.advance(check=False)
        progress(f"warm-up step {w}: {time.perf_counter() - t0:.1f} s, Newton max "
                 f"{max(r['newton_iters'] for r in rw)}, converged "
                 f"{sum(1 for r in rw if r['status'] in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP))}/{len(rw)}")
    barrier()
    dev_ms, wall, lat, results, launches = [], [], [], None, 0
    pcg_ms = pcg_bytes = 0.0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            ctx.restore_state()
            t0 = time.perf_counter()
            rc, results = ctx.advance(check=False)
            wall.append(time.perf_counter() - t0)
            st = ctx.stats()
            dev_ms.append(st["total_ms"])
            pcg_ms += st["pcg_ms"]
            pcg_bytes += st["pcg_bytes"]
            launches += st["kernel_launches"]
            lat += [r["latency_ms"] for r in results]
            progress(f"timed step: {wall[-1]:.1f} s wall, {dev_ms[-1] / 1000:.1f} s device")
    barrier()
    step_ms = max_over_ranks(statistics.mean(dev_ms), world)
    iters_step = sum(r["newton_iters"] for r in results)
    # a solve counts when Newton met its stopping test (IDP_OK, or
    # IDP_WARN_ITER_CAP: converged with a capped, still conservative CCD
    # loop); instances stopped at max_newton are reported as capped
    conv_ok = (idp.IDP_OK, idp.IDP_WARN_ITER_CAP)
    n_conv = sum(1 for r in results if r["status"] in conv_ok)
    metric, unit = METRIC, UNIT
    if budget > 0:
        metric = "Newton iterations/s (summed over instances), mixed batched vs FP64 one at a time"
        unit = "newton_iters/s"
        value = world * iters_step / (step_ms / 1000.0)
    else:
        value = world * n_conv / (step_ms / 1000.0)
    # exact intersection check and inversion status of every instance's result
    counts = ctx.intersection_counts()
    injective = {"checked": nI, "intersection_free": int((counts == 0).sum()),
                 "inverted": sum(1 for r in results if r["status"] == idp.IDP_ERR_INVERTED)}
    fp64_single = fp64_one_at_a_time(idp, probs, results, args.fp64_sample, max_newton, budget, local, progress) \
        if rank == 0 and mode == idp.MODE_MIXED and args.fp64_sample > 0 else None

    # ---- end to end with host buffers (pinned), copies inside the timed region
    Xh = [torch.from_numpy(np.ascontiguousarray(p["X"])).pin_memory() for p in probs]
    Vh = [torch.from_numpy(np.ascontiguousarray((p["target"] - p["X"]) / 0.1)).pin_memory() for p in probs]
    Xo = [torch.empty_like(x).pin_memory() for x in Xh]
    e2e_wall = []
    for _ in range(max(1, args.steps)):
        ctx.restore_state()  # kappa back to its initial value (positions are uploaded below)
        barrier()
        t0 = time.perf_counter()
        for i in range(nI):
            ctx.set_positions_ptr(i, Xh[i].data_ptr())
            ctx.set_velocity_ptr(i, Vh[i].data_ptr())
        ctx.advance(check=False)
        for i in range(nI):
            ctx.state_ptr(i, Xo[i].data_ptr())
        e2e_wall.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(statistics.mean(e2e_wall), world)
    e2e_val = world * (iters_step if budget > 0 else n_conv) / e2e_s
    h2d = 2 * 3 * total_verts * 8
    d2h = 3 * total_verts * 8

    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    achieved = (pcg_bytes / (pcg_ms / 1000.0) / 1e9) if pcg_ms > 0 else None
    status = {}
    for r in results:
        status[str(r["status"])] = status.get(str(r["status"]), 0) + 1
    newton = [r["newton_iters"] for r in results]
    out = {
        "metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mode == idp.MODE_MIXED else "f64", "data": "synthetic",
        "config": {"workload": desc, "instances": nI, "total_tets": total_tets, "mode": args.mode,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (arena %.0f MB)" % (
                       (total_tets * 112 + total_verts * 24 * 6) / 1e6)},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "newton_iters": {"mean": float(np.mean(newton)), "max": int(np.max(newton)), "total": int(iters_step)},
        "status_counts": status,
        "converged": n_conv,
        "capped_at_max_newton": sum(1 for r in results if r["status"] == idp.IDP_ERR_NOT_CONVERGED),
        "injective": injective,
        "fp64_one_at_a_time": fp64_single,
        "e2e": {"value": e2e_val, "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": None,  # the committed ncu capture covers k_pcg_grid on the blob only
                     "kernel": "k_pcg_cluster (block-Jacobi + contact-block PCG, one thread-block cluster per "
                               "instance)",
                     "peak_source": peak_kind},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "wall_ms_per_step": 1000 * statistics.mean(wall),
    }
    if fp64_single:
        ref = fp64_single["newton_iters_per_s"] if budget > 0 else fp64_single["solves_per_s"]
        out["mixed_batched_over_fp64_one_at_a_time"] = (value / ref) if ref else None
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(probs, args.cpu_sample_s, budget)
    print(json.dumps(out))


def fp64_one_at_a_time(idp, probs, results, sample, max_newton, budget, device, progress=None):
    """The plain FP64 path, one instance per context and call, on `sample`
    instances spread evenly over the batch (same start state and Newton
    budget as the batched mixed run); Newton iterations/s and solves/s from
    the library's device time, and the relative energy difference of the
    batched mixed results on the same instances."""
    import numpy as np

    nI = len(probs)
    idx = sorted(set(np.linspace(0, nI - 1, min(sample, nI)).round().astype(int).tolist()))
    ms = its = 0.0
    solved = 0
    rel = []
    for i in idx:
        p = probs[i]
        c = idp.Context(h=0.1, newton_tol=1e-3, max_newton=max_newton, mode=idp.MODE_FP64, device=device)
        c.add_instance(p["X"], p["tets"], p["mass"], p["lam"], p["mu"], p["dHat2"], p["kappa"], p["kappa_max"])
        c.set_velocity(0, (p["target"] - p["X"]) / 0.1)
        c.commit()
        c.save_state()
        c.advance(check=False)  # warm-up: grows the work buffers
        c.restore_state()
        _, r = c.advance(check=False)
        ms += c.stats()["total_ms"]
        its += r[0]["newton_iters"]
        solved += r[0]["status"] in (idp.IDP_OK, idp.IDP_WARN_ITER_CAP)  # converged solves only
        e64, em = r[0]["energy"], results[i]["energy"]
        rel.append(abs(em - e64) / max(abs(e64), 1e-300))
        c.close()
        if progress:
            progress(f"FP64 one at a time: instance {i} ({p['tets'].shape[0]} tets) {r[0]['newton_iters']} iterations, "
                     f"status {r[0]['status']}, rel energy vs mixed batched {rel[-1]:.2e}")
    out = {"instances": idx if len(idx) <= 32 else len(idx), "newton_iters": int(its), "ms": ms,
           "newton_iters_per_s": its / (ms / 1000.0) if ms > 0 else None,
           "solves_per_s": (solved / (ms / 1000.0)) if budget == 0 and ms > 0 else None,
           "converged": solved, "rel_energy_diff_mixed_batched": {"max": max(rel), "mean": float(np.mean(rel))}}
    return out


def serve_pool(seed=0, n_each=8, max_bar=50_000, max_blob=100_000):
    """Config-4 style job pool: n_each bars (tet counts log-uniform in [2k,
    max_bar], bend U[1.5pi, 2.5pi], the config-0 target) and n_each blobs (tet
    counts log-uniform in [2k, max_blob], one normal-flow step of 0.05)."""
    import numpy as np
    from idp_gb300 import meshgen
    from idp_gb300.api import initialize_oipc

    rng = np.random.default_rng(seed)
    pool = []
    for it in meshgen.bar_batch(n_each, 2_000, max_bar, seed=seed):
        pool.append(dict(kind="bar", X=it["X"], tets=it["tets"], v=(it["target"] - it["X"]) / 0.1, flow=0.0))
    for k in range(n_each):
        t = math.exp(rng.uniform(math.log(2_000), math.log(max_blob)))
        n = max(8, int(round((t / 0.84) ** (1.0 / 3.0))))
        X, tets, _ = meshgen.blob(n=n, lmax=8, amp=0.3, seed=seed * 100 + k)
        pool.append(dict(kind="blob", X=X, tets=tets, v=None, flow=0.05))
    for p in pool:
        X, tets = p["X"], p["tets"]
        p["mass"] = meshgen.lumped_mass(X, tets, 1000.0)
        p["lam"], p["mu"] = meshgen.lame(1e4, 0.3)
        diag = float(np.linalg.norm(X.max(0) - X.min(0)))
        p["dHat2"] = (1e-3 * diag) ** 2
        p["kappa"], p["kappa_max"] = initialize_oipc(float(p["mass"].mean()), p["dHat2"])
    return pool


def run_serve(args):
    """Served request stream (config 4, scaled): Poisson arrivals at --rate for
    --duration seconds, each a job drawn from serve_pool(); the continuous-
    batching server (idp_server_*) solves them in mixed precision. The
    reference point is the plain FP64 path one job at a time: every pool
    job's FP64 service time is measured once and the same arrival sequence is
    replayed through a single FIFO server."""
    import numpy as np
    import torch
    import idp_gb300 as idp

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pool = serve_pool(seed=rank, n_each=args.serve_pool, max_bar=args.serve_max_bar_tets,
                      max_blob=args.serve_max_blob_tets)
    rng = np.random.default_rng(1000 + rank)
    arr, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / args.rate)
        if t > args.duration:
            break
        arr.append((t, int(rng.integers(len(pool)))))
    params = dict(h=0.1, newton_tol=1e-3, max_newton=args.serve_newton_cap, device=local, **extra_params(args))
    # FP64 one at a time: service time of every pool job (wall time of one
    # context's add + commit + solve + read back, after a warm-up solve)
    svc, e64 = [], []
    for k, p in enumerate(pool):
        for rep in range(2 if k == 0 else 1):  # the first solve also warms the library up
            t0 = time.perf_counter()
            c = idp.Context(mode=idp.MODE_FP64, **params)
            c.add_instance(p["X"], p["tets"], p["mass"], p["lam"], p["mu"], p["dHat2"], p["kappa"], p["kappa_max"])
            if p["v"] is not None:
                c.set_velocity(0, p["v"])
            c.commit()
            if p["flow"]:
                c.set_normal_flow(0, p["flow"])
            _, r = c.advance(check=False)
            c.state(0)
            c.close()
            dt = time.perf_counter() - t0
        svc.append(dt)
        e64.append(r[0])
    t_free, lat64 = 0.0, []
    for ta, k in arr:
        start = max(ta, t_free)
        t_free = start + svc[k]
        lat64.append(t_free - ta)
    conv_ok = (idp.IDP_OK, idp.IDP_WARN_ITER_CAP)
    n_conv64 = sum(1 for _, k in arr if e64[k]["status"] in conv_ok)
    thr64 = n_conv64 / (t_free - arr[0][0]) if arr else 0.0
    # warm-up of the server's worker contexts on the pool, then the stream
    srv = idp.Server(args.hbm_budget_gb * 1e9, workers=args.serve_workers, max_batch=args.serve_batch,
                     mode=idp.MODE_MIXED, **params)

    def submit(p):
        return srv.submit(p["X"], p["tets"], p["mass"], p["lam"], p["mu"], p["dHat2"], p["kappa"], p["kappa_max"],
                          v=p["v"], normal_flow=p["flow"])

    for _ in range(max(1, args.warmup)):
        for jid in [submit(p) for p in pool]:
            srv.wait(jid)
    ids = []
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for ta, k in arr:
            d = ta - (time.perf_counter() - t0)
            if d > 0:
                time.sleep(d)
            ids.append((submit(pool[k]), k))
        srv.drain()
    infos = [(srv.wait(j)[0], k) for j, k in ids]
    st = srv.stats()
    srv.close()
    lat = [i["done_ms"] - i["submit_ms"] for i, _ in infos]
    span_s = (max(i["done_ms"] for i, _ in infos) - min(i["submit_ms"] for i, _ in infos)) / 1000.0
    # only jobs whose Newton loop met its stopping test count as solves; the
    # jobs stopped at the Newton cap are reported beside them
    n_conv = sum(1 for i, _ in infos if i["status"] in conv_ok)
    thr = n_conv / span_s
    status, rel = {}, []
    for i, k in infos:
        status[str(i["status"])] = status.get(str(i["status"]), 0) + 1
        r64 = e64[k]
        if i["status"] == idp.IDP_OK and r64["status"] == idp.IDP_OK:
            rel.append(abs(i["result"]["energy"] - r64["energy"]) / abs(r64["energy"]))
    if rank != 0:
        return
    kinds = {"bar": sum(1 for _, k in arr if pool[k]["kind"] == "bar"),
             "blob": sum(1 for _, k in arr if pool[k]["kind"] == "blob")}
    out = {
        "metric": METRIC + " (served request stream)", "value": thr, "unit": UNIT, "n_gpus": 1,
        "steps": len(infos), "warmup": args.warmup, "ms_per_step": 1000.0 / thr if thr else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"serve: Poisson arrivals {args.rate:g}/s for {args.duration:g} s, jobs drawn from "
                               f"{args.serve_pool} bars (2k-{args.serve_max_bar_tets // 1000}k tets, bend "
                               f"U[1.5pi,2.5pi]) and {args.serve_pool} blobs (2k-{args.serve_max_blob_tets // 1000}k "
                               f"tets, one normal-flow step 0.05), Newton cap {args.serve_newton_cap} per job",
                   "pool_tets": sorted(int(p["tets"].shape[0]) for p in pool),
                   "jobs": len(infos), "kinds": kinds, "workers": args.serve_workers, "max_batch": args.serve_batch,
                   "hbm_budget_gb": args.hbm_budget_gb, "l2": "no flush; jobs are independent solves"},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "status_counts": status,
        "converged": n_conv,
        "capped_at_max_newton": sum(1 for i, _ in infos if i["status"] == idp.IDP_ERR_NOT_CONVERGED),
        "server": st,
        "fp64_one_at_a_time": {"value": thr64, "unit": UNIT,
                               "latency_ms": {"p50": 1000 * float(np.percentile(lat64, 50)),
                                              "p99": 1000 * float(np.percentile(lat64, 99))},
                               "converged": n_conv64,
                               "basis": "FIFO replay of the same arrivals with each pool job's measured FP64 "
                                        "service time (one context per job); converged jobs per second"},
        "served_over_fp64_one_at_a_time": thr / thr64 if thr64 else None,
        "rel_energy_diff_vs_fp64": {"max": max(rel) if rel else None, "converged_jobs": len(rel)},
        "e2e": {"value": thr, "unit": UNIT,
                "h2d_bytes_per_step": float(np.mean([pool[k]["X"].size * 8 * 2 for _, k in arr])),
                "d2h_bytes_per_step": float(np.mean([pool[k]["X"].size * 8 * 2 for _, k in arr]))},
        "clocks": clocks.summary(),
    }
    print(json.dumps(out))


def run_anim(args):
    """Animation-fix sequence (config 2): a tet cylinder (radius 0.2, length
    3) follows keyframes bent by 2.4 pi sin(2 pi t/120) and twisted by
    pi cos(2 pi t/60); each keyframe is solved to the nearest injective
    configuration (x_tilde = keyframe, h = 0.1, i.e. the config-0 energy with
    weight 1e2 m), warm-started from the previous frame's result."""
    import numpy as np
    import torch
    import idp_gb300 as idp
    from idp_gb300 import meshgen
    from idp_gb300.api import initialize_oipc

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    X0, tets = meshgen.cylinder(n_cross=args.anim_n)
    mass = meshgen.lumped_mass(X0, tets, 1000.0)
    lam, mu = meshgen.lame(1e4, 0.3)
    diag = float(np.linalg.norm(X0.max(0) - X0.min(0)))
    dHat2 = (1e-3 * diag) ** 2
    k, km = initialize_oipc(float(mass.mean()), dHat2)
    mode = idp.MODE_MIXED if args.mode == "mixed" else idp.MODE_FP64
    ctx = idp.Context(h=0.1, newton_tol=1e-3, max_newton=args.max_newton, mode=mode, device=local)
    ctx.add_instance(X0, tets, mass, lam, mu, dHat2, k, km)
    ctx.commit()
    frames = [(args.frame_stride * f) % 120 for f in range(args.frames)]
    rows = []
    Xc = X0.copy()
    with ClockSampler(local) as clocks:
        for t in frames:
            tgt = meshgen.anim_keyframe(X0, t)
            t0 = time.perf_counter()
            ctx.set_velocity(0, (tgt - Xc) / 0.1)
            rc, res = ctx.advance(check=False)
            Xc, _, _ = ctx.state(0)
            wall = time.perf_counter() - t0
            st = ctx.stats()
            dev = np.linalg.norm(Xc - tgt, axis=1)
            rows.append(dict(frame=t, ms=st["total_ms"], wall_ms=1000 * wall, newton=res[0]["newton_iters"],
                             status=res[0]["status"], dev_max=float(dev.max()), dev_mean=float(dev.mean()),
                             penetrating_target=abs(math.sin(2 * math.pi * t / 120)) * 2.4 > 2.0,
                             launches=st["kernel_launches"]))
            print(f"frame {t}: {st['total_ms']:.1f} ms, {res[0]['newton_iters']} Newton, status "
                  f"{res[0]['status']}, deviation max {dev.max():.4f}", file=sys.stderr, flush=True)
    isect = int(ctx.intersection_counts()[0])
    if rank != 0:
        return
    ms = [r["ms"] for r in rows]
    status = {}
    for r in rows:
        status[str(r["status"])] = status.get(str(r["status"]), 0) + 1
    pen = [r for r in rows if r["penetrating_target"]]
    out = {
        "metric": "per-frame solve time and max/mean vertex deviation from the keyframe (animation-fix sequence)",
        "value": 1000.0 * len(rows) / sum(ms), "unit": "frames/s", "n_gpus": 1, "steps": len(rows), "warmup": 0,
        "ms_per_step": statistics.mean(ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if mode == idp.MODE_MIXED else "f64", "data": "synthetic",
        "config": {"workload": f"anim: tet cylinder r=0.2 L=3 ({tets.shape[0]} tets, {X0.shape[0]} verts), keyframes "
                               f"{frames[0]}..{frames[-1]} step {args.frame_stride}, bend 2.4pi sin(2pi t/120), twist "
                               f"pi cos(2pi t/60), warm-started, Newton cap {args.max_newton}",
                   "mode": args.mode, "l2": "inputs larger than L2; no flush"},
        "frame_ms": {"mean": statistics.mean(ms), "p50": float(np.percentile(ms, 50)),
                     "p99": float(np.percentile(ms, 99)), "max": max(ms)},
        "deviation": {"max": max(r["dev_max"] for r in rows), "mean": statistics.mean(r["dev_mean"] for r in rows),
                      "max_penetrating_frames": max((r["dev_max"] for r in pen), default=None)},
        "newton_iters": {"mean": statistics.mean(r["newton"] for r in rows), "max": max(r["newton"] for r in rows)},
        "penetrating_keyframes": len(pen), "status_counts": status,
        "final_state_intersections": isect,
        "gpu_launches": sum(r["launches"] for r in rows),
        "clocks": clocks.summary(),
        "frames": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()} for r in rows],
    }
    print(json.dumps(out))


def run_shellflow(args):
    """Flow mode on a triangle shell (Advance_One_Step_IE_Flow, as the reference's
    normal-flow scripts run it: dt 0.5, predictor x + 0.005 n per step, zero
    velocity): the surface of the bumpy blob (lmax 8, amplitude 0.3, seed 0)
    on a --shell-n grid as a closed shell (thickness 0.01, density 1000),
    d-hat 1e-3 of the bounding-box diagonal. W warm-up and K timed steps
    continue one flow sequence; the FP64 arm re-solves the timed steps from
    the same start states."""
    import numpy as np
    import torch
    import idp_gb300 as idp
    from idp_gb300 import meshgen
    from idp_gb300.api import initialize_oipc

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    Xb, Tb, _ = meshgen.blob(n=args.shell_n, lmax=8, amp=0.3, seed=rank)
    X, F = meshgen.shell_from_tets(Xb, Tb)
    h, step, thick, rho = 0.5, 0.005, 0.01, 1000.0
    diag = float(np.linalg.norm(X.max(0) - X.min(0)))
    dHat2 = (1e-3 * diag) ** 2
    # mean lumped mass (area * thickness * rho / 3 per corner) for kappa
    e1, e2 = X[F[:, 1]] - X[F[:, 0]], X[F[:, 2]] - X[F[:, 0]]
    area = np.linalg.norm(np.cross(e1, e2), axis=1) / 2
    k, km = initialize_oipc(float(area.sum() * thick * rho / X.shape[0]), dHat2)
    mode = idp.MODE_MIXED if args.mode == "mixed" else idp.MODE_FP64

    def make_ctx(m):
        c = idp.Context(h=h, newton_tol=1e-3, max_newton=args.max_newton, mode=m, device=local)
        c.add_shell_instance(X, F, rho, thick, dHat2, k, km)
        c.commit()
        return c

    ctx = make_ctx(mode)
    for _ in range(args.warmup):
        ctx.set_normal_flow(0, step)
        ctx.advance(check=False)
    starts, dev_ms, results = [], [], []
    launches = 0
    pcg_ms = pcg_bytes = 0.0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            starts.append(ctx.state(0))
            ctx.set_normal_flow(0, step)
            _, res = ctx.advance(check=False)
            st = ctx.stats()
            dev_ms.append(st["total_ms"])
            pcg_ms += st["pcg_ms"]
            pcg_bytes += st["pcg_bytes"]
            launches += st["kernel_launches"] + 1
            results.append(res[0])
    isect = int(ctx.intersection_counts()[0])
    value = args.steps / (sum(dev_ms) / 1000.0)
    cd = make_ctx(idp.MODE_FP64)
    d_ms, rel = [], []
    for j, (Xs, vs, ks) in enumerate(starts):
        cd.set_positions(0, Xs)
        cd.set_kappa(0, ks)
        cd.set_normal_flow(0, step)
        _, rd = cd.advance(check=False)
        d_ms.append(cd.stats()["total_ms"])
        rel.append(abs(results[j]["energy"] - rd[0]["energy"]) / max(abs(rd[0]["energy"]), 1e-300))
    cd.close()
    Xh = [torch.from_numpy(np.ascontiguousarray(Xs)).pin_memory() for Xs, _, _ in starts]
    Xo = torch.empty_like(Xh[0]).pin_memory()
    e2e = []
    for j, (Xs, vs, ks) in enumerate(starts):
        ctx.set_kappa(0, ks)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.set_positions_ptr(0, Xh[j].data_ptr())
        ctx.set_normal_flow(0, step)
        ctx.advance(check=False)
        ctx.state_ptr(0, Xo.data_ptr())
        e2e.append(time.perf_counter() - t0)
    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    achieved = (pcg_bytes / (pcg_ms / 1000.0) / 1e9) if pcg_ms > 0 else None
    newton = [r["newton_iters"] for r in results]
    out = {
        "metric": METRIC + " (shell flow mode)", "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(dev_ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mode == idp.MODE_MIXED else "f64", "data": "synthetic",
        "config": {"workload": f"shellflow: surface of the SH blob (lmax 8, amp 0.3) on a {args.shell_n}^3 grid as a "
                               f"closed shell ({X.shape[0]} verts, {F.shape[0]} faces), flow mode dt 0.5, predictor "
                               "x + 0.005 n per step, thickness 0.01, d-hat 1e-3 bbox diag",
                   "mode": args.mode, "l2": "working set fits in L2; no flush"},
        "newton_iters": {"mean": float(np.mean(newton)), "max": int(np.max(newton))},
        "constraints_last_step": int(results[-1]["num_constraints"]),
        "status": sorted({int(r["status"]) for r in results}),
        "fp64": {"solves_per_s": len(d_ms) / (sum(d_ms) / 1000.0), "rel_energy_err_max": max(rel),
                 "mixed_speedup": sum(d_ms) / sum(dev_ms)},
        "final_state_intersections": isect,
        "e2e": {"value": len(e2e) / sum(e2e), "unit": UNIT, "h2d_bytes_per_step": 3 * X.shape[0] * 8,
                "d2h_bytes_per_step": 3 * X.shape[0] * 8},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": None,
                     "kernel": "k_pcg_cluster", "peak_source": peak_kind},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    print(json.dumps(out))


def charseq_synthetic(n, count, folder):
    """A synthetic character sequence: the surface of the bumpy blob (lmax 8,
    amplitude 0.3, seed 0) on an n^3 grid, lifted to stand on y = 0, and
    frames 1..count written as OBJ files: frame k turns it by k degrees
    about the vertical axis, leans it by 0.5 k degrees about z and
    stretches it along y by 1 + 0.003 k."""
    import numpy as np
    from idp_gb300 import meshgen, meshio

    Xb, Tb, _ = meshgen.blob(n=n, lmax=8, amp=0.3, seed=0)
    X, F = meshgen.shell_from_tets(Xb, Tb)
    X = X - [0.0, X[:, 1].min(), 0.0]
    rest = os.path.join(folder, "rest.obj")
    meshio.write_tri_obj(rest, X, F)
    X, F, _ = meshio.read_tri_obj(rest)
    for k in range(1, count + 1):
        a, b = np.deg2rad(1.0 * k), np.deg2rad(0.5 * k)
        Ry = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
        Rz = np.array([[np.cos(b), -np.sin(b), 0], [np.sin(b), np.cos(b), 0], [0, 0, 1]])
        Y = X * [1.0, 1.0 + 0.003 * k, 1.0]
        meshio.write_tri_obj(os.path.join(folder, f"{k}.obj"), Y @ (Rz @ Ry).T, F)
    return rest


def oracle_charseq_frames(shell, F, frames, starts, h, budget_s):
    """The oracle (FP64, sparse Cholesky) solving frames of the character
    sequence from the GPU's start states: frame f's rest shape and DBC
    targets from frames[f], velocity (frame - x)/h, kappa from its masses;
    at least one frame, more while the time budget lasts."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from idp_gb300.api import initialize_oipc

    O.build()
    rows = shell["rows"]
    out, t_used = [], 0.0
    for Y, Xs in zip(frames, starts):
        area = np.linalg.norm(np.cross(Y[F[:, 1]] - Y[F[:, 0]], Y[F[:, 2]] - Y[F[:, 0]]), axis=1) / 2
        mass = np.zeros(Y.shape[0])
        np.add.at(mass, F.reshape(-1), np.repeat(area * shell["thickness"] * shell["density"] / 3, 3))
        k, km = initialize_oipc(float(mass.mean()), shell["dHat2"], 1.0)
        surf = O.shell_surface(Y.shape[0], F)
        hin, info = O.shell_hinges(Y, F, surf["edges"])
        mask = np.zeros(Y.shape[0], np.uint8)
        mask[rows] = 1
        pb = O.Problem(X=Xs.copy(), X0=Y, tets=np.zeros((0, 4), np.int32), mass=mass, lam=np.zeros(0),
                       mu=np.zeros(0), h=h, dHat2=shell["dHat2"], kappa=[k, km, 0.0], v=(Y - Xs) / h, faces=F,
                       mem=O.membrane_rest(Y, F, shell["thickness"], shell["E"], shell["nu"]), hinges=hin, hinfo=info,
                       kbend=O.hinge_stiffness(shell["E"], shell["nu"], shell["thickness"]), dbc=mask, tol=1e-3,
                       max_iters=500)
        pb.surf = surf
        pb.dbc_rows, pb.dbc_target = rows, Y[rows]
        t0 = time.perf_counter()
        it = O.advance_one_step(pb)
        t_used += time.perf_counter() - t0
        out.append(dict(energy=pb.last_energy, newton_iters=it, X=pb.X))
        if t_used >= budget_s:
            break
    return out, t_used


def run_charseq(args):
    """The character-sequence script (Projects/FEMShell/16_fix_char_seq.py)
    through the shell driver: the rest shell is loaded turned -90 degrees
    about x and lifted by 0.75 (add_shell_with_scale_3D), the vertices in
    the script's box (relative to the bounding box: [-0.1, 0.867, -0.1] to
    [1.1, 1.1, 1.1]) are DBC rows, dt 0.04, no gravity, density
    1000, E 100, nu 0.4, thickness 0.01, d-hat 1e-2; every step makes the
    next frame the rest shape, velocity target and DBC target (lv_fn). W
    warm-up and K timed frames; value = frames per second of device time
    of the Newton solves, e2e = frames per second of the whole driver step
    (frame OBJ read, context rebuild, uploads, solve, readback)."""
    import tempfile

    import numpy as np
    import torch
    import idp_gb300 as idp
    from idp_gb300 import meshio
    from idp_gb300.api import ShellFlowSim

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    tmp = tempfile.TemporaryDirectory()
    nframes = args.warmup + args.steps
    if args.charseq_mesh:
        mesh, folder, data = args.charseq_mesh, args.charseq_frames, "reference data files"
        xf = dict(translate=(0, 0.75, 0), rot=-90)
    else:
        folder, data = tmp.name, "synthetic"
        mesh = charseq_synthetic(args.charseq_n, nframes, folder)
        xf = dict(translate=(0, 0, 0), rot=0)
    mode = idp.MODE_MIXED if args.mode == "mixed" else idp.MODE_FP64
    h = 0.04
    sim = ShellFlowSim("double", 3, mode=mode)
    sim.add_shell_with_scale_3D(mesh, xf["translate"], (1, 1, 1), (0, 0, 0), (1, 0, 0), xf["rot"])
    sim.set_DBC((-0.1, 0.867, -0.1), (1.1, 1.1, 1.1), (0, 0, 0), (0, 0, 0), (1, 0, 0), 0)
    sim.dt = sim.frame_dt = h
    sim.gravity = (0.0, 0.0, 0.0)
    sim.initialize(1000, 100, 0.4, 0.01, 0)
    sim.initialize_OIPC(1e-2, 0, 1.0)
    sim.lv_fn, sim.seqDBCPath = 1, folder
    rows = sim.DBC.indices.copy()
    V, F = sim.X.shape[0], sim.Elem.copy()
    for _ in range(args.warmup):
        sim.advance_one_time_step(h)
    recs, starts, frames = [], [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            f = sim.lv_fn
            starts.append(sim.X.copy())
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            it = sim.advance_one_time_step(h)
            wall = time.perf_counter() - t0
            st = sim.context.stats()
            Y, _, _ = meshio.read_tri_obj(os.path.join(folder, f"{f}.obj"))
            frames.append(Y)
            recs.append(dict(frame=f, ms=st["total_ms"], wall_ms=1000 * wall, newton=it,
                             pcg=st["pcg_iters"], dbc_gap=float(np.abs(sim.X[rows] - Y[rows]).max()),
                             launches=st["kernel_launches"],
                             phases={k: st[k + "_ms"] for k in ("pcg", "tet", "contact", "ccd", "barrier", "assembly")}))
            print(f"frame {f}: {st['total_ms']:.1f} ms device, {1000 * wall:.1f} ms wall, {it} Newton",
                  file=sys.stderr, flush=True)
    isect = int(sim.context.intersection_counts()[0])
    if rank != 0:
        return
    ms = [r["ms"] for r in recs]
    wall = [r["wall_ms"] for r in recs]
    out = {
        "metric": "per-frame solve time of the character-sequence script (elastic shell, moving DBC rows)",
        "value": 1000.0 * len(recs) / sum(ms), "unit": "frames/s", "n_gpus": 1, "steps": len(recs),
        "warmup": args.warmup, "ms_per_step": statistics.mean(ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mode == idp.MODE_MIXED else "f64", "data": data,
        "config": {"workload": f"charseq: {os.path.basename(mesh)} ({V} verts, {F.shape[0]} faces, {rows.size} DBC "
                               f"rows), frames {recs[0]['frame']}..{recs[-1]['frame']} of "
                               f"{os.path.basename(os.path.normpath(folder)) if args.charseq_mesh else 'synthetic'}"
                               ", dt 0.04, E 100, nu 0.4, thickness 0.01, d-hat 1e-2, no gravity",
                   "mode": args.mode, "l2": "working set fits in L2; no flush"},
        "frame_ms": {"mean": statistics.mean(ms), "p50": float(np.percentile(ms, 50)),
                     "p99": float(np.percentile(ms, 99)), "max": max(ms)},
        "newton_iters": [r["newton"] for r in recs],
        "pcg_iters": [r["pcg"] for r in recs],
        "phase_ms_mean": {k: statistics.mean(r["phases"][k] for r in recs) for k in recs[0]["phases"]},
        "dbc_gap_max": max(r["dbc_gap"] for r in recs),
        "final_state_intersections": isect,
        "e2e": {"value": 1000.0 * len(recs) / sum(wall), "unit": "frames/s", "h2d_bytes_per_step": 3 * V * 8 * 3,
                "d2h_bytes_per_step": 3 * V * 8 * 2},
        "gpu_launches": sum(r["launches"] for r in recs),
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        shell = dict(rows=rows, thickness=0.01, density=1000.0, E=100.0, nu=0.4, dHat2=sim.dHat2)
        ores, t_or = oracle_charseq_frames(shell, F, frames, starts, h, args.cpu_sample_s)
        n = len(ores)
        out["cpu_baseline"] = {"value": n / t_or, "unit": "frames/s", "cores": cpu_cores(), "kind": "port",
                               "sample": f"oracle (FP64, sparse Cholesky) solving the first {n} timed frame(s) "
                                         "from the GPU's start states"}
        out["oracle_check"] = {"newton_iters": [o["newton_iters"] for o in ores],
                               "max_abs_x_diff": [float(np.abs(o["X"] - s).max()) for o, s in
                                                  zip(ores, [sim_x for sim_x in starts[1:] + [sim.X]])]}
    print(json.dumps(out))
    tmp.cleanup()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "shellflow":
        run_shellflow(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "anim":
        run_anim(args)
    elif args.workload == "charseq":
        run_charseq(args)
    elif args.workload == "blob":
        run_flow(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
