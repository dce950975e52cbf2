"""Benchmark of the injective-deformation Newton step on GB300.

Default workload (the one the benchmark spec's target is quoted on): 256
independent bars, tet counts log-uniform in [1k, 50k], bend angles uniform in
[1.5pi, 2.5pi], jitter 0.05h, all in one device arena (BASELINE config 3).
A step is one implicit-Euler solve of every bar (Newton to convergence with
CCD-filtered line search): ``idp_advance``.

* value: solves/s with inputs resident in HBM (device snapshot restored
  device-to-device before each step); time = the library's CUDA-event time of
  idp_advance on its own stream.
* e2e: the same through the public API with host buffers: pinned positions
  and velocities uploaded, the step solved, positions read back, all inside
  the timed region (host wall clock around synchronous calls).
* roofline: the persistent PCG kernel (dominant), algorithmic bytes per
  launch / event time, against MEASURED_PEAKS.json hbm_gbs.
* cpu_baseline: the CPU oracle (FP64, scipy sparse LU) on a bounded sample,
  extrapolated to the batch by tet count.

``--impl reference`` times the reference's CPU path (here the oracle port,
because the reference does not build in this environment) on the same
metric, one bounded sample per step.
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
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batch256", choices=["batch256", "bar"])
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--max-newton", type=int, default=2000)
    ap.add_argument("--cpu-sample-s", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def cpu_baseline(probs, budget_s):
    """Oracle (FP64, direct solve) on a bounded sample: full solves of the
    smallest instances until the budget is spent; throughput extrapolated to
    the workload by tet count."""
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
                       v=(p["target"] - p["X"]) / 0.1, tol=1e-3, max_iters=2000)
        t0 = time.perf_counter()
        iters += O.advance_one_step(pb)
        t_used += time.perf_counter() - t0
        tets_done += T
        solved += 1
        if t_used >= budget_s:
            break
    mean_tets = sum(p["tets"].shape[0] for p in probs) / len(probs)
    rate = tets_done / t_used / mean_tets  # workload solves per second
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"oracle full solves of the {solved} smallest instance(s) ({tets_done} tets, {iters} Newton "
                      f"iterations, {t_used:.1f} s); solves/s scaled to the mean instance ({mean_tets:.0f} tets)"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    probs, desc = make_workload(args, seed=0)
    vals = []
    bl = None
    for _ in range(args.warmup + args.steps):
        bl = cpu_baseline(probs, args.cpu_sample_s)
        vals.append(bl["value"])
    v = statistics.mean(vals[args.warmup:]) if args.steps else vals[-1]
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v if v else None,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": desc, "instances": len(probs)},
           "cpu_baseline": dict(bl, value=v),
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    ctx = idp.Context(h=0.1, newton_tol=1e-3, max_newton=args.max_newton, mode=mode, device=local)
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

    # ---- resident inputs: restore the device snapshot, advance
    for _ in range(args.warmup):
        ctx.restore_state()
        ctx.advance(check=False)
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
    barrier()
    step_ms = statistics.mean(dev_ms)
    if world > 1:
        t = torch.tensor([step_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms = float(t.item())
    value = world * nI / (step_ms / 1000.0)

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
    e2e_s = statistics.mean(e2e_wall)
    if world > 1:
        t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_val = world * nI / e2e_s
    h2d = 2 * 3 * total_verts * 8
    d2h = 3 * total_verts * 8

    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    achieved = (pcg_bytes / (pcg_ms / 1000.0) / 1e9) if pcg_ms > 0 else None
    traffic = ncu_traffic()
    status = {}
    for r in results:
        status[str(r["status"])] = status.get(str(r["status"]), 0) + 1
    newton = [r["newton_iters"] for r in results]
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mode == idp.MODE_MIXED else "f64", "data": "synthetic",
        "config": {"workload": desc, "instances": nI, "total_tets": total_tets, "mode": args.mode,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (arena %.0f MB)" % (
                       (total_tets * 112 + total_verts * 24 * 6) / 1e6)},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "newton_iters": {"mean": float(np.mean(newton)), "max": int(np.max(newton))},
        "status_counts": status,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": traffic.get("bytes_per_launch") if traffic else None,
                     "kernel": "k_pcg_cta (persistent block-Jacobi PCG, one CTA per instance)",
                     "peak_source": peak_kind},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "wall_ms_per_step": 1000 * statistics.mean(wall),
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(probs, args.cpu_sample_s)
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
