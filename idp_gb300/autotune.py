"""Autotuner for the solver's block and tile shapes.

The tunables are `idp_params` fields that shape the kernels without changing
what is computed beyond rounding:

* ``pcg_grid_cta_vertices`` -- rows (vertices) per CTA of the grid-wide PCG,
  i.e. the tile each CTA stages in shared memory;
* ``pcg_local_degree`` -- degree of the grid PCG's CTA-local polynomial
  preconditioner (0, 2, 4);
* ``pcg_grid_min_vertices`` -- the instance size above which the grid-wide
  PCG (all SMs) replaces one thread-block cluster per instance;
* ``contact_block_vertices`` -- the largest group of contact-coupled vertices
  inverted as one dense block.

``tune`` times one Newton step of the caller's workload (from the same start
state every time, after a warm-up step that grows the work buffers) for each
candidate and keeps the fastest, coordinate by coordinate starting from the
library defaults. Results are cached on disk per workload signature (GPU
name, precision mode, instance count and size buckets), so a later run of
the same kind of workload reads them instead of tuning again.
"""
from __future__ import annotations

import json
import math
import os

DEFAULT_SPACE = {
    "pcg_grid_cta_vertices": [112, 80, 144],
    "pcg_local_degree": [0, 2, 4],
    "pcg_grid_min_vertices": [16384, 8192, 32768],
    "contact_block_vertices": [192, 96],
}


def _bucket(n):
    return int(round(math.log2(max(1, n)) * 2)) / 2.0  # half-octave buckets


def signature(instances, mode, device_name):
    """Workload key: device, mode, instance count and size buckets."""
    V = sorted(int(p["X"].shape[0]) for p in instances)
    T = sum(int(p["tets"].shape[0]) for p in instances)
    return json.dumps({"device": device_name, "mode": int(mode), "instances": len(V),
                       "v_max": _bucket(V[-1]), "v_median": _bucket(V[len(V) // 2]), "tets": _bucket(T)},
                      sort_keys=True)


def default_cache_path():
    return os.path.join(os.path.expanduser("~"), ".cache", "idp_gb300", "autotune.json")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def step_time_ms(instances, params, device=0):
    """Device time (ms) of one Newton step of every instance with `params`,
    measured from the same start state after one warm-up step (an instance's
    "normal_flow" entry sets the normal-flow predictor before each step)."""
    import idp_gb300 as idp

    params = dict(params)
    ctx = idp.Context(device=params.pop("device", device), **params)
    try:
        for i, p in enumerate(instances):
            ctx.add_instance(p["X"], p["tets"], p["mass"], p["lam"], p["mu"], p["dHat2"], p["kappa"],
                             p["kappa_max"])
            if p.get("v") is not None:
                ctx.set_velocity(i, p["v"])
        ctx.commit()
        ctx.save_state()

        def predictor():
            for i, p in enumerate(instances):
                if p.get("normal_flow"):
                    ctx.set_normal_flow(i, p["normal_flow"])

        predictor()
        ctx.advance(check=False)
        ctx.restore_state()
        predictor()
        ctx.advance(check=False)
        return float(ctx.stats()["total_ms"])
    finally:
        ctx.close()


def tune(instances, base=None, space=None, cache_path=None, device_name=None, measure=None, log=None):
    """The fastest parameter set for `instances` (list of dicts with X, tets,
    mass, lam, mu, dHat2, kappa, kappa_max and optionally v) starting from
    `base` (e.g. {"mode": ..., "h": ..., "newton_tol": ...}); one coordinate
    at a time over `space`. Returns (params, record) where record holds every
    timing. `measure(instances, params) -> ms` replaces the GPU timing (tests)."""
    base = dict(base or {})
    space = DEFAULT_SPACE if space is None else space
    measure = measure or step_time_ms
    if device_name is None:
        try:
            import torch

            device_name = torch.cuda.get_device_name(base.get("device", 0))
        except Exception:
            device_name = "unknown"
    key = signature(instances, base.get("mode", 1), device_name)
    path = cache_path or default_cache_path()
    cache = _load(path) if path else {}
    if key in cache:
        hit = cache[key]
        return dict(base, **hit["params"]), dict(hit, cached=True)
    best = {k: v[0] for k, v in space.items()}
    timings = {}

    def run(p):
        tag = json.dumps(p, sort_keys=True)
        if tag not in timings:
            timings[tag] = measure(instances, dict(base, **p))
            if log:
                log(f"autotune {tag}: {timings[tag]:.3f} ms")
        return timings[tag]

    best_ms = run(best)
    for name, values in space.items():
        for v in values[1:]:
            cand = dict(best, **{name: v})
            ms = run(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    record = {"params": best, "ms": best_ms, "timings": timings, "key": key}
    if path:
        cache[key] = record
        _store(path, cache)
    return dict(base, **best), dict(record, cached=False)
