"""Request server on the GB300 (idp_server_*): every job's result is the same
bit for bit whether it is solved alone or admitted into a running mix of
cohorts on concurrent workers; the admission footprint bounds the device
memory a job's context actually holds; a context reused through idp_reset
gives the same results as a fresh one."""
import math
import threading

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def job_pool():
    from idp_gb300 import meshgen

    jobs = []
    for k, (n, ang) in enumerate([((2, 2, 6), 1.2), ((3, 3, 8), 2.2), ((2, 3, 7), 1.6), ((3, 3, 6), 0.8)]):
        X, tets = meshgen.bar(*n, size=(1.0, 1.0, 2.0), seed=k)
        tgt = meshgen.bend_target(X, angle=ang * math.pi, radius=0.45, size=(1.0, 1.0, 2.0))
        jobs.append(dict(X=X, tets=tets, pr=cases.problem(X, tets), v=(tgt - X) / 0.1, flow=0.0))
    for k, n in enumerate([10, 12, 14]):
        X, tets, _ = meshgen.blob(n=n, lmax=4, seed=k)
        jobs.append(dict(X=X, tets=tets, pr=cases.problem(X, tets), v=None, flow=0.05))
    return jobs


def solve_alone(idp, j, max_newton):
    ctx = idp.Context(h=0.1, mode=idp.MODE_MIXED, max_newton=max_newton)
    pr = j["pr"]
    ctx.add_instance(j["X"], j["tets"], pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"], pr["kappa_max"])
    if j["v"] is not None:
        ctx.set_velocity(0, j["v"])
    ctx.commit()
    if j["flow"]:
        ctx.set_normal_flow(0, j["flow"])
    rc, res = ctx.advance(check=False)
    X, v, _ = ctx.state(0)
    nbytes = ctx.device_bytes()
    ctx.close()
    return res[0], X, v, nbytes


def test_results_same_alone_and_in_the_mix(gpu_lib):
    import idp_gb300 as idp

    pool = job_pool()
    max_newton = 40
    alone = [solve_alone(idp, j, max_newton) for j in pool]
    # the admission estimate covers what a one-job context holds
    for j, a in zip(pool, alone):
        fp = idp.job_footprint(j["X"].shape[0], j["tets"].shape[0])
        assert a[3] <= fp, (a[3], fp)
    srv = idp.Server(hbm_budget=8e9, workers=3, max_batch=3, h=0.1, mode=idp.MODE_MIXED, max_newton=max_newton)
    order = [k % len(pool) for k in range(3 * len(pool))]
    rng = np.random.default_rng(0)
    rng.shuffle(order)
    ids, lock = {}, threading.Lock()

    def client(part):
        for k in part:
            j = pool[k]
            pr = j["pr"]
            jid = srv.submit(j["X"], j["tets"], pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"],
                             pr["kappa_max"], v=j["v"], normal_flow=j["flow"])
            with lock:
                ids[jid] = k

    th = [threading.Thread(target=client, args=(order[i::3],)) for i in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    srv.drain()
    sizes = set()
    for jid, k in ids.items():
        info, X, v = srv.wait(jid)
        r0, X0, v0, _ = alone[k]
        sizes.add(info["cohort_size"])
        assert info["status"] == r0["status"]
        assert info["result"]["newton_iters"] == r0["newton_iters"]
        assert info["result"]["energy"] == r0["energy"]
        assert np.array_equal(X, X0) and np.array_equal(v, v0), k
    st = srv.stats()
    assert st["completed"] == len(order)
    assert st["peak_concurrency"] >= 2
    assert max(sizes) > 1  # some jobs really shared a cohort
    srv.close()


def test_reset_context_matches_fresh(gpu_lib):
    import idp_gb300 as idp

    pool = job_pool()
    ctx = idp.Context(h=0.1, mode=idp.MODE_MIXED, max_newton=40)
    for sel in ([0, 4], [1, 2, 5], [6], [3, 4]):
        for i, k in enumerate(sel):
            j = pool[k]
            pr = j["pr"]
            ctx.add_instance(j["X"], j["tets"], pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"],
                             pr["kappa_max"])
            if j["v"] is not None:
                ctx.set_velocity(i, j["v"])
        ctx.commit()
        for i, k in enumerate(sel):
            if pool[k]["flow"]:
                ctx.set_normal_flow(i, pool[k]["flow"])
        rc, res = ctx.advance(check=False)
        for i, k in enumerate(sel):
            r0, X0, _, _ = solve_alone(idp, pool[k], 40)
            X, _, _ = ctx.state(i)
            assert res[i]["energy"] == r0["energy"] and np.array_equal(X, X0), (sel, k)
        ctx.reset()
    ctx.close()
