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


def test_bounded_steps_match_advance(gpu_lib):
    """idp_step_begin + idp_step_iterate in chunks of 3 Newton iterations gives
    idp_advance's results bit for bit, batch and all."""
    import idp_gb300 as idp

    pool = job_pool()
    sel = [1, 4, 2]

    def ctx_for():
        ctx = idp.Context(h=0.1, mode=idp.MODE_MIXED, max_newton=40)
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
        return ctx

    a = ctx_for()
    _, ra = a.advance(check=False)
    b = ctx_for()
    b.step_begin()
    chunks, left = 0, 1
    while left:
        _, left, rb = b.step_iterate(3)
        chunks += 1
    assert chunks > 2
    for i in range(len(sel)):
        assert ra[i]["newton_iters"] == rb[i]["newton_iters"] and ra[i]["energy"] == rb[i]["energy"]
        Xa, va, ka = a.state(i)
        Xb, vb, kb = b.state(i)
        assert np.array_equal(Xa, Xb) and np.array_equal(va, vb) and np.array_equal(ka, kb)
    a.close()
    b.close()


def test_job_joins_a_running_arena(gpu_lib):
    """One worker: a short flow job submitted while a long bar solve is
    iterating joins that worker's arena between Newton iterations, is released
    when it converges (well before the bar), and both results equal the
    results of solving each job alone."""
    import time

    import idp_gb300 as idp

    pool = job_pool()
    max_newton = 120
    bar, blob = pool[1], pool[5]
    alone_bar = solve_alone(idp, bar, max_newton)
    alone_blob = solve_alone(idp, blob, max_newton)
    assert alone_bar[0]["newton_iters"] > 3 * alone_blob[0]["newton_iters"]
    srv = idp.Server(hbm_budget=8e9, workers=1, max_batch=4, h=0.1, mode=idp.MODE_MIXED, max_newton=max_newton)
    pr = bar["pr"]
    jb = srv.submit(bar["X"], bar["tets"], pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"],
                    pr["kappa_max"], v=bar["v"])
    t0 = time.time()
    while srv.stats()["cohorts"] < 1 and time.time() - t0 < 30:
        time.sleep(0.005)
    time.sleep(0.2)
    pr = blob["pr"]
    jf = srv.submit(blob["X"], blob["tets"], pr["mass"], pr["lam"], pr["mu"], pr["dHat2"], pr["kappa"],
                    pr["kappa_max"], normal_flow=blob["flow"])
    info_f, Xf, vf = srv.wait(jf)
    info_b, Xb, vb = srv.wait(jb)
    assert info_b["admit_ms"] < info_f["admit_ms"] < info_b["done_ms"]
    assert info_f["cohort_size"] == 2  # admitted into the bar's running arena
    assert info_f["done_ms"] < info_b["done_ms"]
    for info, X, v, alone in ((info_b, Xb, vb, alone_bar), (info_f, Xf, vf, alone_blob)):
        r0, X0, v0, _ = alone
        assert info["status"] == r0["status"]
        assert info["result"]["newton_iters"] == r0["newton_iters"]
        assert info["result"]["energy"] == r0["energy"]
        assert np.array_equal(X, X0) and np.array_equal(v, v0)
    srv.close()
