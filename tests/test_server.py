"""Request server (idp_server_*): admission and scheduling on the CPU with the
simulated server (no device work), from several submitting threads."""
import threading

import numpy as np
import pytest


def _job(rng, V):
    X = rng.random((V, 3))
    tets = rng.integers(0, V, (max(1, V // 2), 4)).astype(np.int32)
    return X, tets


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g

    g.build()
    import idp_gb300

    return idp_gb300


def test_admission_fifo_budget_and_concurrency(lib):
    rng = np.random.default_rng(0)
    sizes = [int(v) for v in rng.integers(200, 20000, 40)]
    fp = [lib.job_footprint(V, max(1, V // 2)) for V in sizes]
    budget = 3.2 * max(fp)  # about three jobs resident at once
    srv = lib.Server(budget, workers=3, max_batch=4, simulated_ms_per_kvertex=0.5)
    ids, jobs = [], []
    for V in sizes:
        X, tets = _job(rng, V)
        jobs.append(X)
        ids.append(srv.submit(X, tets, np.ones(V), 1.0, 1.0, 1e-6, 1.0, 100.0))
    srv.drain()
    infos = []
    for jid, X in zip(ids, jobs):
        info, Xo, _ = srv.wait(jid)
        assert info["status"] == lib.IDP_OK
        assert np.array_equal(Xo, X)
        assert 1 <= info["cohort_size"] <= 4
        assert info["submit_ms"] <= info["admit_ms"] <= info["done_ms"]
        infos.append(info)
    # FIFO: admission times never decrease in submission order
    adm = [i["admit_ms"] for i in infos]
    assert all(a <= b for a, b in zip(adm, adm[1:]))
    st = srv.stats()
    assert st["submitted"] == st["completed"] == len(sizes)
    assert st["peak_resident"] <= budget
    assert st["peak_device"] <= budget
    assert 2 <= st["peak_concurrency"] <= 3
    # jobs admitted together share their admission time; each completes on
    # its own
    by = {}
    for i in infos:
        by.setdefault(i["cohort"], []).append(i)
    assert len(by) == st["cohorts"]
    for members in by.values():
        assert len({m["admit_ms"] for m in members}) == 1
    srv.close()


def test_oversized_job_is_rejected(lib):
    srv = lib.Server(lib.job_footprint(1000, 500) * 1.5, workers=1, max_batch=2, simulated_ms_per_kvertex=0.0)
    rng = np.random.default_rng(1)
    X, tets = _job(rng, 100000)
    with pytest.raises(lib.IDPError) as e:
        srv.submit(X, tets, np.ones(100000), 1.0, 1.0, 1e-6, 1.0, 100.0)
    assert e.value.code == lib.IDP_ERR_CAPACITY
    X, tets = _job(rng, 1000)
    jid = srv.submit(X, tets, np.ones(1000), 1.0, 1.0, 1e-6, 1.0, 100.0)
    info, _, _ = srv.wait(jid)
    assert info["status"] == lib.IDP_OK
    srv.close()


def test_jobs_arriving_while_others_run(lib):
    """Arrivals from several threads while cohorts are running are admitted
    by the next free worker without waiting for the running cohorts."""
    rng = np.random.default_rng(2)
    budget = 10 * lib.job_footprint(2000, 1000)
    srv = lib.Server(budget, workers=2, max_batch=3, simulated_ms_per_kvertex=20.0)
    # a long job occupies one worker
    Xl, tl = _job(rng, 20000)
    long_id = srv.submit(Xl, tl, np.ones(20000), 1.0, 1.0, 1e-6, 1.0, 100.0)  # ~400 ms
    out, lock = [], threading.Lock()

    def client(seed):
        r = np.random.default_rng(seed)
        for _ in range(3):
            X, t = _job(r, 500)
            jid = srv.submit(X, t, np.ones(500), 1.0, 1.0, 1e-6, 1.0, 100.0)
            with lock:
                out.append(jid)

    th = [threading.Thread(target=client, args=(s,)) for s in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    infos = [srv.wait(j)[0] for j in out]
    long_info = srv.wait(long_id)[0]
    # the short jobs finished while the long cohort was still running
    assert max(i["done_ms"] for i in infos) < long_info["done_ms"]
    assert all(i["status"] == lib.IDP_OK for i in infos)
    assert srv.stats()["peak_concurrency"] == 2
    srv.close()


def test_job_joins_a_running_arena_and_leaves_first(lib):
    """A short job submitted while a long one is iterating on the only worker
    joins its arena between Newton iterations and is released as soon as it
    finishes, long before the long job."""
    import time

    rng = np.random.default_rng(3)
    srv = lib.Server(10 * lib.job_footprint(20000, 10000), workers=1, max_batch=4, simulated_ms_per_kvertex=10.0)
    Xl, tl = _job(rng, 20000)  # 22 simulated iterations of ~20 ms
    long_id = srv.submit(Xl, tl, np.ones(20000), 1.0, 1.0, 1e-6, 1.0, 100.0)
    t0 = time.time()
    while srv.stats()["cohorts"] < 1 and time.time() - t0 < 10:  # the long job is iterating
        time.sleep(0.005)
    time.sleep(0.03)
    Xs, ts = _job(rng, 500)  # 2 iterations
    short_id = srv.submit(Xs, ts, np.ones(500), 1.0, 1.0, 1e-6, 1.0, 100.0)
    short, _, _ = srv.wait(short_id)
    long_, _, _ = srv.wait(long_id)
    assert short["status"] == long_["status"] == lib.IDP_OK
    assert short["admit_ms"] < long_["done_ms"] and long_["admit_ms"] < short["admit_ms"]
    assert short["cohort_size"] == 2  # it ran in the long job's arena
    assert short["done_ms"] < long_["done_ms"] - 100.0
    assert short["result"]["newton_iters"] == 2 and long_["result"]["newton_iters"] == 22
    srv.close()


def test_idle_contexts_count_against_the_budget(lib):
    """An idle worker's context keeps its device memory; admission counts it,
    and idle workers give it back when the head job needs it, so the memory
    in use never exceeds the budget."""
    rng = np.random.default_rng(4)
    V = 20000
    fp = lib.job_footprint(V, V // 2)
    srv = lib.Server(1.5 * fp, workers=2, max_batch=2, simulated_ms_per_kvertex=1.0)
    ids = []
    for _ in range(6):
        X, t = _job(rng, V)
        ids.append(srv.submit(X, t, np.ones(V), 1.0, 1.0, 1e-6, 1.0, 100.0))
    infos = [srv.wait(j)[0] for j in ids]
    assert all(i["status"] == lib.IDP_OK for i in infos)
    st = srv.stats()
    assert st["peak_device"] <= 1.5 * fp
    assert st["peak_concurrency"] == 1  # two big jobs never fit at once
    # one at a time: each job is admitted only after the previous one is done
    order = sorted(infos, key=lambda i: i["admit_ms"])
    assert all(a["done_ms"] <= b["admit_ms"] for a, b in zip(order, order[1:]))
    srv.close()
