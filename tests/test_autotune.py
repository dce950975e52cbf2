"""The autotuner's search and cache, with a stand-in timing function (the
GPU timing itself runs in the GPU tests and the bench)."""
import numpy as np

from idp_gb300 import autotune


def fake_instances(n=3, V=5000):
    return [dict(X=np.zeros((V + 100 * k, 3)), tets=np.zeros((4 * V, 4), np.int32)) for k in range(n)]


def test_coordinate_search_finds_the_fastest_and_caches(tmp_path):
    calls = []

    def measure(inst, params):
        calls.append(params)
        # fastest at cta 80, degree 4; other coordinates indifferent
        return 10.0 + abs(params["pcg_grid_cta_vertices"] - 80) / 10 + (4 - params["pcg_local_degree"]) * 0.5

    cache = tmp_path / "tune.json"
    p, rec = autotune.tune(fake_instances(), base={"mode": 1}, cache_path=str(cache), device_name="GB300",
                           measure=measure)
    assert p["pcg_grid_cta_vertices"] == 80 and p["pcg_local_degree"] == 4 and p["mode"] == 1
    assert not rec["cached"] and rec["ms"] == 10.0
    n = len(calls)
    assert n == 1 + sum(len(v) - 1 for v in autotune.DEFAULT_SPACE.values())
    # the same kind of workload reads the cache; a different one tunes again
    p2, rec2 = autotune.tune(fake_instances(), base={"mode": 1}, cache_path=str(cache), device_name="GB300",
                             measure=measure)
    assert rec2["cached"] and p2 == p and len(calls) == n
    autotune.tune(fake_instances(n=40), base={"mode": 1}, cache_path=str(cache), device_name="GB300",
                  measure=measure)
    assert len(calls) > n


def test_signature_buckets_sizes():
    a = autotune.signature(fake_instances(V=5000), 1, "GB300")
    b = autotune.signature(fake_instances(V=5100), 1, "GB300")
    c = autotune.signature(fake_instances(V=20000), 1, "GB300")
    assert a == b and a != c and a != autotune.signature(fake_instances(V=5000), 0, "GB300")
