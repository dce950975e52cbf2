"""Surface extraction on the device (idp_add_instance for meshes of at least
surface_device_min_tets tets): the same triangles, edges and nodes, in the
same order, as the host extraction and the oracle's restatement of
Find_Surface_TriMesh / Find_Surface_Primitives (Utils/MESHIO.h:485-544,
768-834)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def meshes():
    import bench
    from idp_gb300 import meshgen

    out = {"one tet": (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]]), np.array([[0, 1, 2, 3]], np.int32))}
    out["bar"] = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 2.6), seed=0)
    out["two bars"] = cases.two_bars(gap=2e-3, seed=0)
    p = bench.blob_problem(24)
    out["blob 24"] = (p["X"], p["tets"])
    # reversed vertex numbering: the order of the lists follows the ids
    X, t = meshgen.bar(2, 2, 5, size=(1.0, 1.0, 2.0), seed=1)
    perm = np.arange(X.shape[0])[::-1]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    out["bar, reversed ids"] = (X[perm], inv[t].astype(np.int32))
    return out


def test_device_surface_matches_host_and_oracle(oracle, gpu_lib):
    import idp_gb300 as idp

    for name, (X, tets) in meshes().items():
        m = np.ones(X.shape[0])
        got = []
        for dev_min in (1, -1):  # device, host
            ctx = idp.Context(surface_device_min_tets=dev_min)
            ctx.add_instance(X, tets, m, 1.0, 1.0, 1e-6, 1.0, 10.0)
            got.append(ctx.surface(0))
            ctx.close()
        o = oracle.surface(X, tets)
        for k in ("tris", "edges", "nodes"):
            assert np.array_equal(got[0][k], got[1][k]), (name, k)
            assert np.array_equal(got[0][k], o[k]), (name, k)
