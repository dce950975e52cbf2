"""Exact intersection check (Check_Edge_Tri_Intersect / segTriIntersect,
FEM/IPC.h:2390-2517) on the CPU.

Three implementations are compared on the same inputs:
  * exact rational arithmetic in Python (fractions): orient3d as a determinant
    and the reference's own segTriIntersect formula (plane sides, then the
    (u, v, t) solve with inclusive bounds) evaluated without rounding;
  * the oracle's restatement (oracle/idp_oracle.cpp);
  * the product's predicate header (idp_gb300/csrc/predicates.cuh), compiled
    for the host with the same no-contraction rule the device build uses.
Near-degenerate inputs (points on planes, segments through vertices and
edges) are built from dyadic coordinates so the degeneracies are exact.
"""
import os
import subprocess
from fractions import Fraction as Fr

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "idp_gb300", "csrc")

SHIM = r"""
#include "predicates.cuh"
extern "C" int p_orient(const double* a, const double* b, const double* c, const double* d) {
    return idp::pred::orient3d_sign(a, b, c, d);
}
extern "C" int p_orient_exact(const double* a, const double* b, const double* c, const double* d) {
    return idp::pred::orient3d_exact(a, b, c, d);
}
extern "C" int p_segtri(const double* e0, const double* e1, const double* t0, const double* t1, const double* t2) {
    return idp::pred::seg_tri_intersect(e0, e1, t0, t1, t2) ? 1 : 0;
}
"""


@pytest.fixture(scope="module")
def pred(tmp_path_factory):
    import ctypes as C

    d = tmp_path_factory.mktemp("pred")
    src, so = d / "shim.cpp", d / "libpred.so"
    src.write_text(SHIM)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", CSRC, str(src), "-o",
                    str(so)], check=True)
    L = C.CDLL(str(so))
    dp = C.POINTER(C.c_double)
    for f in ("p_orient", "p_orient_exact"):
        getattr(L, f).argtypes = [dp] * 4
    L.p_segtri.argtypes = [dp] * 5
    return L


def _p(a):
    import ctypes as C

    a = np.ascontiguousarray(a, np.float64)
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fr_orient(a, b, c, d):
    m = [[Fr(float(x)) - Fr(float(y)) for x, y in zip(p, d)] for p in (a, b, c)]
    det = (m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]))
    return (det > 0) - (det < 0)


def fr_segtri_reference(e0, e1, t0, t1, t2):
    """segTriIntersect (FEM/IPC.h:2390-2442) in exact arithmetic: coplanar
    endpoint or same side -> False; else solve [t1-t0, t2-t0, e0-e1] (u,v,t)
    = e0 - t0 and test u, v >= 0, u + v <= 1, 0 <= t <= 1."""
    o0, o1 = fr_orient(t0, t1, t2, e0), fr_orient(t0, t1, t2, e1)
    if o0 == 0 or o1 == 0 or o0 == o1:
        return False
    F = lambda v: [Fr(float(x)) for x in v]
    T0, T1, T2, E0, E1 = F(t0), F(t1), F(t2), F(e0), F(e1)
    cols = [[T1[k] - T0[k] for k in range(3)], [T2[k] - T0[k] for k in range(3)], [E0[k] - E1[k] for k in range(3)]]
    rhs = [E0[k] - T0[k] for k in range(3)]

    def det3(c0, c1, c2):
        return (c0[0] * (c1[1] * c2[2] - c1[2] * c2[1]) - c1[0] * (c0[1] * c2[2] - c0[2] * c2[1]) +
                c2[0] * (c0[1] * c1[2] - c0[2] * c1[1]))

    D = det3(*cols)
    if D == 0:
        return False
    u = det3(rhs, cols[1], cols[2]) / D
    v = det3(cols[0], rhs, cols[2]) / D
    t = det3(cols[0], cols[1], rhs) / D
    return u >= 0 and v >= 0 and u + v <= 1 and 0 <= t <= 1


def near_coplanar_cases(rng, n):
    out = []
    for k in range(n):
        a, b, c = rng.random((3, 3))
        t, u = rng.random(2)
        d = a + t * (b - a) + u * (c - a)  # on the plane up to rounding
        if k % 3 == 1:
            d = d + rng.normal(size=3) * 1e-16
        if k % 3 == 2:  # exactly coplanar dyadic points
            a, b, c = rng.integers(-8, 8, (3, 3)) / 8.0
            d = a + (b - a) * (rng.integers(0, 8) / 8.0) + (c - a) * (rng.integers(0, 8) / 8.0)
        out.append((a, b, c, d))
    return out


def test_orient3d_matches_rationals(oracle, pred):
    rng = np.random.default_rng(11)
    for a, b, c, d in near_coplanar_cases(rng, 1500):
        want = fr_orient(a, b, c, d)
        assert oracle.orient3d(a, b, c, d) == want
        assert pred.p_orient(_p(a), _p(b), _p(c), _p(d)) == want
        assert pred.p_orient_exact(_p(a), _p(b), _p(c), _p(d)) == want


def test_orient3d_large_spread_of_magnitudes(oracle, pred):
    rng = np.random.default_rng(5)
    for _ in range(300):
        s = 10.0 ** rng.uniform(-40, 40, size=(4, 1))
        a, b, c, d = rng.normal(size=(4, 3)) * s
        d2 = a + 0.25 * (b - a) + 0.5 * (c - a)
        for q in (d, d2):
            want = fr_orient(a, b, c, q)
            assert oracle.orient3d(a, b, c, q) == want
            assert pred.p_orient(_p(a), _p(b), _p(c), _p(q)) == want


def segtri_cases(rng, n):
    t0, t1, t2 = np.array([0.0, 0, 0]), np.array([1.0, 0, 0]), np.array([0.0, 1, 0])
    fixed = [
        # through the interior, through a vertex, through an edge midpoint, outside
        (np.array([0.25, 0.25, -1.0]), np.array([0.25, 0.25, 1.0])),
        (np.array([0.0, 0.0, -1.0]), np.array([0.0, 0.0, 1.0])),
        (np.array([0.5, 0.5, -1.0]), np.array([0.5, 0.5, 1.0])),
        (np.array([0.5, 0.0, -0.5]), np.array([0.5, 0.0, 0.25])),
        (np.array([0.75, 0.75, -1.0]), np.array([0.75, 0.75, 1.0])),
        # endpoint on the plane (coplanar contact: not an intersection)
        (np.array([0.25, 0.25, 0.0]), np.array([0.25, 0.25, 1.0])),
        # same side, in the plane, degenerate segment
        (np.array([0.25, 0.25, 0.5]), np.array([0.25, 0.25, 1.0])),
        (np.array([-1.0, 0.5, 0.0]), np.array([2.0, 0.5, 0.0])),
        (np.array([0.25, 0.25, -1.0]), np.array([0.25, 0.25, -1.0])),
    ]
    out = [(e0, e1, t0, t1, t2) for e0, e1 in fixed]
    for k in range(n):
        T = rng.integers(-8, 9, (3, 3)) / 4.0
        if k % 2 == 0:  # aim at a dyadic point of the triangle (often its boundary)
            w = rng.integers(0, 5, 3).astype(float)
            w = w / w.sum() if w.sum() > 0 else np.array([1.0, 0, 0])
            p = w @ T
            dirn = rng.integers(-4, 5, 3) / 4.0
            e0, e1 = p - dirn, p + dirn * (rng.integers(1, 4) / 2.0)
        else:
            e0, e1 = rng.integers(-8, 9, (2, 3)) / 4.0
        out.append((e0, e1, T[0], T[1], T[2]))
    return out


def test_segment_triangle_matches_reference_formula(oracle, pred):
    rng = np.random.default_rng(3)
    for e0, e1, t0, t1, t2 in segtri_cases(rng, 2000):
        want = fr_segtri_reference(e0, e1, t0, t1, t2)
        got = pred.p_segtri(_p(e0), _p(e1), _p(t0), _p(t1), _p(t2))
        assert bool(got) == want, (e0, e1, t0, t1, t2)
    # the oracle's mesh-level entry on one triangle and many edges
    cases = segtri_cases(np.random.default_rng(4), 400)
    for e0, e1, t0, t1, t2 in cases:
        X = np.array([t0, t1, t2, e0, e1])
        surf = {"tris": np.array([[0, 1, 2]], np.int32), "edges": np.array([[3, 4]], np.int32)}
        pairs = oracle.edge_tri_intersections(X, surf)
        assert (len(pairs) == 1) == fr_segtri_reference(e0, e1, t0, t1, t2)


def _two_bars(offset):
    from idp_gb300 import meshgen

    X1, T1 = meshgen.bar(2, 2, 4, size=(1.0, 1.0, 2.0), seed=0)
    X2, T2 = meshgen.bar(2, 2, 4, size=(1.0, 1.0, 2.0), seed=1)
    X = np.vstack([X1, X2 + np.asarray(offset)])
    return X, np.vstack([T1, T2 + X1.shape[0]])


def test_mesh_intersections(oracle):
    from idp_gb300 import meshgen

    # rest bar: intersection-free
    X, tets = meshgen.bar(3, 3, 8, size=(1.0, 1.0, 4.0), seed=0)
    surf = oracle.surface(X, tets)
    assert len(oracle.edge_tri_intersections(X, surf)) == 0
    # its self-intersecting bend target: intersecting
    Xt = meshgen.bend_target(X, angle=2.2 * np.pi)
    assert len(oracle.edge_tri_intersections(Xt, surf)) > 0
    # two bars apart / overlapping
    Xa, ta = _two_bars((3.0, 0.0, 0.0))
    sa = oracle.surface(Xa, ta)
    assert len(oracle.edge_tri_intersections(Xa, sa)) == 0
    Xb, tb = _two_bars((0.4, 0.3, 0.5))
    sb = oracle.surface(Xb, tb)
    pairs = oracle.edge_tri_intersections(Xb, sb)
    assert len(pairs) > 0
    # every reported pair really intersects (exact rationals), none shares a vertex
    for f, e in pairs[:200]:
        t = sb["tris"][f]
        a, b = sb["edges"][e]
        assert not set(t) & {a, b}
        assert fr_segtri_reference(Xb[a], Xb[b], Xb[t[0]], Xb[t[1]], Xb[t[2]])
    # all-DBC pairs are excluded
    dbc = np.ones(Xb.shape[0], np.uint8)
    assert len(oracle.edge_tri_intersections(Xb, sb, dbc)) == 0
