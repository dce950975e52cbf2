"""The point-triangle distance-type classifier's 2x2 solve.

The reference solves the classifier's normal equations with Eigen's LDLT
(``Math/Distance/DISTANCE_TYPE.h:46,54,62``): diagonal pivoting, then
D0 = m00, l = m10 / D0, D1 = m11 - l * (D0 * l). This file restates that
solve once more in plain Python floats (every operation rounded on its own,
as the oracle's -ffp-contract=off build does) and checks the oracle against
it bit for bit, on random triangles, on points next to the classifier's
decision boundaries (s = 0, s = 1, t = 0) and on triangles large enough that
the pivot swaps the equations (|n| > 1). Away from those boundaries the
classification must also agree with exact rational arithmetic.
"""
from fractions import Fraction

import numpy as np
import pytest

TINY = 2.2250738585072014e-308


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def eigen_ldlt_solve2(a00, a01, a11, b0, b1):
    """Eigen's LDLT of a symmetric 2x2 and its solve, one rounded operation
    at a time (returns x0, x1, pivoted)."""
    piv = abs(a11) > abs(a00)
    m00, m11 = (a11, a00) if piv else (a00, a11)
    y0, y1 = (b1, b0) if piv else (b0, b1)
    d0 = m00
    lo = a01 / d0 if abs(d0) > 0.0 else a01
    d1 = m11 - lo * (d0 * lo)
    y1 = y1 - lo * y0
    y0 = y0 / d0 if abs(d0) > TINY else 0.0
    y1 = y1 / d1 if abs(d1) > TINY else 0.0
    y0 = y0 - lo * y1
    return (y1, y0, piv) if piv else (y0, y1, piv)


def py_pt_params(p, t0, t1, t2):
    n = _cross(_sub(t1, t0), _sub(t2, t0))
    out, pivs = [], []
    for r0, o in ((_sub(t1, t0), t0), (_sub(t2, t1), t1), (_sub(t0, t2), t2)):
        r1 = _cross(r0, n)
        q = _sub(p, o)
        s, t, pv = eigen_ldlt_solve2(_dot(r0, r0), _dot(r0, r1), _dot(r1, r1), _dot(r0, q), _dot(r1, q))
        out += [s, t]
        pivs.append(pv)
    return out, pivs


def classify(st):
    s0, u0, s1, u1, s2, u2 = st
    if 0.0 < s0 < 1.0 and u0 >= 0.0:
        return 3
    if 0.0 < s1 < 1.0 and u1 >= 0.0:
        return 4
    if 0.0 < s2 < 1.0 and u2 >= 0.0:
        return 5
    if s0 <= 0.0 and s2 >= 1.0:
        return 0
    if s1 <= 0.0 and s0 >= 1.0:
        return 1
    if s2 <= 0.0 and s1 >= 1.0:
        return 2
    return 6


def exact_params(p, t0, t1, t2):
    """The same three 2x2 systems solved in exact rationals."""
    F = [tuple(Fraction(float(c)) for c in v) for v in (p, t0, t1, t2)]
    p, t0, t1, t2 = F
    n = _cross(_sub(t1, t0), _sub(t2, t0))
    out = []
    for r0, o in ((_sub(t1, t0), t0), (_sub(t2, t1), t1), (_sub(t0, t2), t2)):
        r1 = _cross(r0, n)
        q = _sub(p, o)
        a00, a01, a11 = _dot(r0, r0), _dot(r0, r1), _dot(r1, r1)
        b0, b1 = _dot(r0, q), _dot(r1, q)
        det = a00 * a11 - a01 * a01
        out += [(b0 * a11 - a01 * b1) / det, (a00 * b1 - a01 * b0) / det]
    return out


def oracle_params(oracle, p, t0, t1, t2):
    st = np.zeros(6)
    args = [oracle._d(oracle.f64(a)) for a in (p, t0, t1, t2)]
    oracle.lib().ora_pt_params(*args, oracle._d(st))
    ty = oracle.lib().ora_type_pt(*args)
    return [float(x) for x in st], ty


def boundary_cases(rng, scale, n):
    """Points placed next to the s = 0, s = 1 and t = 0 boundaries of random
    triangles of the given size (plus plain random points)."""
    out = []
    for _ in range(n):
        t0, t1, t2 = (rng.normal(size=3) * scale for _ in range(3))
        nrm = np.cross(t1 - t0, t2 - t0)
        e = t1 - t0
        w = np.cross(e, nrm)
        w /= np.linalg.norm(w)
        nh = nrm / np.linalg.norm(nrm)
        for s in (0.0, 1e-17, -1e-17, 1e-15, 1.0, 1.0 - 1e-16, 1.0 + 1e-16, 0.5):
            for u in (0.0, 1e-16 * scale, -1e-16 * scale, 0.3 * scale):
                p = t0 + s * e + u * w + rng.uniform(-1, 1) * 1e-3 * scale * nh
                out.append((p, t0, t1, t2))
        out.append((rng.normal(size=3) * scale, t0, t1, t2))
    return out


@pytest.mark.parametrize("scale", [0.05, 1.0, 6.0])
def test_pt_classifier_matches_eigen_ldlt_restatement(oracle, scale):
    rng = np.random.default_rng(int(scale * 1000))
    n_piv = 0
    for p, t0, t1, t2 in boundary_cases(rng, scale, 40):
        mine, pivs = py_pt_params(tuple(p), tuple(t0), tuple(t1), tuple(t2))
        got, ty = oracle_params(oracle, p, t0, t1, t2)
        assert got == mine, (p, t0, t1, t2)
        assert ty == classify(mine)
        n_piv += any(pivs)
    if scale >= 6.0:
        assert n_piv > 0  # triangles with |n| > 1 take the pivoted branch
    if scale <= 0.05:
        assert n_piv == 0


def test_pt_classifier_agrees_with_exact_arithmetic_off_boundary(oracle):
    rng = np.random.default_rng(11)
    checked = 0
    for scale in (0.05, 1.0, 6.0):
        for p, t0, t1, t2 in boundary_cases(rng, scale, 10):
            ex = exact_params(p, t0, t1, t2)
            got, ty = oracle_params(oracle, p, t0, t1, t2)
            # decisions taken at least 1e-9 away from the thresholds 0 and 1
            if all(abs(float(v)) > 1e-9 and abs(float(v) - 1) > 1e-9 for v in ex):
                assert ty == classify([float(v) for v in ex]), (p, t0, t1, t2)
                checked += 1
            # and the rounded parameters are close to the exact ones
            for g, e in zip(got, ex):
                assert abs(g - float(e)) <= 1e-9 * max(1.0, abs(float(e)))
    assert checked > 50
