// Exact orientation predicate and the segment-triangle intersection test of
// the intersection check (Check_Edge_Tri_Intersect / segTriIntersect,
// FEM/IPC.h:2390-2517).
//
// orient3d_sign(a, b, c, d) is the exact sign of det[a-d; b-d; c-d]. It
// follows the method of J. R. Shewchuk, "Adaptive Precision Floating-Point
// Arithmetic and Fast Robust Geometric Predicates" (Discrete Comput. Geom.
// 18, 1997): a floating-point evaluation whose sign is accepted when the
// determinant clears that paper's a-priori error bound (7 + 56 eps) eps times
// the permanent, and otherwise an exact evaluation with floating-point
// expansions. The exact stage here is this file's own: the 4x4 form
// det[a 1; b 1; c 1; d 1] is expanded into 24 signed triple products of input
// coordinates, each split exactly into four doubles with fused multiply-add
// error-free products, and all of them are accumulated into one
// nonoverlapping expansion (grow-expansion with zero elimination); its sign is
// the sign of its largest component. Exact for finite inputs whose triple
// products neither overflow nor underflow (|coordinate| between 1e-90 and
// 1e90, or zero).
//
// Translation units that include this must be compiled with --fmad=false
// (the filter's bound assumes every operation is rounded separately).
#pragma once
#include <cmath>

namespace idp {
namespace pred {

#if defined(__CUDACC__)
#define IDP_HD __host__ __device__ __forceinline__
#else
#define IDP_HD inline
#endif

// x + y = a + b exactly (Knuth's two-sum; any magnitudes)
IDP_HD void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    const double bv = x - a;
    const double av = x - bv;
    y = (a - av) + (b - bv);
}

// x + y = a * b exactly
IDP_HD void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
    y = fma(a, b, -x);
}

// e[0, n): nonoverlapping, increasing magnitude, no zeros. Adds b in place
// and returns the new length (at most n + 1).
IDP_HD int grow(double* e, int n, double b) {
    double q = b;
    int m = 0;
    for (int i = 0; i < n; ++i) {
        double hh;
        two_sum(q, e[i], q, hh);
        if (hh != 0.0) e[m++] = hh;
    }
    if (q != 0.0) e[m++] = q;
    return m;
}

// adds s * p * q * r exactly (four doubles) to the expansion
IDP_HD int grow_triple(double* e, int n, double s, double p, double q, double r) {
    double x, y, x1, y1, x2, y2;
    two_prod(p, q, x, y);
    two_prod(x, r, x1, y1);
    two_prod(y, r, x2, y2);
    n = grow(e, n, s * y2);
    n = grow(e, n, s * x2);
    n = grow(e, n, s * y1);
    return grow(e, n, s * x1);
}

// adds sgn * det[p; q; r] (rows) to the expansion
IDP_HD int grow_det3(double* e, int n, double sgn, const double p[3], const double q[3], const double r[3]) {
    n = grow_triple(e, n, sgn, p[0], q[1], r[2]);
    n = grow_triple(e, n, -sgn, p[0], q[2], r[1]);
    n = grow_triple(e, n, -sgn, p[1], q[0], r[2]);
    n = grow_triple(e, n, sgn, p[1], q[2], r[0]);
    n = grow_triple(e, n, sgn, p[2], q[0], r[1]);
    return grow_triple(e, n, -sgn, p[2], q[1], r[0]);
}

#if defined(__CUDACC__)
#define IDP_HD_COLD __host__ __device__ __noinline__
#else
#define IDP_HD_COLD __attribute__((noinline))
#endif

// exact stage: det[a 1; b 1; c 1; d 1] by cofactors of the column of ones
// (out of line: it runs only when the filter cannot decide)
IDP_HD_COLD int orient3d_exact(const double a[3], const double b[3], const double c[3], const double d[3]) {
    double e[100];
    int n = 0;
    n = grow_det3(e, n, -1.0, b, c, d);
    n = grow_det3(e, n, 1.0, a, c, d);
    n = grow_det3(e, n, -1.0, a, b, d);
    n = grow_det3(e, n, 1.0, a, b, c);
    if (n == 0) return 0;
    return e[n - 1] > 0.0 ? 1 : -1;
}

// sign of det[a-d; b-d; c-d]: +1, -1 or 0 (exact)
IDP_HD int orient3d_sign(const double a[3], const double b[3], const double c[3], const double d[3]) {
    const double adx = a[0] - d[0], ady = a[1] - d[1], adz = a[2] - d[2];
    const double bdx = b[0] - d[0], bdy = b[1] - d[1], bdz = b[2] - d[2];
    const double cdx = c[0] - d[0], cdy = c[1] - d[1], cdz = c[2] - d[2];
    const double bc = bdx * cdy, cb = cdx * bdy;
    const double ca = cdx * ady, ac = adx * cdy;
    const double ab = adx * bdy, ba = bdx * ady;
    const double det = adz * (bc - cb) + bdz * (ca - ac) + cdz * (ab - ba);
    const double perm = (fabs(bc) + fabs(cb)) * fabs(adz) + (fabs(ca) + fabs(ac)) * fabs(bdz) +
                        (fabs(ab) + fabs(ba)) * fabs(cdz);
    const double eps = 1.1102230246251565e-16;  // 2^-53
    const double bound = (7.0 + 56.0 * eps) * eps * perm;
    if (det > bound) return 1;
    if (-det > bound) return -1;
    return orient3d_exact(a, b, c, d);
}

// Does the closed segment e0-e1 cross the closed triangle t0 t1 t2?
// segTriIntersect (FEM/IPC.h:2390-2442) with exact predicates: false when
// either endpoint lies in the triangle's plane (coplanar contact is the
// distance test's business) or both lie on the same side; otherwise the
// crossing point is inside the closed triangle iff the line e0-e1 passes no
// triangle edge on the outside, i.e. the three orientations of (e0, e1, ti,
// tj) have no two strictly opposite signs.
IDP_HD bool seg_tri_intersect(const double e0[3], const double e1[3], const double t0[3], const double t1[3],
                              const double t2[3]) {
    const int o0 = orient3d_sign(t0, t1, t2, e0);
    const int o1 = orient3d_sign(t0, t1, t2, e1);
    if (o0 == 0 || o1 == 0 || o0 == o1) return false;
    const int s0 = orient3d_sign(e0, e1, t0, t1);
    const int s1 = orient3d_sign(e0, e1, t1, t2);
    const int s2 = orient3d_sign(e0, e1, t2, t0);
    const bool pos = s0 > 0 || s1 > 0 || s2 > 0;
    const bool neg = s0 < 0 || s1 < 0 || s2 < 0;
    return !(pos && neg);
}

#undef IDP_HD
#undef IDP_HD_COLD

}  // namespace pred
}  // namespace idp
