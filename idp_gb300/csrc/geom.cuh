// FP64 contact geometry on the device: squared distances, distance-type
// classifiers, unclassified distances, edge-edge mollifier and the log
// barrier. Translation units that must reproduce the constraint set and the
// CCD step bit for bit (contact.cu, ccd.cu) are compiled with --fmad=false,
// so every product and sum below is rounded separately, in the order written.
//
// Reference functions: Math/Distance/POINT_POINT.h:11-17, POINT_EDGE.h:11-25,
// POINT_TRIANGLE.h:11-22, EDGE_EDGE.h:11-22, DISTANCE_TYPE.h:11-164,
// DISTANCE_UNCLASSIFIED.h:15-148, EDGE_EDGE_MOLLIFIER.h:9-18,440-477,582-590,
// Math/BARRIER.h:9-62.
#pragma once
#include "common.cuh"

namespace idp {
namespace geo {

__device__ __forceinline__ double d_PP(D3 a, D3 b) { return sqn(a - b); }
__device__ __forceinline__ double d_PE(D3 p, D3 e0, D3 e1) { return sqn(cross(e0 - p, e1 - p)) / sqn(e1 - e0); }
__device__ __forceinline__ double d_PT(D3 p, D3 t0, D3 t1, D3 t2) {
    D3 b = cross(t1 - t0, t2 - t0);
    double aTb = dot(p - t0, b);
    return aTb * aTb / sqn(b);
}
__device__ __forceinline__ double d_EE(D3 ea0, D3 ea1, D3 eb0, D3 eb1) {
    D3 b = cross(ea1 - ea0, eb1 - eb0);
    double aTb = dot(eb0 - ea0, b);
    return aTb * aTb / sqn(b);
}

// Solve of the PT classifier's 2x2 normal equations (the reference's
// `(basis * basis.transpose()).ldlt().solve(basis * (p - o))`,
// DISTANCE_TYPE.h:46,54,62) by Eigen's LDLT with diagonal pivoting: the
// larger diagonal entry first (ties keep the identity); D0 = m00,
// l = m10 / D0, D1 = m11 - l * (D0 * l); forward substitution, division by
// D_i (0 when |D_i| <= DBL_MIN), back substitution, inverse permutation.
__device__ __forceinline__ void pt_param(D3 r0, D3 n, D3 p, D3 o, double& s, double& t) {
    D3 r1 = cross(r0, n);
    D3 q = p - o;
    double a00 = dot(r0, r0), a01 = dot(r0, r1), a11 = dot(r1, r1);
    double b0 = dot(r0, q), b1 = dot(r1, q);
    const bool piv = fabs(a11) > fabs(a00);
    const double m00 = piv ? a11 : a00, m11 = piv ? a00 : a11;
    double y0 = piv ? b1 : b0, y1 = piv ? b0 : b1;
    const double D0 = m00;
    double l = a01;
    if (fabs(D0) > 0.0) l = a01 / D0;
    const double D1 = m11 - l * (D0 * l);
    y1 = y1 - l * y0;
    const double tiny = 2.2250738585072014e-308;
    y0 = fabs(D0) > tiny ? y0 / D0 : 0.0;
    y1 = fabs(D1) > tiny ? y1 / D1 : 0.0;
    y0 = y0 - l * y1;
    s = piv ? y1 : y0;
    t = piv ? y0 : y1;
}

__device__ inline int type_PT(D3 p, D3 t0, D3 t1, D3 t2) {
    D3 n = cross(t1 - t0, t2 - t0);
    double s0, u0, s1, u1, s2, u2;
    pt_param(t1 - t0, n, p, t0, s0, u0);
    if (s0 > 0.0 && s0 < 1.0 && u0 >= 0.0) return 3;
    pt_param(t2 - t1, n, p, t1, s1, u1);
    if (s1 > 0.0 && s1 < 1.0 && u1 >= 0.0) return 4;
    pt_param(t0 - t2, n, p, t2, s2, u2);
    if (s2 > 0.0 && s2 < 1.0 && u2 >= 0.0) return 5;
    if (s0 <= 0.0 && s2 >= 1.0) return 0;
    if (s1 <= 0.0 && s0 >= 1.0) return 1;
    if (s2 <= 0.0 && s1 >= 1.0) return 2;
    return 6;
}

__device__ inline int type_EE(D3 ea0, D3 ea1, D3 eb0, D3 eb1) {
    D3 u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0;
    double a = sqn(u), b = dot(u, v), c = sqn(v), d = dot(u, w), e = dot(v, w);
    double D = a * c - b * b;
    double tD = D;
    double sN, tN;
    int defaultCase = 8;
    sN = (b * e - c * d);
    if (sN <= 0.0) {
        tN = e; tD = c; defaultCase = 2;
    } else if (sN >= D) {
        tN = e + b; tD = c; defaultCase = 5;
    } else {
        tN = (a * e - b * d);
        D3 uv = cross(u, v);
        if (tN > 0.0 && tN < tD && (dot(uv, w) == 0.0 || sqn(uv) < 1.0e-20 * a * c)) {
            if (sN < D / 2) { tN = e; tD = c; defaultCase = 2; }
            else { tN = e + b; tD = c; defaultCase = 5; }
        }
    }
    if (tN <= 0.0) {
        if (-d <= 0.0) return 0;
        else if (-d >= a) return 3;
        else return 6;
    } else if (tN >= tD) {
        if ((-d + b) <= 0.0) return 1;
        else if ((-d + b) >= a) return 4;
        else return 7;
    }
    return defaultCase;
}

__device__ inline double d_PT_unclassified(D3 p, D3 t0, D3 t1, D3 t2) {
    switch (type_PT(p, t0, t1, t2)) {
        case 0: return d_PP(p, t0);
        case 1: return d_PP(p, t1);
        case 2: return d_PP(p, t2);
        case 3: return d_PE(p, t0, t1);
        case 4: return d_PE(p, t1, t2);
        case 5: return d_PE(p, t2, t0);
        default: return d_PT(p, t0, t1, t2);
    }
}
// The same value as d_PT_unclassified, scheduled for a single long-running
// thread: the classifier's three 2x2 solves and all seven candidate
// distances are independent of one another, so they are all evaluated (their
// divisions overlap) and the classifier's decision then selects one. Every
// operation of the selected branch is the one d_PT_unclassified performs, so
// the result is bit-identical; the unselected values (which may be inf or
// NaN on degenerate inputs) are discarded.
__device__ inline double d_PT_unclassified_ilp(D3 p, D3 t0, D3 t1, D3 t2) {
    D3 n = cross(t1 - t0, t2 - t0);
    double s0, u0, s1, u1, s2, u2;
    pt_param(t1 - t0, n, p, t0, s0, u0);
    pt_param(t2 - t1, n, p, t1, s1, u1);
    pt_param(t0 - t2, n, p, t2, s2, u2);
    const double dpp0 = d_PP(p, t0), dpp1 = d_PP(p, t1), dpp2 = d_PP(p, t2);
    const double dpe0 = d_PE(p, t0, t1), dpe1 = d_PE(p, t1, t2), dpe2 = d_PE(p, t2, t0);
    const double dpt = d_PT(p, t0, t1, t2);
    if (s0 > 0.0 && s0 < 1.0 && u0 >= 0.0) return dpe0;
    if (s1 > 0.0 && s1 < 1.0 && u1 >= 0.0) return dpe1;
    if (s2 > 0.0 && s2 < 1.0 && u2 >= 0.0) return dpe2;
    if (s0 <= 0.0 && s2 >= 1.0) return dpp0;
    if (s1 <= 0.0 && s0 >= 1.0) return dpp1;
    if (s2 <= 0.0 && s1 >= 1.0) return dpp2;
    return dpt;
}
__device__ inline double d_EE_unclassified(D3 ea0, D3 ea1, D3 eb0, D3 eb1) {
    switch (type_EE(ea0, ea1, eb0, eb1)) {
        case 0: return d_PP(ea0, eb0);
        case 1: return d_PP(ea0, eb1);
        case 2: return d_PE(ea0, eb0, eb1);
        case 3: return d_PP(ea1, eb0);
        case 4: return d_PP(ea1, eb1);
        case 5: return d_PE(ea1, eb0, eb1);
        case 6: return d_PE(eb0, ea0, ea1);
        case 7: return d_PE(eb1, ea0, ea1);
        default: return d_EE(ea0, ea1, eb0, eb1);
    }
}

__device__ __forceinline__ double ee_cross_norm2(D3 ea0, D3 ea1, D3 eb0, D3 eb1) {
    return sqn(cross(ea1 - ea0, eb1 - eb0));
}
__device__ __forceinline__ double mollifier_threshold(D3 a0r, D3 a1r, D3 b0r, D3 b1r) {
    return 1.0e-3 * sqn(a0r - a1r) * sqn(b0r - b1r);
}
__device__ __forceinline__ double mollifier(double c, double eps_x) {
    if (c < eps_x) {
        double q = c / eps_x;
        return (-q + 2.0) * q;
    }
    return 1.0;
}

__device__ __forceinline__ double barrier(double d, double dHat, double kappa) {
    return -kappa * (d - dHat) * (d - dHat) * log(d / dHat);
}
__device__ __forceinline__ double barrier_g(double d, double dHat, double kappa) {
    double t2 = d - dHat;
    return kappa * (t2 * log(d / dHat) * -2.0 - (t2 * t2) / d);
}
__device__ __forceinline__ double barrier_h(double d, double dHat, double kappa) {
    double t2 = d - dHat;
    return kappa * ((log(d / dHat) * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2));
}

// Constraint stencil decoded from the sign-tagged int4 of FEM/IPC.h:202-250,
// 439-547, 652. kind: 0 PP, 1 PE, 2 PT, 3 EE, 4 EE mollified, 5 PE
// mollified, 6 PP mollified. v[] in derivative order; mult = multiplicity.
struct Stencil {
    int kind, nv;
    int v[4];
    int mult;
};
__device__ __forceinline__ Stencil decode(int4 c) {
    Stencil s;
    s.mult = 1;
    if (c.x >= 0) {
        s.nv = 4;
        if (c.w >= 0 && c.z >= 0) { s.kind = 3; s.v[0] = c.x; s.v[1] = c.y; s.v[2] = c.z; s.v[3] = c.w; }
        else if (c.w >= 0) { s.kind = 4; s.v[0] = c.x; s.v[1] = c.y; s.v[2] = -c.z - 1; s.v[3] = c.w; }
        else if (c.z >= 0) { s.kind = 5; s.v[0] = c.x; s.v[1] = -c.w - 1; s.v[2] = c.y; s.v[3] = c.z; }
        else { s.kind = 6; s.v[0] = c.x; s.v[1] = -c.z - 1; s.v[2] = c.y; s.v[3] = -c.w - 1; }
    } else {
        s.v[0] = -c.x - 1;
        s.v[1] = c.y;
        if (c.w >= 0) { s.kind = 2; s.nv = 4; s.v[2] = c.z; s.v[3] = c.w; }
        else if (c.z >= 0) { s.kind = 1; s.nv = 3; s.v[2] = c.z; s.v[3] = -1; s.mult = -c.w; }
        else { s.kind = 0; s.nv = 2; s.v[2] = -1; s.v[3] = -1; s.mult = -c.w; }
    }
    return s;
}

// raw squared distance of a decoded constraint (FEM/IPC.h:2288-2384)
__device__ inline double stencil_dist2(const Stencil& s, const double* X) {
    D3 a = ld3(X, s.v[0]);
    switch (s.kind) {
        case 0: return d_PP(a, ld3(X, s.v[1]));
        case 1: return d_PE(a, ld3(X, s.v[1]), ld3(X, s.v[2]));
        case 2: return d_PT(a, ld3(X, s.v[1]), ld3(X, s.v[2]), ld3(X, s.v[3]));
        case 3: case 4: return d_EE(a, ld3(X, s.v[1]), ld3(X, s.v[2]), ld3(X, s.v[3]));
        case 5: return d_PE(a, ld3(X, s.v[2]), ld3(X, s.v[3]));
        default: return d_PP(a, ld3(X, s.v[2]));
    }
}

}  // namespace geo
}  // namespace idp
