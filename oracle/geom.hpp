// ORACLE — test infrastructure only. CPU restatement of the reference's FP64
// geometry for the IPC contact path. Nothing in the product links this file.
//
// Parity status: unpinned. The reference ships no tests and no golden vectors,
// and cannot be built here (Eigen/CHOLMOD/Boost/Kokkos absent), so this
// restatement is checked against analytic known-answer cases and finite
// differences instead (tests/test_oracle_*.py).
//
// Floating-point order: every dot product is evaluated left to right,
// ((a0*b0 + a1*b1) + a2*b2); every cross product as
// (a1*b2 - a2*b1, a2*b0 - a0*b2, a0*b1 - a1*b0). The build uses
// -ffp-contract=off so no multiply-add is fused.
#pragma once
#include <cmath>
#include <algorithm>

namespace ora {

struct V3 {
    double x, y, z;
};
inline V3 v3(const double* p) { return {p[0], p[1], p[2]}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double sq(V3 a) { return dot(a, a); }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// ---- squared distances (Math/Distance/POINT_POINT.h:11-17, POINT_EDGE.h:11-25,
//      POINT_TRIANGLE.h:11-22, EDGE_EDGE.h:11-22)
inline double d_PP(V3 a, V3 b) { return sq(a - b); }
inline double d_PE(V3 p, V3 e0, V3 e1) { return sq(cross(e0 - p, e1 - p)) / sq(e1 - e0); }
inline double d_PT(V3 p, V3 t0, V3 t1, V3 t2) {
    V3 b = cross(t1 - t0, t2 - t0);
    double aTb = dot(p - t0, b);
    return aTb * aTb / sq(b);
}
inline double d_EE(V3 ea0, V3 ea1, V3 eb0, V3 eb1) {
    V3 b = cross(ea1 - ea0, eb1 - eb0);
    double aTb = dot(eb0 - ea0, b);
    return aTb * aTb / sq(b);
}

// ---- distance-type classifiers (Math/Distance/DISTANCE_TYPE.h)
inline int type_PE(V3 p, V3 e0, V3 e1) {  // DISTANCE_TYPE.h:11-28
    V3 e = e1 - e0;
    double ratio = dot(e, p - e0) / sq(e);
    if (ratio < 0) return 0;
    if (ratio > 1) return 1;
    return 2;
}

// 2x2 solve of the PT classifier's normal equations, restating the
// reference's `(basis * basis.transpose()).ldlt().solve(...)`
// (DISTANCE_TYPE.h:46,54,62) with Eigen's LDLT as published in its source
// (Eigen/src/Cholesky/LDLT.h, ldlt_inplace<Lower>::unblocked and
// LDLT::_solve_impl, Eigen 3.3/3.4):
//   pivot: the larger diagonal entry goes first (|a11| > |a00|, strictly: a
//          tie keeps the identity, as Eigen's maxCoeff keeps the first maximum);
//   factor: D0 = m00; l = m10 / D0 (left unscaled when D0 == 0);
//           D1 = m11 - l * (D0 * l);
//   solve: y = P b; y1 = y1 - l * y0; y_i = y_i / D_i if |D_i| > DBL_MIN
//          else 0; y0 = y0 - l * y1; x = P^T y.
// The reference is compiled with -mfma under GCC's default
// -ffp-contract=fast (its CMakeLists.txt:20), so which of its products are
// fused into multiply-adds is the compiler's choice; this restatement rounds
// every operation separately (built with -ffp-contract=off).
inline void solve2(double a00, double a01, double a11, double b0, double b1, double& x0, double& x1) {
    const bool piv = std::fabs(a11) > std::fabs(a00);
    const double m00 = piv ? a11 : a00, m11 = piv ? a00 : a11;
    double y0 = piv ? b1 : b0, y1 = piv ? b0 : b1;
    const double D0 = m00;
    double l = a01;
    if (std::fabs(D0) > 0.0) l = a01 / D0;
    const double D1 = m11 - l * (D0 * l);
    y1 = y1 - l * y0;
    const double tiny = 2.2250738585072014e-308;  // numeric_limits<double>::min()
    y0 = std::fabs(D0) > tiny ? y0 / D0 : 0.0;
    y1 = std::fabs(D1) > tiny ? y1 / D1 : 0.0;
    y0 = y0 - l * y1;
    x0 = piv ? y1 : y0;
    x1 = piv ? y0 : y1;
}

inline void pt_param(V3 r0, V3 n, V3 p, V3 o, double& s, double& t) {
    V3 r1 = cross(r0, n);
    V3 q = p - o;
    solve2(dot(r0, r0), dot(r0, r1), dot(r1, r1), dot(r0, q), dot(r1, q), s, t);
}

inline int type_PT(V3 p, V3 t0, V3 t1, V3 t2) {  // DISTANCE_TYPE.h:30-82
    V3 n = cross(t1 - t0, t2 - t0);
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

inline int type_EE(V3 ea0, V3 ea1, V3 eb0, V3 eb1) {  // DISTANCE_TYPE.h:85-164
    V3 u = ea1 - ea0, v = eb1 - eb0, w = ea0 - eb0;
    double a = sq(u), b = dot(u, v), c = sq(v), d = dot(u, w), e = dot(v, w);
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
        V3 uv = cross(u, v);
        if (tN > 0.0 && tN < tD && (dot(uv, w) == 0.0 || sq(uv) < 1.0e-20 * a * c)) {
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

// ---- unclassified distances used by ACCD (DISTANCE_UNCLASSIFIED.h:15-148)
inline double d_PT_unclassified(V3 p, V3 t0, V3 t1, V3 t2) {
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
inline double d_EE_unclassified(V3 ea0, V3 ea1, V3 eb0, V3 eb1) {
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

// ---- edge-edge mollifier (EDGE_EDGE_MOLLIFIER.h:9-18, 440-477, 582-590)
inline double ee_cross_norm2(V3 ea0, V3 ea1, V3 eb0, V3 eb1) { return sq(cross(ea1 - ea0, eb1 - eb0)); }
inline double ee_mollifier_threshold(V3 a0r, V3 a1r, V3 b0r, V3 b1r) {
    return 1.0e-3 * sq(a0r - a1r) * sq(b0r - b1r);
}
inline double ee_mollifier(double c, double eps_x) {
    if (c < eps_x) {
        double q = c / eps_x;
        return (-q + 2.0) * q;
    }
    return 1.0;
}

// ---- log barrier (Math/BARRIER.h:9-62, non-elastic branch)
inline double barrier(double d, double dHat, double kappa) {
    return -kappa * (d - dHat) * (d - dHat) * std::log(d / dHat);
}
inline double barrier_g(double d, double dHat, double kappa) {
    double t2 = d - dHat;
    return kappa * (t2 * std::log(d / dHat) * -2.0 - (t2 * t2) / d);
}
inline double barrier_h(double d, double dHat, double kappa) {
    double t2 = d - dHat;
    return kappa * ((std::log(d / dHat) * -2.0 - t2 * 4.0 / d) + 1.0 / (d * d) * (t2 * t2));
}

}  // namespace ora
