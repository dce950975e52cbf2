// ORACLE — test infrastructure only. CPU restatement of the discrete-shell
// elasticity of the reference's Advance_One_Step_IE_Hinge path
// (FEM/Shell/DISCRETE_SHELL.h:1110 = <double, 3, KL = false, ...>):
//   * neo-Hookean membrane on the first fundamental form
//     (FEM/Shell/MEMBRANE.h:7-322, useNH = true);
//   * hinge bending on the dihedral angle of every interior edge
//     (FEM/Shell/BENDING.h:9-602, the !KL branches; Math/DIHEDRAL_ANGLE.h),
//     with the hinge stencils and rest data of
//     Compute_Discrete_Shell_Inv_Basis (DISCRETE_SHELL.h:132-216) and the
//     stiffness of Initialize_Discrete_Shell (DISCRETE_SHELL.h:218-357).
// Nothing in the product links this file.
#pragma once
#include <cmath>

#include "geom.hpp"

namespace ora {

// ---- membrane, one face x1 x2 x3 with the inverse (ib00, ib01, ib11) of its
// rest first fundamental form and det of that inverse (MEMBRANE.h:19-49)
struct MemFace {
    double ib00, ib01, ib11, detib, vol, lam, mu;
};

// dA/dx rows (A00, A10, A01, A11) x 9 columns (x1, x2, x3), MEMBRANE.h:87-97
inline void membrane_dA(V3 e01, V3 e02, double dA[4][9]) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 9; ++c) dA[r][c] = 0.0;
    const double a[3] = {e01.x, e01.y, e01.z}, b[3] = {e02.x, e02.y, e02.z};
    for (int d = 0; d < 3; ++d) {
        dA[0][3 + d] += 2.0 * a[d];
        dA[0][d] -= 2.0 * a[d];
        for (int r = 1; r <= 2; ++r) {
            dA[r][6 + d] += a[d];
            dA[r][3 + d] += b[d];
            dA[r][d] += -a[d] - b[d];
        }
        dA[3][6 + d] += 2.0 * b[d];
        dA[3][d] -= 2.0 * b[d];
    }
}

// w * vol * (mu/2 (tr(IB^-1 A) - 2 - 2 lnJ) + lam/2 lnJ^2), lnJ = ln(det A det IB^-1)/2;
// gradient g[9] (may be null) and Hessian H[81] (may be null, unprojected)
inline double membrane_face(V3 x1, V3 x2, V3 x3, const MemFace& m, double w, double* g, double* H) {
    const V3 e01 = x2 - x1, e02 = x3 - x1;
    const double a00 = sq(e01), a01 = dot(e01, e02), a11 = sq(e02);
    const double detA = a00 * a11 - a01 * a01;
    const double lnJ = std::log(detA * m.detib) / 2;
    const double trIA = m.ib00 * a00 + 2.0 * m.ib01 * a01 + m.ib11 * a11;
    const double E = w * m.vol * (m.mu / 2 * (trIA - 2 - 2 * lnJ) + m.lam / 2 * lnJ * lnJ);
    if (!g && !H) return E;
    double dA[4][9];
    membrane_dA(e01, e02, dA);
    // A^-1 (symmetric): (a11, -a01, -a01, a00) / detA, in (00, 10, 01, 11) order
    const double IA[4] = {a11 / detA, -a01 / detA, -a01 / detA, a00 / detA};
    const double IB[4] = {m.ib00, m.ib01, m.ib01, m.ib11};
    const double term1 = (-m.mu + m.lam * lnJ) / 2;
    if (g) {
        double temp[4];
        for (int r = 0; r < 4; ++r) temp[r] = w * m.vol * (m.mu / 2 * IB[r] + term1 * IA[r]);
        for (int i = 0; i < 9; ++i) g[i] = dA[0][i] * temp[0] + dA[1][i] * temp[1] + dA[2][i] * temp[2] + dA[3][i] * temp[3];
    }
    if (H) {
        double ainvda[9];
        for (int i = 0; i < 9; ++i)
            ainvda[i] = dA[0][i] * IA[0] + dA[1][i] * IA[1] + dA[2][i] * IA[2] + dA[3][i] * IA[3];
        const double c0 = -term1 + m.lam / 4, c1 = term1 / detA;
        const int adj[4] = {3, 1, 2, 0};
        const double sgn[4] = {1.0, -1.0, -1.0, 1.0};
        for (int i = 0; i < 9; ++i)
            for (int j = 0; j < 9; ++j) {
                double s = c0 * ainvda[i] * ainvda[j];
                double t = 0;
                for (int r = 0; r < 4; ++r) t += sgn[r] * dA[adj[r]][i] * dA[r][j];
                H[i * 9 + j] = s + c1 * t;
            }
        // constant second derivatives of A (MEMBRANE.h:140-170): coefficient
        // of block (p, q) of vertex pairs for each entry r of A
        for (int r = 0; r < 4; ++r) {
            const double c = term1 * IA[r] + m.mu / 2 * IB[r];
            double blk[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            if (r == 0) { blk[0][0] = 2; blk[1][1] = 2; blk[0][1] = blk[1][0] = -2; }
            else if (r == 3) { blk[0][0] = 2; blk[2][2] = 2; blk[0][2] = blk[2][0] = -2; }
            else { blk[1][2] = blk[2][1] = 1; blk[0][1] = blk[0][2] = blk[1][0] = blk[2][0] = -1; blk[0][0] = 2; }
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q)
                    if (blk[p][q] != 0)
                        for (int d = 0; d < 3; ++d) H[(3 * p + d) * 9 + 3 * q + d] += c * blk[p][q];
        }
        for (int i = 0; i < 81; ++i) H[i] *= w * m.vol;
    }
    return E;
}

// ---- dihedral angle of the hinge (x0, x1, x2, x3), hinge edge x1-x2,
// Compute_Dihedral_Angle (DIHEDRAL_ANGLE.h:10-24)
inline double dihedral_angle(V3 x0, V3 x1, V3 x2, V3 x3) {
    const V3 n1 = cross(x1 - x0, x2 - x0), n2 = cross(x2 - x3, x1 - x3);
    double c = dot(n1, n2) / std::sqrt(sq(n1) * sq(n2));
    c = std::max(-1.0, std::min(1.0, c));
    double t = std::acos(c);
    if (dot(cross(n2, n1), x1 - x2) < 0) t = -t;
    return t;
}

inline V3 unit(V3 a) { return (1.0 / std::sqrt(sq(a))) * a; }
// Compute_mHat (DIHEDRAL_ANGLE.h:1179-1188)
inline V3 mhat(V3 xp, V3 xe0, V3 xe1) {
    const V3 e = xe1 - xe0;
    return unit(xe0 + (dot(xp - xe0, e) / sq(e)) * e - xp);
}

// gradient (12) and Hessian (144) of the dihedral angle: the hinge-angle
// derivatives of Tamstorf & Grinspun ("Discrete bending forces and their
// Jacobians", 2013) as the reference's Compute_Dihedral_Angle_Hessian
// (DIHEDRAL_ANGLE.h:1190-1277) writes them, with the stencil's x0, x1, x2,
// x3 in the roles v2, v0, v1, v3 (hinge v0-v1); the gradient in the same
// quantities: -n1/h01 (x0), cos a3/h3 n1 + cos a4/h4 n2 (x1),
// cos a1/h1 n1 + cos a2/h2 n2 (x2), -n2/h02 (x3) with unit normals
inline void dihedral_derivs(V3 x0, V3 x1, V3 x2, V3 x3, double* g, double* H) {
    const V3 v2 = x0, v0 = x1, v1 = x2, v3 = x3;
    const V3 e[5] = {v1 - v0, v2 - v0, v3 - v0, v2 - v1, v3 - v1};
    double ne[5];
    for (int i = 0; i < 5; ++i) ne[i] = std::sqrt(sq(e[i]));
    const V3 n1 = cross(e[0], e[1]), n2 = cross(e[2], e[0]);
    const double n1n = std::sqrt(sq(n1)), n2n = std::sqrt(sq(n2));
    const double ca1 = dot(e[0], e[1]) / (ne[0] * ne[1]);
    const double ca2 = dot(e[0], e[2]) / (ne[0] * ne[2]);
    const double ca3 = -dot(e[0], e[3]) / (ne[0] * ne[3]);
    const double ca4 = -dot(e[0], e[4]) / (ne[0] * ne[4]);
    const double h1 = n1n / ne[1], h2 = n2n / ne[2], h3 = n1n / ne[3], h4 = n2n / ne[4];
    const double h01 = n1n / ne[0], h02 = n2n / ne[0];
    if (g) {
        const V3 u1 = (1.0 / n1n) * n1, u2 = (1.0 / n2n) * n2;
        const V3 gg[4] = {(-1.0 / h01) * u1, (ca3 / h3) * u1 + (ca4 / h4) * u2, (ca1 / h1) * u1 + (ca2 / h2) * u2,
                          (-1.0 / h02) * u2};
        for (int k = 0; k < 4; ++k) {
            g[3 * k] = gg[k].x;
            g[3 * k + 1] = gg[k].y;
            g[3 * k + 2] = gg[k].z;
        }
    }
    if (!H) return;
    const V3 m1 = mhat(v1, v0, v2), m2 = mhat(v1, v0, v3), m3 = mhat(v0, v1, v2), m4 = mhat(v0, v1, v3);
    const V3 m01 = mhat(v2, v0, v1), m02 = mhat(v3, v0, v1);
    // a b^T scaled
    auto outer = [](V3 a, V3 b, double s, double M[9]) {
        const double A[3] = {a.x, a.y, a.z}, B[3] = {b.x, b.y, b.z};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[i * 3 + j] = s * A[i] * B[j];
    };
    double N1_01[9], N1_3[9], N1_1[9], N2_4[9], N2_2[9], N2_02[9];
    outer(n1, m01, 1.0 / (h01 * h01 * n1n), N1_01);
    outer(n1, m3, 1.0 / (h01 * h3 * n1n), N1_3);
    outer(n1, m1, 1.0 / (h01 * h1 * n1n), N1_1);
    outer(n2, m4, 1.0 / (h02 * h4 * n2n), N2_4);
    outer(n2, m2, 1.0 / (h02 * h2 * n2n), N2_2);
    outer(n2, m02, 1.0 / (h02 * h02 * n2n), N2_02);
    double M3_01_1[9], M1_01_1[9], M1_1_1[9], M3_3_1[9], M3_1_1[9], M1_3_1[9];
    double M4_02_2[9], M2_02_2[9], M4_4_2[9], M2_4_2[9], M4_2_2[9], M2_2_2[9], B1[9], B2[9];
    outer(m01, n1, ca3 / (h3 * h01 * n1n), M3_01_1);
    outer(m01, n1, ca1 / (h1 * h01 * n1n), M1_01_1);
    outer(m1, n1, ca1 / (h1 * h1 * n1n), M1_1_1);
    outer(m3, n1, ca3 / (h3 * h3 * n1n), M3_3_1);
    outer(m1, n1, ca3 / (h3 * h1 * n1n), M3_1_1);
    outer(m3, n1, ca1 / (h1 * h3 * n1n), M1_3_1);
    outer(m02, n2, ca4 / (h4 * h02 * n2n), M4_02_2);
    outer(m02, n2, ca2 / (h2 * h02 * n2n), M2_02_2);
    outer(m4, n2, ca4 / (h4 * h4 * n2n), M4_4_2);
    outer(m4, n2, ca2 / (h2 * h4 * n2n), M2_4_2);
    outer(m2, n2, ca4 / (h4 * h2 * n2n), M4_2_2);
    outer(m2, n2, ca2 / (h2 * h2 * n2n), M2_2_2);
    outer(n1, m01, 1.0 / (ne[0] * ne[0] * n1n), B1);
    outer(n2, m02, 1.0 / (ne[0] * ne[0] * n2n), B2);
    auto T = [](const double* M, int i, int j) { return M[j * 3 + i]; };
    for (int i = 0; i < 144; ++i) H[i] = 0.0;
    auto put = [&](int bi, int bj, int i, int j, double v) { H[(3 * bi + i) * 12 + 3 * bj + j] = v; };
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int k = i * 3 + j;
            put(0, 0, i, j, -(N1_01[k] + T(N1_01, i, j)));
            const double b10 = M3_01_1[k] - N1_3[k], b20 = M1_01_1[k] - N1_1[k];
            put(1, 0, i, j, b10);
            put(0, 1, j, i, b10);
            put(2, 0, i, j, b20);
            put(0, 2, j, i, b20);
            put(1, 1, i, j, M3_3_1[k] + T(M3_3_1, i, j) - B1[k] + M4_4_2[k] + T(M4_4_2, i, j) - B2[k]);
            const double b12 = M3_1_1[k] + T(M1_3_1, i, j) + B1[k] + M4_2_2[k] + T(M2_4_2, i, j) + B2[k];
            put(1, 2, i, j, b12);
            put(2, 1, j, i, b12);
            const double b13 = M4_02_2[k] - N2_4[k], b23 = M2_02_2[k] - N2_2[k];
            put(1, 3, i, j, b13);
            put(3, 1, j, i, b13);
            put(2, 2, i, j, M1_1_1[k] + T(M1_1_1, i, j) - B1[k] + M2_2_2[k] + T(M2_2_2, i, j) - B2[k]);
            put(2, 3, i, j, b23);
            put(3, 2, j, i, b23);
            put(3, 3, i, j, -(N2_02[k] + T(N2_02, i, j)));
        }
}

// ---- hinge bending of one stencil (BENDING.h:52-76, 176-211, 430-485):
// E = w k (theta - thetabar)^2 ebar / hbar with w = h^2
inline double bending_hinge(V3 x0, V3 x1, V3 x2, V3 x3, double thetabar, double ebar, double hbar, double k,
                            double w, double* g, double* H) {
    const double th = dihedral_angle(x0, x1, x2, x3);
    const double E = w * k * (th - thetabar) * (th - thetabar) * ebar / hbar;
    if (!g && !H) return E;
    double dg[12], dH[144];
    dihedral_derivs(x0, x1, x2, x3, dg, H ? dH : nullptr);
    const double cg = w * k * 2 * (th - thetabar) * ebar / hbar;
    if (g)
        for (int i = 0; i < 12; ++i) g[i] = cg * dg[i];
    if (H) {
        const double cq = w * k * 2 * ebar / hbar;
        for (int i = 0; i < 12; ++i)
            for (int j = 0; j < 12; ++j) H[i * 12 + j] = cg * dH[i * 12 + j] + (cq * dg[i]) * dg[j];
    }
    return E;
}

}  // namespace ora
