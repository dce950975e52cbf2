// ORACLE — test infrastructure only. Gradients and Hessians of the squared
// distances and of the edge-edge cross norm, in vertex coordinates.
//
// The reference ships Matlab-generated expressions (g_PT/H_PT at
// POINT_TRIANGLE.h:24-550, g_EE/H_EE at EDGE_EDGE.h:24-733, g_PE3D/H_PE3D at
// POINT_EDGE.h:61-588, g_EECN2/H_EECN2 at EDGE_EDGE_MOLLIFIER.h:21-383). This
// restatement derives the same functions by the chain rule instead:
//   PT, EE:  d = s^2 / D,  s = w . (u x v),  D = |u x v|^2
//   PE:      d = |a x b|^2 / |b - a|^2
//   EECN2:   c = |u x v|^2
// with (w, u, v) or (a, b) differences of the vertices, mapped back to the
// 12 (or 9, 6) vertex coordinates by a constant +-1 block map.
#pragma once
#include "geom.hpp"

namespace ora {

// 3x3 helpers on row-major double[9]
inline void eps_mat(V3 v, double* E) {  // E_ij = eps_ijk v_k
    E[0] = 0;     E[1] = v.z;   E[2] = -v.y;
    E[3] = -v.z;  E[4] = 0;     E[5] = v.x;
    E[6] = v.y;   E[7] = -v.x;  E[8] = 0;
}

// D = |u x v|^2 : gradient (6) and Hessian (6x6 row-major) in (u, v)
inline void crossnorm2_derivs(V3 u, V3 v, double* g, double* H) {
    double uu = dot(u, u), vv = dot(v, v), uv = dot(u, v);
    double ua[3] = {u.x, u.y, u.z}, va[3] = {v.x, v.y, v.z};
    for (int i = 0; i < 3; ++i) {
        g[i] = 2.0 * (vv * ua[i] - uv * va[i]);
        g[3 + i] = 2.0 * (uu * va[i] - uv * ua[i]);
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double dij = (i == j) ? 1.0 : 0.0;
            H[i * 6 + j] = 2.0 * (vv * dij - va[i] * va[j]);
            H[(3 + i) * 6 + 3 + j] = 2.0 * (uu * dij - ua[i] * ua[j]);
            double c = 2.0 * (2.0 * ua[i] * va[j] - va[i] * ua[j] - uv * dij);
            H[i * 6 + 3 + j] = c;        // d2D / du_i dv_j
            H[(3 + j) * 6 + i] = c;      // symmetric
        }
}

// map z-space derivatives to vertex space: x-block a = sum_k C[a][k] z-block k
template <int NX, int NZ>
inline void map_to_vertices(const int (&C)[NX][NZ], const double* gz, const double* Hz, double* gx, double* Hx) {
    const int nz = 3 * NZ, nx = 3 * NX;
    for (int a = 0; a < NX; ++a)
        for (int d = 0; d < 3; ++d) {
            double s = 0;
            for (int k = 0; k < NZ; ++k) s += C[a][k] * gz[3 * k + d];
            gx[3 * a + d] = s;
        }
    if (!Hx) return;
    for (int a = 0; a < NX; ++a)
        for (int b = 0; b < NX; ++b)
            for (int di = 0; di < 3; ++di)
                for (int dj = 0; dj < 3; ++dj) {
                    double s = 0;
                    for (int k = 0; k < NZ; ++k) {
                        if (!C[a][k]) continue;
                        for (int l = 0; l < NZ; ++l) {
                            if (!C[b][l]) continue;
                            s += C[a][k] * C[b][l] * Hz[(3 * k + di) * nz + 3 * l + dj];
                        }
                    }
                    Hx[(3 * a + di) * nx + 3 * b + dj] = s;
                }
}

// d = s^2/D with s = w.(u x v), D = |u x v|^2, in z = (w, u, v)
inline void triple_ratio_derivs(V3 w, V3 u, V3 v, double* gz, double* Hz) {
    V3 n = cross(u, v);
    double s = dot(w, n), D = sq(n);
    double gs[9], gD[9] = {0, 0, 0};
    V3 gsw = n, gsu = cross(v, w), gsv = cross(w, u);
    double tmp[9] = {gsw.x, gsw.y, gsw.z, gsu.x, gsu.y, gsu.z, gsv.x, gsv.y, gsv.z};
    for (int i = 0; i < 9; ++i) gs[i] = tmp[i];
    double gDuv[6], HDuv[36];
    crossnorm2_derivs(u, v, gDuv, HDuv);
    for (int i = 0; i < 6; ++i) gD[3 + i] = gDuv[i];
    double c1 = 2.0 * s / D, c2 = s * s / (D * D);
    for (int i = 0; i < 9; ++i) gz[i] = c1 * gs[i] - c2 * gD[i];
    if (!Hz) return;
    double Hs[81] = {0}, HD[81] = {0};
    double Ew[9], Eu[9], Ev[9];
    eps_mat(w, Ew); eps_mat(u, Eu); eps_mat(v, Ev);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            Hs[(0 + i) * 9 + 3 + j] = Ev[i * 3 + j];  // d2s/dw du
            Hs[(3 + j) * 9 + 0 + i] = Ev[i * 3 + j];
            Hs[(3 + i) * 9 + 6 + j] = Ew[i * 3 + j];  // d2s/du dv
            Hs[(6 + j) * 9 + 3 + i] = Ew[i * 3 + j];
            Hs[(6 + i) * 9 + 0 + j] = Eu[i * 3 + j];  // d2s/dv dw
            Hs[(0 + j) * 9 + 6 + i] = Eu[i * 3 + j];
        }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) HD[(3 + i) * 9 + 3 + j] = HDuv[i * 6 + j];
    double a1 = 2.0 / D, a3 = 2.0 * s / (D * D), a4 = 2.0 * s * s / (D * D * D);
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j)
            Hz[i * 9 + j] = a1 * gs[i] * gs[j] + c1 * Hs[i * 9 + j] - a3 * (gs[i] * gD[j] + gD[i] * gs[j]) +
                            a4 * gD[i] * gD[j] - c2 * HD[i * 9 + j];
}

// ---- public derivative functions (vertex space) ----
inline void dPP_grad_hess(V3 a, V3 b, double* g, double* H) {
    V3 d = a - b;
    double da[3] = {d.x, d.y, d.z};
    for (int i = 0; i < 3; ++i) { g[i] = 2.0 * da[i]; g[3 + i] = -2.0 * da[i]; }
    if (!H) return;
    for (int i = 0; i < 36; ++i) H[i] = 0;
    for (int i = 0; i < 3; ++i) {
        H[i * 6 + i] = 2; H[(3 + i) * 6 + 3 + i] = 2;
        H[i * 6 + 3 + i] = -2; H[(3 + i) * 6 + i] = -2;
    }
}

inline void dPE_grad_hess(V3 p, V3 e0, V3 e1, double* g, double* H) {
    V3 a = e0 - p, b = e1 - p;
    double gN[6], HN[36];
    crossnorm2_derivs(a, b, gN, HN);
    double N = sq(cross(a, b));
    V3 ba = b - a;
    double Q = sq(ba);
    double bav[3] = {ba.x, ba.y, ba.z};
    double gQ[6];
    for (int i = 0; i < 3; ++i) { gQ[i] = -2.0 * bav[i]; gQ[3 + i] = 2.0 * bav[i]; }
    double gz[6], Hz[36];
    for (int i = 0; i < 6; ++i) gz[i] = gN[i] / Q - N * gQ[i] / (Q * Q);
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            int bi = i / 3, bj = j / 3;
            double HQ = (i % 3 == j % 3) ? (bi == bj ? 2.0 : -2.0) : 0.0;
            Hz[i * 6 + j] = HN[i * 6 + j] / Q - (gN[i] * gQ[j] + gQ[i] * gN[j]) / (Q * Q) +
                            2.0 * N * gQ[i] * gQ[j] / (Q * Q * Q) - N * HQ / (Q * Q);
        }
    static const int C[3][2] = {{-1, -1}, {1, 0}, {0, 1}};
    map_to_vertices<3, 2>(C, gz, H ? Hz : nullptr, g, H);
}

inline void dPT_grad_hess(V3 p, V3 t0, V3 t1, V3 t2, double* g, double* H) {
    double gz[9], Hz[81];
    triple_ratio_derivs(p - t0, t1 - t0, t2 - t0, gz, H ? Hz : nullptr);
    static const int C[4][3] = {{1, 0, 0}, {-1, -1, -1}, {0, 1, 0}, {0, 0, 1}};
    map_to_vertices<4, 3>(C, gz, H ? Hz : nullptr, g, H);
}

inline void dEE_grad_hess(V3 ea0, V3 ea1, V3 eb0, V3 eb1, double* g, double* H) {
    double gz[9], Hz[81];
    triple_ratio_derivs(eb0 - ea0, ea1 - ea0, eb1 - eb0, gz, H ? Hz : nullptr);
    static const int C[4][3] = {{-1, -1, 0}, {0, 1, 0}, {1, 0, -1}, {0, 0, 1}};
    map_to_vertices<4, 3>(C, gz, H ? Hz : nullptr, g, H);
}

inline void eecn2_grad_hess(V3 ea0, V3 ea1, V3 eb0, V3 eb1, double* g, double* H) {
    double gz[6], Hz[36];
    crossnorm2_derivs(ea1 - ea0, eb1 - eb0, gz, Hz);
    static const int C[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
    map_to_vertices<4, 2>(C, gz, H ? Hz : nullptr, g, H);
}

// mollifier e(c) gradient/Hessian in vertex space (EDGE_EDGE_MOLLIFIER.h:478-524)
inline void mollifier_grad_hess(V3 ea0, V3 ea1, V3 eb0, V3 eb1, double eps_x, double* g, double* H) {
    double c = ee_cross_norm2(ea0, ea1, eb0, eb1);
    if (!(c < eps_x)) {
        for (int i = 0; i < 12; ++i) g[i] = 0;
        if (H) for (int i = 0; i < 144; ++i) H[i] = 0;
        return;
    }
    double gc[12], Hc[144];
    eecn2_grad_hess(ea0, ea1, eb0, eb1, gc, H ? Hc : nullptr);
    double one_div = 1.0 / eps_x;
    double q_g = 2.0 * one_div * (-one_div * c + 1.0);
    double q_H = -2.0 / (eps_x * eps_x);
    for (int i = 0; i < 12; ++i) g[i] = q_g * gc[i];
    if (!H) return;
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) H[i * 12 + j] = q_g * Hc[i * 12 + j] + q_H * gc[i] * gc[j];
}

}  // namespace ora
