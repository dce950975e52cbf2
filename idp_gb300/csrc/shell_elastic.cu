// Discrete-shell elasticity of the Hinge path (Advance_One_Step_IE_Hinge,
// FEM/Shell/DISCRETE_SHELL.h:1110, KL = false) on elastic shell instances:
//   * neo-Hookean membrane on the first fundamental form A of every face
//     (FEM/Shell/MEMBRANE.h:7-322): h^2 vol (mu/2 (tr(IB^-1 A) - 2 - 2 lnJ)
//     + lam/2 lnJ^2), lnJ = ln(det A det IB^-1) / 2;
//   * hinge bending on the dihedral angle of every interior edge
//     (FEM/Shell/BENDING.h:52-76,176-211,430-485): h^2 k (theta - thetabar)^2
//     ebar / hbar, with the angle's gradient and Hessian in the form of
//     Tamstorf & Grinspun that the reference's Math/DIHEDRAL_ANGLE.h
//     writes out.
// Elements whose vertices are all fixed (DBC) are skipped, as in the
// reference. Energies per element are summed per chunk in a fixed tree and
// chunk sums per instance in order; gradients go to per-element slots that a
// per-vertex gather sums in a fixed order; element Hessians are evaluated in
// FP64, rounded to the working precision, projected to PSD (makePD, one
// warp per matrix) and stored as upper 3x3 blocks after the tets' blocks,
// where the BSR assembly gathers them.
#include "engine.hpp"
#include "psd.cuh"

namespace idp {
namespace {

struct D3s {
    double x, y, z;
};
__device__ __forceinline__ D3s ld(const double* X, int v) { return {X[3 * v], X[3 * v + 1], X[3 * v + 2]}; }
__device__ __forceinline__ D3s sub(D3s a, D3s b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3s add(D3s a, D3s b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3s scl(double s, D3s a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dt(D3s a, D3s b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3s crs(D3s a, D3s b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double comp(D3s a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

__device__ double block_sum_shell(double v) {
    __shared__ double sh[kBlock];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int st = kBlock / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    double r = sh[0];
    __syncthreads();
    return r;
}

// ---- membrane of one face; mem = (IB^-1 00, 01, 11, det IB^-1, vol, lam, mu)
__device__ double membrane_face(D3s x1, D3s x2, D3s x3, const double* m, double w, double* g, double* H) {
    const D3s e01 = sub(x2, x1), e02 = sub(x3, x1);
    const double a00 = dt(e01, e01), a01 = dt(e01, e02), a11 = dt(e02, e02);
    const double detA = a00 * a11 - a01 * a01;
    const double lnJ = log(detA * m[3]) / 2;
    const double trIA = m[0] * a00 + 2.0 * m[1] * a01 + m[2] * a11;
    const double vol = m[4], lam = m[5], mu = m[6];
    const double E = w * vol * (mu / 2 * (trIA - 2 - 2 * lnJ) + lam / 2 * lnJ * lnJ);
    if (!g && !H) return E;
    // dA/dx rows (A00, A10, A01, A11) x (x1, x2, x3) (MEMBRANE.h:87-97)
    double dA[4][9];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 9; ++c) dA[r][c] = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double a = comp(e01, d), b = comp(e02, d);
        dA[0][3 + d] += 2.0 * a;
        dA[0][d] -= 2.0 * a;
        for (int r = 1; r <= 2; ++r) {
            dA[r][6 + d] += a;
            dA[r][3 + d] += b;
            dA[r][d] += -a - b;
        }
        dA[3][6 + d] += 2.0 * b;
        dA[3][d] -= 2.0 * b;
    }
    const double IA[4] = {a11 / detA, -a01 / detA, -a01 / detA, a00 / detA};
    const double IB[4] = {m[0], m[1], m[1], m[2]};
    const double term1 = (-mu + lam * lnJ) / 2;
    if (g) {
        double temp[4];
        for (int r = 0; r < 4; ++r) temp[r] = w * vol * (mu / 2 * IB[r] + term1 * IA[r]);
        for (int i = 0; i < 9; ++i) g[i] = dA[0][i] * temp[0] + dA[1][i] * temp[1] + dA[2][i] * temp[2] + dA[3][i] * temp[3];
    }
    if (H) {
        double ainvda[9];
        for (int i = 0; i < 9; ++i)
            ainvda[i] = dA[0][i] * IA[0] + dA[1][i] * IA[1] + dA[2][i] * IA[2] + dA[3][i] * IA[3];
        const double c0 = -term1 + lam / 4, c1 = term1 / detA;
        for (int i = 0; i < 9; ++i)
            for (int j = 0; j < 9; ++j) {
                const double t = dA[3][i] * dA[0][j] - dA[1][i] * dA[1][j] - dA[2][i] * dA[2][j] + dA[0][i] * dA[3][j];
                H[i * 9 + j] = c0 * ainvda[i] * ainvda[j] + c1 * t;
            }
        // constant second derivatives of A (MEMBRANE.h:140-170)
        for (int r = 0; r < 4; ++r) {
            const double c = term1 * IA[r] + mu / 2 * IB[r];
            for (int d = 0; d < 3; ++d) {
                if (r == 0) {
                    H[(0 + d) * 9 + 0 + d] += 2 * c; H[(3 + d) * 9 + 3 + d] += 2 * c;
                    H[(0 + d) * 9 + 3 + d] -= 2 * c; H[(3 + d) * 9 + 0 + d] -= 2 * c;
                } else if (r == 3) {
                    H[(0 + d) * 9 + 0 + d] += 2 * c; H[(6 + d) * 9 + 6 + d] += 2 * c;
                    H[(0 + d) * 9 + 6 + d] -= 2 * c; H[(6 + d) * 9 + 0 + d] -= 2 * c;
                } else {
                    H[(3 + d) * 9 + 6 + d] += c; H[(6 + d) * 9 + 3 + d] += c;
                    H[(0 + d) * 9 + 3 + d] -= c; H[(0 + d) * 9 + 6 + d] -= c;
                    H[(3 + d) * 9 + 0 + d] -= c; H[(6 + d) * 9 + 0 + d] -= c;
                    H[(0 + d) * 9 + 0 + d] += 2 * c;
                }
            }
        }
        for (int i = 0; i < 81; ++i) H[i] *= w * vol;
    }
    return E;
}

// ---- dihedral angle of hinge (x0, x1, x2, x3), hinge edge x1-x2
// (DIHEDRAL_ANGLE.h:10-24)
__device__ double dihedral_angle(D3s x0, D3s x1, D3s x2, D3s x3) {
    const D3s n1 = crs(sub(x1, x0), sub(x2, x0)), n2 = crs(sub(x2, x3), sub(x1, x3));
    double c = dt(n1, n2) / sqrt(dt(n1, n1) * dt(n2, n2));
    c = fmax(-1.0, fmin(1.0, c));
    double t = acos(c);
    if (dt(crs(n2, n1), sub(x1, x2)) < 0) t = -t;
    return t;
}

__device__ __forceinline__ D3s unitv(D3s a) { return scl(1.0 / sqrt(dt(a, a)), a); }
__device__ __forceinline__ D3s mhat(D3s xp, D3s xe0, D3s xe1) {
    const D3s e = sub(xe1, xe0);
    return unitv(sub(add(xe0, scl(dt(sub(xp, xe0), e) / dt(e, e), e)), xp));
}
// s a b^T into M (3x3, row-major)
__device__ __forceinline__ void outer(D3s a, D3s b, double s, double* M) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[i * 3 + j] = s * comp(a, i) * comp(b, j);
}

// gradient (12) and Hessian (144) of the dihedral angle, the stencil's
// x0, x1, x2, x3 in the roles v2, v0, v1, v3 of the hinge formulas
// (DIHEDRAL_ANGLE.h:1190-1277)
__device__ void dihedral_derivs(D3s x0, D3s x1, D3s x2, D3s x3, double* g, double* H) {
    const D3s v2 = x0, v0 = x1, v1 = x2, v3 = x3;
    const D3s e[5] = {sub(v1, v0), sub(v2, v0), sub(v3, v0), sub(v2, v1), sub(v3, v1)};
    double ne[5];
    for (int i = 0; i < 5; ++i) ne[i] = sqrt(dt(e[i], e[i]));
    const D3s n1 = crs(e[0], e[1]), n2 = crs(e[2], e[0]);
    const double n1n = sqrt(dt(n1, n1)), n2n = sqrt(dt(n2, n2));
    const double ca1 = dt(e[0], e[1]) / (ne[0] * ne[1]);
    const double ca2 = dt(e[0], e[2]) / (ne[0] * ne[2]);
    const double ca3 = -dt(e[0], e[3]) / (ne[0] * ne[3]);
    const double ca4 = -dt(e[0], e[4]) / (ne[0] * ne[4]);
    const double h1 = n1n / ne[1], h2 = n2n / ne[2], h3 = n1n / ne[3], h4 = n2n / ne[4];
    const double h01 = n1n / ne[0], h02 = n2n / ne[0];
    if (g) {
        const D3s u1 = scl(1.0 / n1n, n1), u2 = scl(1.0 / n2n, n2);
        const D3s gg[4] = {scl(-1.0 / h01, u1), add(scl(ca3 / h3, u1), scl(ca4 / h4, u2)),
                           add(scl(ca1 / h1, u1), scl(ca2 / h2, u2)), scl(-1.0 / h02, u2)};
        for (int k = 0; k < 4; ++k) {
            g[3 * k] = gg[k].x;
            g[3 * k + 1] = gg[k].y;
            g[3 * k + 2] = gg[k].z;
        }
    }
    if (!H) return;
    const D3s m1 = mhat(v1, v0, v2), m2 = mhat(v1, v0, v3), m3 = mhat(v0, v1, v2), m4 = mhat(v0, v1, v3);
    const D3s m01 = mhat(v2, v0, v1), m02 = mhat(v3, v0, v1);
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
    for (int i = 0; i < 144; ++i) H[i] = 0.0;
#define PUT(bi, bj, i, j, v) H[(3 * (bi) + (i)) * 12 + 3 * (bj) + (j)] = (v)
#define TR(M, i, j) ((M)[(j) * 3 + (i)])
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int k = i * 3 + j;
            PUT(0, 0, i, j, -(N1_01[k] + TR(N1_01, i, j)));
            const double b10 = M3_01_1[k] - N1_3[k], b20 = M1_01_1[k] - N1_1[k];
            PUT(1, 0, i, j, b10);
            PUT(0, 1, j, i, b10);
            PUT(2, 0, i, j, b20);
            PUT(0, 2, j, i, b20);
            PUT(1, 1, i, j, M3_3_1[k] + TR(M3_3_1, i, j) - B1[k] + M4_4_2[k] + TR(M4_4_2, i, j) - B2[k]);
            const double b12 = M3_1_1[k] + TR(M1_3_1, i, j) + B1[k] + M4_2_2[k] + TR(M2_4_2, i, j) + B2[k];
            PUT(1, 2, i, j, b12);
            PUT(2, 1, j, i, b12);
            const double b13 = M4_02_2[k] - N2_4[k], b23 = M2_02_2[k] - N2_2[k];
            PUT(1, 3, i, j, b13);
            PUT(3, 1, j, i, b13);
            PUT(2, 2, i, j, M1_1_1[k] + TR(M1_1_1, i, j) - B1[k] + M2_2_2[k] + TR(M2_2_2, i, j) - B2[k]);
            PUT(2, 3, i, j, b23);
            PUT(3, 2, j, i, b23);
            PUT(3, 3, i, j, -(N2_02[k] + TR(N2_02, i, j)));
        }
#undef PUT
#undef TR
}

// ---- hinge bending; hk = (thetabar, k ebar / hbar)
__device__ double bending_hinge(D3s x0, D3s x1, D3s x2, D3s x3, const double* hk, double w, double* g, double* H) {
    const double th = dihedral_angle(x0, x1, x2, x3);
    const double E = w * hk[1] * (th - hk[0]) * (th - hk[0]);
    if (!g && !H) return E;
    double dg[12];
    dihedral_derivs(x0, x1, x2, x3, dg, H);
    const double cg = w * hk[1] * 2 * (th - hk[0]);
    if (g)
        for (int i = 0; i < 12; ++i) g[i] = cg * dg[i];
    if (H) {
        const double cq = w * hk[1] * 2;
        for (int i = 0; i < 12; ++i)
            for (int j = 0; j < 12; ++j) H[i * 12 + j] = cg * H[i * 12 + j] + (cq * dg[i]) * dg[j];
    }
    return E;
}

__device__ __forceinline__ bool all_fixed(const unsigned char* dbc, const int* v, int n) {
    for (int k = 0; k < n; ++k)
        if (!dbc[v[k]]) return false;
    return true;
}

__global__ void k_membrane_energy(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                                  const double* __restrict__ X, const int* __restrict__ mface,
                                  const double* __restrict__ mem, const unsigned char* __restrict__ dbc, double w,
                                  double* __restrict__ part) {
    const Chunk c = chunks[blockIdx.x];
    double acc = 0.0;
    if (active[c.inst])
        for (int f = c.begin + threadIdx.x; f < c.end; f += blockDim.x) {
            const int* t = mface + 3L * f;
            if (all_fixed(dbc, t, 3)) continue;
            acc += membrane_face(ld(X, t[0]), ld(X, t[1]), ld(X, t[2]), mem + 7L * f, w, nullptr, nullptr);
        }
    const double s = block_sum_shell(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_bending_energy(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                                 const double* __restrict__ X, const int4* __restrict__ hinge,
                                 const double* __restrict__ hk, const unsigned char* __restrict__ dbc, double w,
                                 double* __restrict__ part) {
    const Chunk c = chunks[blockIdx.x];
    double acc = 0.0;
    if (active[c.inst])
        for (int i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
            const int4 hh = hinge[i];
            const int v[4] = {hh.x, hh.y, hh.z, hh.w};
            if (all_fixed(dbc, v, 4)) continue;
            acc += bending_hinge(ld(X, v[0]), ld(X, v[1]), ld(X, v[2]), ld(X, v[3]), hk + 2L * i, w, nullptr, nullptr);
        }
    const double s = block_sum_shell(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// element gradients: face f at slots 3f..3f+2, hinge i at 3 Fm + 4i ..
__global__ void k_membrane_grad(long Fm, const int* __restrict__ finst, const unsigned char* __restrict__ active,
                                const double* __restrict__ X, const int* __restrict__ mface,
                                const double* __restrict__ mem, const unsigned char* __restrict__ dbc, double w,
                                double* __restrict__ gout) {
    const long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= Fm || !active[finst[f]]) return;
    const int* t = mface + 3 * f;
    double g[9];
    if (all_fixed(dbc, t, 3))
        for (int i = 0; i < 9; ++i) g[i] = 0.0;
    else
        membrane_face(ld(X, t[0]), ld(X, t[1]), ld(X, t[2]), mem + 7 * f, w, g, nullptr);
    for (int i = 0; i < 9; ++i) gout[9 * f + i] = g[i];
}

__global__ void k_bending_grad(long Hn, long Fm, const int* __restrict__ hinst, const unsigned char* __restrict__ active,
                               const double* __restrict__ X, const int4* __restrict__ hinge,
                               const double* __restrict__ hk, const unsigned char* __restrict__ dbc, double w,
                               double* __restrict__ gout) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Hn || !active[hinst[i]]) return;
    const int4 hh = hinge[i];
    const int v[4] = {hh.x, hh.y, hh.z, hh.w};
    double g[12];
    if (all_fixed(dbc, v, 4))
        for (int q = 0; q < 12; ++q) g[q] = 0.0;
    else
        bending_hinge(ld(X, v[0]), ld(X, v[1]), ld(X, v[2]), ld(X, v[3]), hk + 2 * i, w, g, nullptr);
    double* o = gout + 9 * Fm + 12 * i;
    for (int q = 0; q < 12; ++q) o[q] = g[q];
}

// per vertex: its element slots (faces ascending, then hinges ascending)
__global__ void k_grad_gather_shell(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                                    const int* __restrict__ vsp, const int* __restrict__ vs,
                                    const double* __restrict__ gel, double* __restrict__ g) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    const int k0 = vsp[v], k1 = vsp[v + 1];
    if (k0 == k1) return;
    double s0 = 0, s1 = 0, s2 = 0;
    for (int k = k0; k < k1; ++k) {
        const double* p = gel + 3L * vs[k];
        s0 += p[0];
        s1 += p[1];
        s2 += p[2];
    }
    g[3 * v] += s0;
    g[3 * v + 1] += s1;
    g[3 * v + 2] += s2;
}

// the upper 3x3 blocks (a <= b) of an nv-vertex element's 3nv x 3nv matrix
template <class S, class T>
__device__ __forceinline__ void store_blocks(const S* H, int nv, T* ho) {
    const int n = 3 * nv;
    int k = 0;
    for (int a = 0; a < nv; ++a)
        for (int b = a; b < nv; ++b, ++k)
            for (int d = 0; d < 3; ++d)
                for (int e = 0; e < 3; ++e) ho[k * 9 + d * 3 + e] = (T)H[(3 * a + d) * n + 3 * b + e];
}

// blocks of shell element e: faces e < Fm (6 blocks at 54 e), then hinges
// (10 blocks at 54 Fm + 90 (e - Fm))
__device__ __forceinline__ long shell_block_off(long e, long Fm) { return e < Fm ? 54 * e : 54 * Fm + 90 * (e - Fm); }

// an element Hessian (n x n, FP64) in the working precision T: stored as it
// is when the Cholesky test finds it positive definite, else queued for the
// warp projection (an element Hessian is singular along its rigid motions,
// so nearly all are queued)
template <class T>
__device__ void shell_element_out(const double* H, int n, long e, long Fm, T* __restrict__ hout,
                                  T* __restrict__ hloc, int* __restrict__ hn, int* __restrict__ plist,
                                  unsigned int* __restrict__ pcount) {
    T Ht[144];
    for (int k = 0; k < n * n; ++k) Ht[k] = (T)H[k];
    if (chol_pd(Ht, n)) {
        store_blocks(Ht, n / 3, hout + shell_block_off(e, Fm));
        return;
    }
    T* hl = hloc + 144 * e;
    for (int k = 0; k < n * n; ++k) hl[k] = Ht[k];
    hn[e] = n;
    plist[atomicAdd(pcount, 1u)] = (int)e;
}

template <class T>
__global__ void k_membrane_hess(long Fm, const int* __restrict__ finst, const unsigned char* __restrict__ active,
                                const double* __restrict__ X, const int* __restrict__ mface,
                                const double* __restrict__ mem, const unsigned char* __restrict__ dbc, double w,
                                T* __restrict__ hout, T* __restrict__ hloc, int* __restrict__ hn,
                                int* __restrict__ plist, unsigned int* __restrict__ pcount) {
    const long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= Fm || !active[finst[f]]) return;
    const int* t = mface + 3 * f;
    if (all_fixed(dbc, t, 3)) {
        for (int k = 0; k < 54; ++k) hout[54 * f + k] = T(0);
        return;
    }
    double H[81];
    membrane_face(ld(X, t[0]), ld(X, t[1]), ld(X, t[2]), mem + 7 * f, w, nullptr, H);
    shell_element_out(H, 9, f, Fm, hout, hloc, hn, plist, pcount);
}

template <class T>
__global__ void k_bending_hess(long Hn, long Fm, const int* __restrict__ hinst, const unsigned char* __restrict__ active,
                               const double* __restrict__ X, const int4* __restrict__ hinge,
                               const double* __restrict__ hk, const unsigned char* __restrict__ dbc, double w,
                               T* __restrict__ hout, T* __restrict__ hloc, int* __restrict__ hn,
                               int* __restrict__ plist, unsigned int* __restrict__ pcount) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Hn || !active[hinst[i]]) return;
    const int4 hh = hinge[i];
    const int v[4] = {hh.x, hh.y, hh.z, hh.w};
    if (all_fixed(dbc, v, 4)) {
        for (int q = 0; q < 90; ++q) hout[54 * Fm + 90 * i + q] = T(0);
        return;
    }
    double H[144];
    bending_hinge(ld(X, v[0]), ld(X, v[1]), ld(X, v[2]), ld(X, v[3]), hk + 2 * i, w, nullptr, H);
    shell_element_out(H, 12, Fm + i, Fm, hout, hloc, hn, plist, pcount);
}

// makePD of the queued element Hessians, one warp per matrix
// (psd_warp_project), written to the element's blocks
template <class T>
__global__ void __launch_bounds__(32 * kPsdWarps) k_shell_psd_warp(const int* __restrict__ plist,
                                                                     const unsigned int* __restrict__ pcount,
                                                                     const T* __restrict__ hloc,
                                                                     const int* __restrict__ hn, long Fm,
                                                                     T* __restrict__ hout) {
    __shared__ T sA[kPsdWarps][144], sV[kPsdWarps][144], sCS[kPsdWarps][6][2], sW[kPsdWarps][12];
    __shared__ int sPQ[kPsdWarps][6][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* A = sA[w];
    T* Vm = sV[w];
    const unsigned int cnt = *pcount;
    for (unsigned int item = blockIdx.x * kPsdWarps + w; item < cnt; item += gridDim.x * kPsdWarps) {
        const long e = plist[item];
        const int n = hn[e];
        for (int k = lane; k < n * n; k += 32) {
            A[k] = hloc[144 * e + k];
            Vm[k] = (k / n == k % n) ? T(1) : T(0);
        }
        __syncwarp();
        psd_warp_project(A, Vm, n, sCS[w], sPQ[w], sW[w], lane);
        const int nv = n / 3, nb = nv * (nv + 1) / 2;
        T* ho = hout + shell_block_off(e, Fm);
        for (int t = lane; t < 9 * nb; t += 32) {
            const int blk = t / 9, d = (t % 9) / 3, c = t % 3;
            int a = 0, b = 0, kk = blk;
            for (a = 0; a < nv; ++a) {
                if (kk < nv - a) {
                    b = a + kk;
                    break;
                }
                kk -= nv - a;
            }
            ho[t] = A[(3 * a + d) * n + 3 * b + c];
        }
        __syncwarp();
    }
}

}  // namespace

int shell_energy(Arena& A, Work& W, const double* X, double w_h2, double* inst_E, cudaStream_t s) {
    if (A.Fm == 0 && A.Hn == 0) return IDP_OK;
    if (W[W_CHUNK_SUM].ensure(sizeof(double) *
                              (A.n_mface_chunks + A.n_hinge_chunks + A.n_face_chunks + A.n_tet_chunks + A.n_vert_chunks + 2)))
        return IDP_ERR_CUDA;
    double* part = W[W_CHUNK_SUM].as<double>();
    int rc = IDP_OK;
    if (A.Fm) {
        (::idp::count_launch(), k_membrane_energy<<<A.n_mface_chunks, kBlock, 0, s>>>(A.mface_chunks, A.active, X, A.mface,
                                                                                      A.mem, A.dbc_excl, w_h2, part));
        rc = chunk_reduce_off(A, A.mface_chunk_off, part, inst_E, true, s);
        if (rc) return rc;
    }
    if (A.Hn) {
        (::idp::count_launch(), k_bending_energy<<<A.n_hinge_chunks, kBlock, 0, s>>>(A.hinge_chunks, A.active, X, A.hinge,
                                                                                     A.hk, A.dbc_excl, w_h2, part));
        rc = chunk_reduce_off(A, A.hinge_chunk_off, part, inst_E, true, s);
    }
    return rc;
}

int shell_gradient(Arena& A, Work& W, const double* X, double w_h2, double* g, cudaStream_t s) {
    if (A.Fm == 0 && A.Hn == 0) return IDP_OK;
    if (W[W_SHELL_GRAD].ensure(sizeof(double) * (9 * A.Fm + 12 * A.Hn + 12))) return IDP_ERR_CUDA;
    double* gel = W[W_SHELL_GRAD].as<double>();
    if (A.Fm)
        (::idp::count_launch(), k_membrane_grad<<<grid_for(A.Fm), kBlock, 0, s>>>(A.Fm, A.finst, A.active, X, A.mface,
                                                                                   A.mem, A.dbc_excl, w_h2, gel));
    if (A.Hn)
        (::idp::count_launch(), k_bending_grad<<<grid_for(A.Hn), kBlock, 0, s>>>(A.Hn, A.Fm, A.hinst, A.active, X, A.hinge,
                                                                                  A.hk, A.dbc_excl, w_h2, gel));
    (::idp::count_launch(), k_grad_gather_shell<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.vshell_ptr,
                                                                                 A.vshell, gel, g));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

// element blocks after the tets' (10 per tet): 6 per face, 10 per hinge
template <class T>
static int shell_hessian_t(Arena& A, Work& W, const double* X, double w_h2, T* base, cudaStream_t s) {
    // PSD queue: local matrices (144 per element) | sizes | list | count
    const long Ne = A.Fm + A.Hn;
    const size_t o_n = ((sizeof(T) * 144 * (size_t)Ne) + 255) & ~size_t(255);
    const size_t o_l = o_n + ((sizeof(int) * (size_t)Ne + 255) & ~size_t(255));
    const size_t o_c = o_l + ((sizeof(int) * (size_t)Ne + 255) & ~size_t(255));
    if (W[W_SHELL_PSD].ensure(o_c + 256)) return IDP_ERR_CUDA;
    char* pb = W[W_SHELL_PSD].as<char>();
    T* hloc = reinterpret_cast<T*>(pb);
    int* hn = reinterpret_cast<int*>(pb + o_n);
    int* plist = reinterpret_cast<int*>(pb + o_l);
    unsigned int* pcount = reinterpret_cast<unsigned int*>(pb + o_c);
    IDP_CUDA_TRY(cudaMemsetAsync(pcount, 0, sizeof(unsigned int), s));
    if (A.Fm)
        (::idp::count_launch(), k_membrane_hess<T><<<grid_for(A.Fm, 64), 64, 0, s>>>(
                                    A.Fm, A.finst, A.active, X, A.mface, A.mem, A.dbc_excl, w_h2, base, hloc, hn, plist,
                                    pcount));
    if (A.Hn)
        (::idp::count_launch(), k_bending_hess<T><<<grid_for(A.Hn, 64), 64, 0, s>>>(
                                    A.Hn, A.Fm, A.hinst, A.active, X, A.hinge, A.hk, A.dbc_excl, w_h2, base, hloc, hn,
                                    plist, pcount));
    const int pgrid = (int)std::min<long>((Ne + kPsdWarps - 1) / kPsdWarps, 8L * 152);
    (::idp::count_launch(), k_shell_psd_warp<T><<<pgrid, 32 * kPsdWarps, 0, s>>>(plist, pcount, hloc, hn, A.Fm, base));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int shell_hessian(Arena& A, Work& W, const double* X, double w_h2, bool fp64, cudaStream_t s) {
    if (A.Fm == 0 && A.Hn == 0) return IDP_OK;
    const size_t el = fp64 ? sizeof(double) : sizeof(float);
    if (W[W_TET_HESS].ensure(el * 9 * (10 * (A.T + 1) + 6 * A.Fm + 10 * A.Hn))) return IDP_ERR_CUDA;
    if (fp64) return shell_hessian_t(A, W, X, w_h2, W[W_TET_HESS].as<double>() + 90 * A.T, s);
    return shell_hessian_t(A, W, X, w_h2, W[W_TET_HESS].as<float>() + 90 * A.T, s);
}

}  // namespace idp
