// IPC log-barrier kernels over the constraint set: energy (FP64), gradient
// (FP64) and the PSD-projected local Hessian (FP32 in mixed mode, FP64 in the
// plain path), plus the deterministic scatter of local gradients into g and
// of local Hessian blocks into the contact tail of the system matrix.
//
// Reference: Compute_Barrier (FEM/IPC.h:742-941), Compute_Barrier_Gradient
// (IPC.h:943-1256), Compute_Barrier_Hessian (IPC.h:1258-1731) with makePD
// (Math/UTILS.h:10-27), mollifier (Math/Distance/EDGE_EDGE_MOLLIFIER.h).
// Distance derivatives are derived here by the chain rule
// (PT, EE: d = s^2/D, s = w.(u x v), D = |u x v|^2; PE: d = |a x b|^2/|b-a|^2).
#include "engine.hpp"
#include "geom.cuh"
#include "prims.cuh"
#include "psd.cuh"

namespace idp {

using namespace geo;

namespace {

// ---------------------------------------------------------------- derivatives
__device__ __forceinline__ void eps_mat(D3 v, double E[9]) {
    E[0] = 0;     E[1] = v.z;   E[2] = -v.y;
    E[3] = -v.z;  E[4] = 0;     E[5] = v.x;
    E[6] = v.y;   E[7] = -v.x;  E[8] = 0;
}

// D = |u x v|^2 in (u, v): g (6), H (6x6)
__device__ void crossnorm2_d(D3 u, D3 v, double g[6], double H[36]) {
    double uu = dot(u, u), vv = dot(v, v), uv = dot(u, v);
    double ua[3] = {u.x, u.y, u.z}, va[3] = {v.x, v.y, v.z};
    for (int i = 0; i < 3; ++i) {
        g[i] = 2.0 * (vv * ua[i] - uv * va[i]);
        g[3 + i] = 2.0 * (uu * va[i] - uv * ua[i]);
    }
    if (!H) return;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double dij = (i == j) ? 1.0 : 0.0;
            H[i * 6 + j] = 2.0 * (vv * dij - va[i] * va[j]);
            H[(3 + i) * 6 + 3 + j] = 2.0 * (uu * dij - ua[i] * ua[j]);
            double c = 2.0 * (2.0 * ua[i] * va[j] - va[i] * ua[j] - uv * dij);
            H[i * 6 + 3 + j] = c;
            H[(3 + j) * 6 + i] = c;
        }
}

// maps z-space (NZ blocks of 3) derivatives to NX vertex blocks through the
// constant +-1 coefficients C (row-major NX x NZ); output dims 3*NX
template <int NX, int NZ>
__device__ void to_vertices(const signed char* C, const double* gz, const double* Hz, double* gx, double* Hx) {
    for (int a = 0; a < NX; ++a)
        for (int d = 0; d < 3; ++d) {
            double s = 0;
            for (int k = 0; k < NZ; ++k) s += C[a * NZ + k] * gz[3 * k + d];
            gx[3 * a + d] = s;
        }
    if (!Hx) return;
    const int nz = 3 * NZ, nx = 3 * NX;
    for (int a = 0; a < NX; ++a)
        for (int b = 0; b < NX; ++b)
            for (int di = 0; di < 3; ++di)
                for (int dj = 0; dj < 3; ++dj) {
                    double s = 0;
                    for (int k = 0; k < NZ; ++k) {
                        int ca = C[a * NZ + k];
                        if (!ca) continue;
                        for (int l = 0; l < NZ; ++l) {
                            int cb = C[b * NZ + l];
                            if (!cb) continue;
                            s += ca * cb * Hz[(3 * k + di) * nz + 3 * l + dj];
                        }
                    }
                    Hx[(3 * a + di) * nx + 3 * b + dj] = s;
                }
}

// d = s^2 / D, s = w.(u x v), D = |u x v|^2 ; z = (w, u, v)
__device__ void triple_ratio_d(D3 w, D3 u, D3 v, double gz[9], double* Hz) {
    D3 n = cross(u, v);
    double s = dot(w, n), D = sqn(n);
    D3 gsu = cross(v, w), gsv = cross(w, u);
    double gs[9] = {n.x, n.y, n.z, gsu.x, gsu.y, gsu.z, gsv.x, gsv.y, gsv.z};
    double gD[9], HDuv[36], gDuv[6];
    crossnorm2_d(u, v, gDuv, Hz ? HDuv : nullptr);
    gD[0] = gD[1] = gD[2] = 0;
    for (int i = 0; i < 6; ++i) gD[3 + i] = gDuv[i];
    double c1 = 2.0 * s / D, c2 = s * s / (D * D);
    for (int i = 0; i < 9; ++i) gz[i] = c1 * gs[i] - c2 * gD[i];
    if (!Hz) return;
    double Ew[9], Eu[9], Ev[9];
    eps_mat(w, Ew);
    eps_mat(u, Eu);
    eps_mat(v, Ev);
    double a1 = 2.0 / D, a3 = 2.0 * s / (D * D), a4 = 2.0 * s * s / (D * D * D);
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) {
            int bi = i / 3, bj = j / 3, ii = i % 3, jj = j % 3;
            double hs = 0;
            if (bi == 0 && bj == 1) hs = Ev[ii * 3 + jj];
            else if (bi == 1 && bj == 0) hs = Ev[jj * 3 + ii];
            else if (bi == 1 && bj == 2) hs = Ew[ii * 3 + jj];
            else if (bi == 2 && bj == 1) hs = Ew[jj * 3 + ii];
            else if (bi == 2 && bj == 0) hs = Eu[ii * 3 + jj];
            else if (bi == 0 && bj == 2) hs = Eu[jj * 3 + ii];
            double hd = (bi >= 1 && bj >= 1) ? HDuv[(i - 3) * 6 + (j - 3)] : 0.0;
            Hz[i * 9 + j] = a1 * gs[i] * gs[j] + c1 * hs - a3 * (gs[i] * gD[j] + gD[i] * gs[j]) + a4 * gD[i] * gD[j] - c2 * hd;
        }
}

__constant__ signed char C_PT[12] = {1, 0, 0, -1, -1, -1, 0, 1, 0, 0, 0, 1};
__constant__ signed char C_EE[12] = {-1, -1, 0, 0, 1, 0, 1, 0, -1, 0, 0, 1};
__constant__ signed char C_PE[6] = {-1, -1, 1, 0, 0, 1};
__constant__ signed char C_CN[8] = {-1, 0, 1, 0, 0, -1, 0, 1};

// squared distance derivatives in vertex space for stencil kinds PP(0) PE(1) PT(2) EE(3)
__device__ double dist_derivs(int kind, const D3* x, double* g, double* H) {
    if (kind == 0) {
        D3 d = x[0] - x[1];
        double da[3] = {d.x, d.y, d.z};
        for (int i = 0; i < 3; ++i) { g[i] = 2.0 * da[i]; g[3 + i] = -2.0 * da[i]; }
        if (H) {
            for (int i = 0; i < 36; ++i) H[i] = 0;
            for (int i = 0; i < 3; ++i) {
                H[i * 6 + i] = 2; H[(3 + i) * 6 + 3 + i] = 2;
                H[i * 6 + 3 + i] = -2; H[(3 + i) * 6 + i] = -2;
            }
        }
        return d_PP(x[0], x[1]);
    }
    if (kind == 1) {
        D3 a = x[1] - x[0], b = x[2] - x[0];
        double gN[6], HN[36];
        crossnorm2_d(a, b, gN, H ? HN : nullptr);
        double N = sqn(cross(a, b));
        D3 ba = b - a;
        double Q = sqn(ba);
        double bav[3] = {ba.x, ba.y, ba.z};
        double gQ[6];
        for (int i = 0; i < 3; ++i) { gQ[i] = -2.0 * bav[i]; gQ[3 + i] = 2.0 * bav[i]; }
        double gz[6], Hz[36];
        for (int i = 0; i < 6; ++i) gz[i] = gN[i] / Q - N * gQ[i] / (Q * Q);
        if (H)
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) {
                    double HQ = (i % 3 == j % 3) ? ((i / 3) == (j / 3) ? 2.0 : -2.0) : 0.0;
                    Hz[i * 6 + j] = HN[i * 6 + j] / Q - (gN[i] * gQ[j] + gQ[i] * gN[j]) / (Q * Q) +
                                    2.0 * N * gQ[i] * gQ[j] / (Q * Q * Q) - N * HQ / (Q * Q);
                }
        to_vertices<3, 2>(C_PE, gz, H ? Hz : nullptr, g, H);
        return d_PE(x[0], x[1], x[2]);
    }
    double gz[9], Hz[81];
    if (kind == 2) {
        triple_ratio_d(x[0] - x[1], x[2] - x[1], x[3] - x[1], gz, H ? Hz : nullptr);
        to_vertices<4, 3>(C_PT, gz, H ? Hz : nullptr, g, H);
        return d_PT(x[0], x[1], x[2], x[3]);
    }
    triple_ratio_d(x[2] - x[0], x[1] - x[0], x[3] - x[2], gz, H ? Hz : nullptr);
    to_vertices<4, 3>(C_EE, gz, H ? Hz : nullptr, g, H);
    return d_EE(x[0], x[1], x[2], x[3]);
}

__device__ void mollifier_d(const D3* x, double eps_x, double& e, double* g, double* H) {
    double c = ee_cross_norm2(x[0], x[1], x[2], x[3]);
    e = mollifier(c, eps_x);
    if (!(c < eps_x)) {
        for (int i = 0; i < 12; ++i) g[i] = 0;
        if (H) for (int i = 0; i < 144; ++i) H[i] = 0;
        return;
    }
    double gz[6], Hz[36], gc[12];
    crossnorm2_d(x[1] - x[0], x[3] - x[2], gz, H ? Hz : nullptr);
    double Hc[144];
    to_vertices<4, 2>(C_CN, gz, H ? Hz : nullptr, gc, H ? Hc : nullptr);
    double one_div = 1.0 / eps_x;
    double q_g = 2.0 * one_div * (-one_div * c + 1.0);
    double q_H = -2.0 / (eps_x * eps_x);
    for (int i = 0; i < 12; ++i) g[i] = q_g * gc[i];
    if (H)
        for (int i = 0; i < 12; ++i)
            for (int j = 0; j < 12; ++j) H[i * 12 + j] = q_g * Hc[i * 12 + j] + q_H * gc[i] * gc[j];
}

struct BarrierCtx {
    double dHat2i, kappa, th2;
};

// local gradient g (12, FP64) and, when Hout != nullptr, the local Hessian
// (3nv x 3nv, FP64) of one constraint's weighted barrier term
__device__ int barrier_local(const Stencil& st, const double* X, const double* X0, const BarrierCtx& bc, double* g,
                             double* Hl) {
    D3 x[4];
    for (int k = 0; k < 4; ++k) x[k] = (k < st.nv) ? ld3(X, st.v[k]) : mk3(0.0, 0.0, 0.0);
    double dg[12], dH[144];
    int dkind, nd;
    D3 xd[4];
    int map[4] = {0, 1, 2, 3};
    switch (st.kind) {
        case 0: dkind = 0; nd = 2; xd[0] = x[0]; xd[1] = x[1]; break;
        case 1: dkind = 1; nd = 3; xd[0] = x[0]; xd[1] = x[1]; xd[2] = x[2]; break;
        case 2: dkind = 2; nd = 4; xd[0] = x[0]; xd[1] = x[1]; xd[2] = x[2]; xd[3] = x[3]; break;
        case 3: case 4: dkind = 3; nd = 4; xd[0] = x[0]; xd[1] = x[1]; xd[2] = x[2]; xd[3] = x[3]; break;
        case 5: dkind = 1; nd = 3; xd[0] = x[0]; xd[1] = x[2]; xd[2] = x[3]; map[1] = 2; map[2] = 3; break;
        default: dkind = 0; nd = 2; xd[0] = x[0]; xd[1] = x[2]; map[1] = 2; break;
    }
    double d = dist_derivs(dkind, xd, dg, Hl ? dH : nullptr) - bc.th2;
    double bg = barrier_g(d, bc.dHat2i, bc.kappa);
    double bh = Hl ? barrier_h(d, bc.dHat2i, bc.kappa) : 0.0;
    if (st.kind <= 3) {
        double m = (double)st.mult;
        int n = 3 * st.nv;
        for (int i = 0; i < n; ++i) g[i] = m * bg * dg[i];
        if (Hl)
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) Hl[i * n + j] = m * (bh * dg[i] * dg[j] + bg * dH[i * n + j]);
        return st.nv;
    }
    double bv = barrier(d, bc.dHat2i, bc.kappa);
    double eps_x = mollifier_threshold(ld3(X0, st.v[0]), ld3(X0, st.v[1]), ld3(X0, st.v[2]), ld3(X0, st.v[3]));
    double e, eg[12], eH[144];
    mollifier_d(x, eps_x, e, eg, Hl ? eH : nullptr);
    double dg12[12];
    for (int i = 0; i < 12; ++i) dg12[i] = 0;
    for (int a = 0; a < nd; ++a)
        for (int k = 0; k < 3; ++k) dg12[3 * map[a] + k] = dg[3 * a + k];
    for (int i = 0; i < 12; ++i) g[i] = e * bg * dg12[i] + bv * eg[i];
    if (!Hl) return 4;
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) Hl[i * 12 + j] = bg * (dg12[i] * eg[j] + eg[i] * dg12[j]) + bv * eH[i * 12 + j] + e * bh * dg12[i] * dg12[j];
    for (int a = 0; a < nd; ++a)
        for (int b = 0; b < nd; ++b)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l)
                    Hl[(3 * map[a] + k) * 12 + 3 * map[b] + l] += e * bg * dH[(3 * a + k) * (3 * nd) + 3 * b + l];
    return 4;
}

__device__ __forceinline__ BarrierCtx make_ctx(int inst, const double* dHat2, const double* kappa, const double* thick) {
    BarrierCtx bc;
    double dh2 = dHat2[inst], th = thick[inst];
    bc.dHat2i = dh2 + 2 * sqrt(dh2) * th;
    bc.kappa = kappa[inst];
    bc.th2 = th * th;
    return bc;
}

// ---------------------------------------------------------------- kernels
__global__ void k_barrier_energy(long C, const int4* __restrict__ cons, const int* __restrict__ cinst,
                                 const unsigned char* __restrict__ active, const double* __restrict__ X,
                                 const double* __restrict__ X0, const double* __restrict__ dHat2,
                                 const double* __restrict__ kappa, const double* __restrict__ thick,
                                 double* __restrict__ val, int* __restrict__ inst_bad) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    int inst = cinst[i];
    if (!active[inst]) { val[i] = 0; return; }
    BarrierCtx bc = make_ctx(inst, dHat2, kappa, thick);
    int4 c = cons[i];
    Stencil st = decode(c);
    double d = stencil_dist2(st, X) - bc.th2;
    if (d <= 0) {
        inst_bad[inst] = 1;
        val[i] = 0;
        return;
    }
    double e = barrier(d, bc.dHat2i, bc.kappa);
    if (st.kind >= 4) {
        double eps_x = mollifier_threshold(ld3(X0, st.v[0]), ld3(X0, st.v[1]), ld3(X0, st.v[2]), ld3(X0, st.v[3]));
        e *= mollifier(ee_cross_norm2(ld3(X, st.v[0]), ld3(X, st.v[1]), ld3(X, st.v[2]), ld3(X, st.v[3])), eps_x);
    }
    if (st.kind <= 1 && c.w < -1) e *= (double)(-c.w);
    val[i] = e;  // stencil weight is 1 for offset IPC (IPC.h:656-660)
}

// per-instance fixed-order sum of val[off[i] .. off[i+1])
__global__ void k_segment_sum(int nI, const int* __restrict__ off, const double* __restrict__ val,
                              double* __restrict__ out, int accumulate) {
    __shared__ double sh[kBlock];
    int inst = blockIdx.x;
    double s = 0;
    for (int k = off[inst] + threadIdx.x; k < off[inst + 1]; k += blockDim.x) s += val[k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int st = kBlock / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[inst] = accumulate ? out[inst] + sh[0] : sh[0];
}

// the 10 upper 3x3 blocks (a <= b) of an nv-vertex stencil's 3nv x 3nv matrix
template <class T>
__device__ __forceinline__ void write_upper_blocks(const T* H, int n, T* ho) {
    const int nv = n / 3;
    int k = 0;
    for (int a = 0; a < 4; ++a)
        for (int b = a; b < 4; ++b, ++k)
            for (int d = 0; d < 3; ++d)
                for (int e = 0; e < 3; ++e)
                    ho[k * 9 + d * 3 + e] = (a < nv && b < nv) ? H[(3 * a + d) * n + 3 * b + e] : T(0);
}

template <class T>
__global__ void k_barrier_gh(long C, const int4* __restrict__ cons, const int* __restrict__ cinst,
                             const unsigned char* __restrict__ active, const double* __restrict__ X,
                             const double* __restrict__ X0, const double* __restrict__ dHat2,
                             const double* __restrict__ kappa, const double* __restrict__ thick,
                             double* __restrict__ gout, T* __restrict__ hout, T* __restrict__ hloc,
                             int* __restrict__ hn, int* __restrict__ plist, unsigned int* __restrict__ pcount) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    int inst = cinst[i];
    double* go = gout + 12 * i;
    if (!active[inst]) {
        for (int k = 0; k < 12; ++k) go[k] = 0;
        return;
    }
    BarrierCtx bc = make_ctx(inst, dHat2, kappa, thick);
    Stencil st = decode(cons[i]);
    double g[12], Hd[144];
    int nv = barrier_local(st, X, X0, bc, g, hout ? Hd : nullptr);
    for (int k = 0; k < 12; ++k) go[k] = (k < 3 * nv) ? g[k] : 0.0;
    if (!hout) return;
    int n = 3 * nv;
    T H[144];
    for (int k = 0; k < n * n; ++k) H[k] = (T)Hd[k];
    if (!chol_pd(H, n)) {
        // indefinite: projected by k_psd_warp (one warp per matrix)
        T* hl = hloc + 144 * i;
        for (int k = 0; k < n * n; ++k) hl[k] = H[k];
        hn[i] = n;
        plist[atomicAdd(pcount, 1u)] = (int)i;
        return;
    }
    write_upper_blocks(H, n, hout + 90 * i);
}

// The 12x12 PSD projection of makePD (Math/UTILS.h:10-27) for the matrices
// k_barrier_gh found indefinite, one warp per matrix (psd_warp_project).
template <class T>
__global__ void __launch_bounds__(32 * kPsdWarps) k_psd_warp(const int* __restrict__ plist,
                                                               const unsigned int* __restrict__ pcount,
                                                               const T* __restrict__ hloc,
                                                               const int* __restrict__ hn, T* __restrict__ hout) {
    __shared__ T sA[kPsdWarps][144], sV[kPsdWarps][144], sCS[kPsdWarps][6][2], sW[kPsdWarps][12];
    __shared__ int sPQ[kPsdWarps][6][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* A = sA[w];
    T* Vm = sV[w];
    const unsigned int cnt = *pcount;
    for (unsigned int item = blockIdx.x * kPsdWarps + w; item < cnt; item += gridDim.x * kPsdWarps) {
        const int i = plist[item];
        const int n = hn[i];
        for (int k = lane; k < n * n; k += 32) {
            A[k] = hloc[144L * i + k];
            Vm[k] = (k / n == k % n) ? T(1) : T(0);
        }
        __syncwarp();
        psd_warp_project(A, Vm, n, sCS[w], sPQ[w], sW[w], lane);
        const int nv = n / 3;
        T* ho = hout + 90L * i;
        for (int t = lane; t < 90; t += 32) {
            const int blk = t / 9, d = (t % 9) / 3, e = t % 3;
            int a = 0, b = 0, kk = blk;
            for (a = 0; a < 4; ++a) {
                if (kk < 4 - a) { b = a + kk; break; }
                kk -= 4 - a;
            }
            ho[t] = (a < nv && b < nv) ? A[(3 * a + d) * n + 3 * b + e] : T(0);
        }
        __syncwarp();
    }
}

// gradient entries: key = vertex, value = constraint*4 + slot
__global__ void k_grad_entries(long C, const int4* __restrict__ cons, const int* __restrict__ cinst,
                               const unsigned char* __restrict__ active, long V, uint64_t* __restrict__ keys,
                               uint32_t* __restrict__ vals) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    Stencil st = decode(cons[i]);
    bool act = active[cinst[i]] != 0;
    for (int a = 0; a < 4; ++a) {
        bool use = act && a < st.nv;
        keys[4 * i + a] = use ? (uint64_t)st.v[a] : (uint64_t)V;
        vals[4 * i + a] = (uint32_t)(4 * i + a);
    }
}

__global__ void k_grad_gather(long n, long V, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                              const double* __restrict__ lg, double* __restrict__ g) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t k = keys[i];
    if (k >= (uint64_t)V) return;
    if (i > 0 && keys[i - 1] == k) return;
    double s0 = 0, s1 = 0, s2 = 0;
    for (long j = i; j < n && keys[j] == k; ++j) {
        uint32_t v = vals[j];
        const double* p = lg + 12 * (v >> 2) + 3 * (v & 3);
        s0 += p[0];
        s1 += p[1];
        s2 += p[2];
    }
    g[3 * k] += s0;
    g[3 * k + 1] += s1;
    g[3 * k + 2] += s2;
}

// Hessian tail entries: key = row * V + col, value = constraint*16 + a*4 + b
__global__ void k_hess_entries(long C, const int4* __restrict__ cons, const int* __restrict__ cinst,
                               const unsigned char* __restrict__ active, long V, uint64_t* __restrict__ keys,
                               uint32_t* __restrict__ vals) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    Stencil st = decode(cons[i]);
    bool act = active[cinst[i]] != 0;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
            bool use = act && a < st.nv && b < st.nv;
            long e = 16 * i + 4 * a + b;
            keys[e] = use ? (uint64_t)st.v[a] * (uint64_t)V + (uint64_t)st.v[b] : (uint64_t)V * (uint64_t)V;
            vals[e] = (uint32_t)e;
        }
}

__global__ void k_heads(long n, uint64_t marker, const uint64_t* __restrict__ keys, uint32_t* __restrict__ head) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    head[i] = (keys[i] != marker) && (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

template <class T>
__global__ void k_tail_blocks(long n, long V, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                              const uint32_t* __restrict__ head, const uint32_t* __restrict__ pos,
                              const T* __restrict__ bh, int* __restrict__ tcol, int* __restrict__ trow,
                              T* __restrict__ tval) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !head[i]) return;
    uint64_t k = keys[i];
    T acc[9];
    for (int q = 0; q < 9; ++q) acc[q] = T(0);
    for (long j = i; j < n && keys[j] == k; ++j) {
        uint32_t e = vals[j];
        long c = e >> 4;
        int a = (e >> 2) & 3, b = e & 3;
        int lo = a < b ? a : b, hi = a < b ? b : a;
        int kb = lo * 4 - lo * (lo - 1) / 2 + (hi - lo);
        const T* blk = bh + 90 * c + 9 * kb;
        if (a <= b)
            for (int q = 0; q < 9; ++q) acc[q] += blk[q];
        else
            for (int r = 0; r < 3; ++r)
                for (int s = 0; s < 3; ++s) acc[r * 3 + s] += blk[s * 3 + r];
    }
    uint32_t p = pos[i];
    tcol[p] = (int)(k % (uint64_t)V);
    trow[p] = (int)(k / (uint64_t)V);
    for (int q = 0; q < 9; ++q) tval[9 * (long)p + q] = acc[q];
}

__global__ void k_tail_rowptr(long V, long nb, const int* __restrict__ trow, int* __restrict__ rowptr) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v > V) return;
    long lo = 0, hi = nb;
    while (lo < hi) {
        long mid = (lo + hi) >> 1;
        if (trow[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    rowptr[v] = (int)lo;
}

}  // namespace

int barrier_energy(Arena& A, Work& W, const double* X, const ContactSet& cs, double* inst_E, int* inst_bad,
                   cudaStream_t s) {
    if (cs.C <= 0) return IDP_OK;
    if (W[W_MISC].ensure(sizeof(double) * (cs.C + 1))) return IDP_ERR_CUDA;
    double* val = W[W_MISC].as<double>();
    (::idp::count_launch(), k_barrier_energy<<<grid_for(cs.C), kBlock, 0, s>>>(cs.C, W[W_CONS].as<int4>(), W[W_CONS_INST].as<int>(), A.active, X,
                                                       A.X0, A.dHat2, A.kappa, A.thickness, val, inst_bad));
    (::idp::count_launch(), k_segment_sum<<<A.nI, kBlock, 0, s>>>(A.nI, cs.d_off, val, inst_E, 1));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

// computes local gradients (and Hessians when fp64 >= 0), adds the gradient
// into g in a fixed order and builds the contact tail of the system matrix
static int barrier_gh(Arena& A, Work& W, const double* X, const ContactSet& cs, double* g, int hess_mode,
                      cudaStream_t s) {
    long C = cs.C;
    const int4* cons = W[W_CONS].as<int4>();
    const int* cinst = W[W_CONS_INST].as<int>();
    long Ca = C > 0 ? C : 1;
    size_t el = hess_mode == 1 ? sizeof(double) : sizeof(float);
    if (W[W_BG].ensure(sizeof(double) * 12 * Ca)) return IDP_ERR_CUDA;
    if (hess_mode >= 0 && W[W_BH].ensure(el * 90 * Ca)) return IDP_ERR_CUDA;
    if (C > 0) {
        if (hess_mode < 0) {
            (::idp::count_launch(), k_barrier_gh<float><<<grid_for(C, 64), 64, 0, s>>>(
                                        C, cons, cinst, A.active, X, A.X0, A.dHat2, A.kappa, A.thickness,
                                        W[W_BG].as<double>(), nullptr, nullptr, nullptr, nullptr, nullptr));
        } else {
            // PSD scratch: local matrices (144 per constraint) | sizes | list | count
            const size_t o_n = ((el * 144 * (size_t)Ca) + 255) & ~size_t(255);
            const size_t o_l = o_n + ((sizeof(int) * (size_t)Ca + 255) & ~size_t(255));
            const size_t o_c = o_l + ((sizeof(int) * (size_t)Ca + 255) & ~size_t(255));
            if (W[W_PSD].ensure(o_c + 256)) return IDP_ERR_CUDA;
            char* pb = W[W_PSD].as<char>();
            int* hn = reinterpret_cast<int*>(pb + o_n);
            int* plist = reinterpret_cast<int*>(pb + o_l);
            unsigned int* pcount = reinterpret_cast<unsigned int*>(pb + o_c);
            IDP_CUDA_TRY(cudaMemsetAsync(pcount, 0, sizeof(unsigned int), s));
            const int pgrid = (int)std::min<long>((C + kPsdWarps - 1) / kPsdWarps, 8L * 152);
            if (hess_mode == 1) {
                (::idp::count_launch(), k_barrier_gh<double><<<grid_for(C, 64), 64, 0, s>>>(
                                            C, cons, cinst, A.active, X, A.X0, A.dHat2, A.kappa, A.thickness,
                                            W[W_BG].as<double>(), W[W_BH].as<double>(), reinterpret_cast<double*>(pb),
                                            hn, plist, pcount));
                (::idp::count_launch(), k_psd_warp<double><<<pgrid, 32 * kPsdWarps, 0, s>>>(
                                            plist, pcount, reinterpret_cast<const double*>(pb), hn,
                                            W[W_BH].as<double>()));
            } else {
                (::idp::count_launch(), k_barrier_gh<float><<<grid_for(C, 64), 64, 0, s>>>(
                                            C, cons, cinst, A.active, X, A.X0, A.dHat2, A.kappa, A.thickness,
                                            W[W_BG].as<double>(), W[W_BH].as<float>(), reinterpret_cast<float*>(pb),
                                            hn, plist, pcount));
                (::idp::count_launch(), k_psd_warp<float><<<pgrid, 32 * kPsdWarps, 0, s>>>(
                                            plist, pcount, reinterpret_cast<const float*>(pb), hn,
                                            W[W_BH].as<float>()));
            }
        }
    }
    // gradient scatter: sort (vertex, constraint*4+slot) pairs, sum runs in order
    if (g && C > 0) {
        long n = 4 * C;
        if (W[W_GENT_KEY].ensure(8 * n) || W[W_GENT_VAL].ensure(4 * n) || W[W_GENT_KEY2].ensure(8 * n) ||
            W[W_GENT_VAL2].ensure(4 * n) || W[W_SCRATCH].ensure(radix_sort_scratch_bytes(n) + 64))
            return IDP_ERR_CUDA;
        (::idp::count_launch(), k_grad_entries<<<grid_for(C), kBlock, 0, s>>>(C, cons, cinst, A.active, A.V, W[W_GENT_KEY].as<uint64_t>(),
                                                      W[W_GENT_VAL].as<uint32_t>()));
        if (radix_sort_pairs(W[W_GENT_KEY].as<uint64_t>(), W[W_GENT_VAL].as<uint32_t>(), W[W_GENT_KEY2].as<uint64_t>(),
                             W[W_GENT_VAL2].as<uint32_t>(), n, bits_for((uint64_t)A.V), W[W_SCRATCH].p, s) != cudaSuccess)
            return IDP_ERR_CUDA;
        (::idp::count_launch(), k_grad_gather<<<grid_for(n), kBlock, 0, s>>>(n, A.V, W[W_GENT_KEY].as<uint64_t>(), W[W_GENT_VAL].as<uint32_t>(),
                                                     W[W_BG].as<double>(), g));
    }
    if (hess_mode < 0) return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
    // Hessian tail: sort (row*V+col) keys, sum equal keys in order
    long n = 16 * C;
    long na = n > 0 ? n : 1;
    if (W[W_GENT_KEY].ensure(8 * na) || W[W_GENT_VAL].ensure(4 * na) || W[W_GENT_KEY2].ensure(8 * na) ||
        W[W_GENT_VAL2].ensure(4 * na) || W[W_GENT_HEAD].ensure(8 * (na + 1)) ||
        W[W_SCRATCH].ensure(radix_sort_scratch_bytes(na) + scan_scratch_bytes(na) + 64) ||
        W[W_TAIL_ROWPTR].ensure(sizeof(int) * (A.V + 1)) || W[W_TAIL_COL].ensure(sizeof(int) * 2 * na) ||
        W[W_TAIL_VAL].ensure(el * 9 * na))
        return IDP_ERR_CUDA;
    long nb = 0;
    if (n > 0) {
        uint64_t* keys = W[W_GENT_KEY].as<uint64_t>();
        uint32_t* vals = W[W_GENT_VAL].as<uint32_t>();
        (::idp::count_launch(), k_hess_entries<<<grid_for(C), kBlock, 0, s>>>(C, cons, cinst, A.active, A.V, keys, vals));
        uint64_t marker = (uint64_t)A.V * (uint64_t)A.V;
        int bits = bits_for(marker);
        if (radix_sort_pairs(keys, vals, W[W_GENT_KEY2].as<uint64_t>(), W[W_GENT_VAL2].as<uint32_t>(), n, bits,
                             W[W_SCRATCH].p, s) != cudaSuccess)
            return IDP_ERR_CUDA;
        uint32_t* head = W[W_GENT_HEAD].as<uint32_t>();
        uint32_t* pos = head + na + 1;
        (::idp::count_launch(), k_heads<<<grid_for(n), kBlock, 0, s>>>(n, marker, keys, head));
        if (scan_exclusive(head, pos, n, pos + n, W[W_SCRATCH].p, s) != cudaSuccess) return IDP_ERR_CUDA;
        uint32_t hnb = 0;
        IDP_CUDA_TRY(cudaMemcpyAsync(&hnb, pos + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        nb = hnb;
        int* tcol = W[W_TAIL_COL].as<int>();
        int* trow = tcol + na;
        if (hess_mode == 1)
            (::idp::count_launch(), k_tail_blocks<double><<<grid_for(n), kBlock, 0, s>>>(n, A.V, keys, vals, head, pos, W[W_BH].as<double>(), tcol,
                                                                 trow, W[W_TAIL_VAL].as<double>()));
        else
            (::idp::count_launch(), k_tail_blocks<float><<<grid_for(n), kBlock, 0, s>>>(n, A.V, keys, vals, head, pos, W[W_BH].as<float>(), tcol,
                                                                trow, W[W_TAIL_VAL].as<float>()));
        (::idp::count_launch(), k_tail_rowptr<<<grid_for(A.V + 1), kBlock, 0, s>>>(A.V, nb, trow, W[W_TAIL_ROWPTR].as<int>()));
    } else {
        IDP_CUDA_TRY(cudaMemsetAsync(W[W_TAIL_ROWPTR].p, 0, sizeof(int) * (A.V + 1), s));
    }
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int barrier_gradient(Arena& A, Work& W, const double* X, const ContactSet& cs, double* g, cudaStream_t s) {
    return barrier_gh(A, W, X, cs, g, -1, s);
}

int barrier_hessian(Arena& A, Work& W, const double* X, const ContactSet& cs, bool fp64, cudaStream_t s) {
    return barrier_gh(A, W, X, cs, nullptr, fp64 ? 1 : 0, s);
}

}  // namespace idp
