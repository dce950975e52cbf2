// Sparse system assembly and the linear solve that replaces the direct
// factorisation of Math/DIRECT_SOLVER.h:13-65, plus the per-vertex vector
// kernels of the Newton loop.
//
// Matrix: 3x3 BSR over the fixed tet stencil (pattern built once per
// context) + a per-iteration contact tail (CSR of 3x3 blocks from the barrier
// Hessians) + the lumped mass on the diagonal, with the DBC rows and columns
// replaced by identity (Math/CSR_MATRIX.h:130-141). Each BSR block is the sum,
// in a fixed order, of the element blocks listed for it, so assembly is
// deterministic.
//
// Solve: block-Jacobi PCG per instance (every instance of the batch carries
// its own scalars and stops on its own). Mixed mode runs PCG in FP32 and
// recovers the direction by iterative refinement against an FP64 residual
// r = b - A x (FP32 matrix, FP64 accumulation); FP64 mode runs PCG in FP64.
#include <atomic>
#include <cooperative_groups.h>
#include "engine.hpp"
#include "prims.cuh"

namespace cg = cooperative_groups;

namespace idp {

namespace {

template <class T>
__device__ __forceinline__ T blk_get(const T* tet_hess, int code, int q) {
    // code = (tet*10 + k)*2 + transposed
    long base = (long)(code >> 1) * 9;
    if (code & 1) return tet_hess[base + (q % 3) * 3 + q / 3];
    return tet_hess[base + q];
}

template <class T>
__global__ void k_assemble_tet(long B, const int* __restrict__ src_ptr, const int* __restrict__ src,
                               const T* __restrict__ tet_hess, const int* __restrict__ brow,
                               const int* __restrict__ colidx, const double* __restrict__ mass,
                               const unsigned char* __restrict__ dbc, const int* __restrict__ vinst,
                               const unsigned char* __restrict__ active, const double* __restrict__ fvol, double h,
                               const double* __restrict__ dstiff, const unsigned char* __restrict__ excl,
                               T* __restrict__ val) {
    long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    int row = brow[b], col = colidx[b];
    if (!active[vinst[row]]) return;
    T acc[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] = T(0);
    for (int k = src_ptr[b]; k < src_ptr[b + 1]; ++k) {
        int code = src[k];
        if (code < 0) {
            // shell face in flow mode: -h L (INC_POTENTIAL.h:323-339),
            // 2 h vol/6 I on the diagonal, -h vol/6 I off it
            const int cf = -code - 1;
            const double w = h * fvol[cf >> 1] / 6.0;
            const T d = (T)((cf & 1) ? 2.0 * w : -w);
            acc[0] += d; acc[4] += d; acc[8] += d;
            continue;
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] += blk_get(tet_hess, code, q);
    }
    if (row == col) {
        T m = (T)mass[row];
        acc[0] += m; acc[4] += m; acc[8] += m;
        // moving-DBC penalty stiff * m on the diagonal (Compute_DBC_Hessian,
        // FEM/Shell/DIRICHLET.h:72-90)
        if (excl[row] && dstiff[vinst[row]] > 0) {
            T k = (T)(dstiff[vinst[row]] * mass[row]);
            acc[0] += k; acc[4] += k; acc[8] += k;
        }
    }
    if (dbc[row] || dbc[col]) {
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] = T(0);
        if (row == col) { acc[0] = acc[4] = acc[8] = T(1); }
    }
    T* o = val + 9 * b;
#pragma unroll
    for (int q = 0; q < 9; ++q) o[q] = acc[q];
}

template <class T>
__device__ __forceinline__ void inv3(const T a[9], T o[9]) {
    T c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
    T det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    T id = T(1) / det;
    o[0] = c00 * id;
    o[1] = (a[2] * a[7] - a[1] * a[8]) * id;
    o[2] = (a[1] * a[5] - a[2] * a[4]) * id;
    o[3] = c01 * id;
    o[4] = (a[0] * a[8] - a[2] * a[6]) * id;
    o[5] = (a[2] * a[3] - a[0] * a[5]) * id;
    o[6] = c02 * id;
    o[7] = (a[1] * a[6] - a[0] * a[7]) * id;
    o[8] = (a[0] * a[4] - a[1] * a[3]) * id;
}

// block-Jacobi: inverse of (tet diagonal block + tail diagonal block)
template <class T>
__global__ void k_diag_inv(long V, const int* __restrict__ diagblk, const T* __restrict__ val,
                           const int* __restrict__ trp, const int* __restrict__ tcol, const T* __restrict__ tval,
                           const unsigned char* __restrict__ dbc, const int* __restrict__ vinst,
                           const unsigned char* __restrict__ active, T* __restrict__ dinv) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    T a[9];
    const T* d = val + 9 * (long)diagblk[v];
#pragma unroll
    for (int q = 0; q < 9; ++q) a[q] = d[q];
    if (!dbc[v])
        for (int k = trp[v]; k < trp[v + 1]; ++k)
            if (tcol[k] == v)
#pragma unroll
                for (int q = 0; q < 9; ++q) a[q] += tval[9 * (long)k + q];
    T o[9];
    inv3(a, o);
#pragma unroll
    for (int q = 0; q < 9; ++q) dinv[9 * v + q] = o[q];
}

// y = A x for the rows of instances with run[inst] != 0; optional partial
// dot products p.y per vertex chunk
template <class T, class TX, class TY>
__device__ __forceinline__ void spmv_row(long v, const int* __restrict__ rowptr, const int* __restrict__ colidx,
                                         const T* __restrict__ val, const int* __restrict__ trp,
                                         const int* __restrict__ tcol, const T* __restrict__ tval,
                                         const unsigned char* __restrict__ dbc, const TX* __restrict__ x, TY y[3]) {
    if (dbc[v]) {
        y[0] = (TY)x[3 * v]; y[1] = (TY)x[3 * v + 1]; y[2] = (TY)x[3 * v + 2];
        return;
    }
    TY a0 = 0, a1 = 0, a2 = 0;
    for (int k = rowptr[v]; k < rowptr[v + 1]; ++k) {
        int c = colidx[k];
        const T* m = val + 9 * (long)k;
        TY x0 = (TY)x[3 * c], x1 = (TY)x[3 * c + 1], x2 = (TY)x[3 * c + 2];
        a0 += (TY)m[0] * x0 + (TY)m[1] * x1 + (TY)m[2] * x2;
        a1 += (TY)m[3] * x0 + (TY)m[4] * x1 + (TY)m[5] * x2;
        a2 += (TY)m[6] * x0 + (TY)m[7] * x1 + (TY)m[8] * x2;
    }
    for (int k = trp[v]; k < trp[v + 1]; ++k) {
        int c = tcol[k];
        if (dbc[c]) continue;
        const T* m = tval + 9 * (long)k;
        TY x0 = (TY)x[3 * c], x1 = (TY)x[3 * c + 1], x2 = (TY)x[3 * c + 2];
        a0 += (TY)m[0] * x0 + (TY)m[1] * x1 + (TY)m[2] * x2;
        a1 += (TY)m[3] * x0 + (TY)m[4] * x1 + (TY)m[5] * x2;
        a2 += (TY)m[6] * x0 + (TY)m[7] * x1 + (TY)m[8] * x2;
    }
    y[0] = a0; y[1] = a1; y[2] = a2;
}

__device__ double cta_sum(double v) {
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

// FP64 residual res = b - A x64 (FP32/FP64 matrix, FP64 accumulation), one
// thread per block row in small CTAs (the FP64 pipe, not memory, limits it);
// the squared norm is reduced afterwards per vertex chunk
template <class T>
__global__ void k_residual64(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                             const int* __restrict__ rowptr, const int* __restrict__ colidx, const T* __restrict__ val,
                             const int* __restrict__ trp, const int* __restrict__ tcol, const T* __restrict__ tval,
                             const unsigned char* __restrict__ dbc, const double* __restrict__ b,
                             const double* __restrict__ x, double* __restrict__ res) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    double y[3];
    spmv_row<T, double, double>(v, rowptr, colidx, val, trp, tcol, tval, dbc, x, y);
#pragma unroll
    for (int d = 0; d < 3; ++d) res[3 * v + d] = dbc[v] ? 0.0 : b[3 * v + d] - y[d];
}

__global__ void k_norm2_chunks(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                               const double* __restrict__ a, double* __restrict__ part) {
    Chunk c = chunks[blockIdx.x];
    double acc = 0;
    if (active[c.inst])
        for (int k = 3 * c.begin + threadIdx.x; k < 3 * c.end; k += blockDim.x) acc += a[k] * a[k];
    double s = cta_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_zero_masked(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                              double* __restrict__ x) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    x[3 * v] = 0.0;
    x[3 * v + 1] = 0.0;
    x[3 * v + 2] = 0.0;
}

template <class T>
__global__ void k_add_correction(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                                 const T* __restrict__ e, double* __restrict__ x) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    for (int d = 0; d < 3; ++d) x[3 * v + d] += (double)e[3 * v + d];
}

template <class T>
__global__ void k_spmv_plain(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                             const int* __restrict__ rowptr, const int* __restrict__ colidx, const T* __restrict__ val,
                             const int* __restrict__ trp, const int* __restrict__ tcol, const T* __restrict__ tval,
                             const unsigned char* __restrict__ dbc, const double* __restrict__ x,
                             double* __restrict__ y) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    double o[3];
    spmv_row<T, double, double>(v, rowptr, colidx, val, trp, tcol, tval, dbc, x, o);
    y[3 * v] = o[0]; y[3 * v + 1] = o[1]; y[3 * v + 2] = o[2];
}

// ---- per-vertex Newton kernels
__global__ void k_grad_gather_tet(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                                  const int* __restrict__ vcp, const int* __restrict__ vc,
                                  const double* __restrict__ tg, const double* __restrict__ mass,
                                  const double* __restrict__ X, const double* __restrict__ Xt, double* __restrict__ g) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    double s0 = 0, s1 = 0, s2 = 0;
    for (int k = vcp[v]; k < vcp[v + 1]; ++k) {
        int code = vc[k];  // tet*4 + corner
        const double* p = tg + 12 * (long)(code >> 2) + 3 * (code & 3);
        s0 += p[0]; s1 += p[1]; s2 += p[2];
    }
    double m = mass[v];
    g[3 * v] = s0 + m * (X[3 * v] - Xt[3 * v]);
    g[3 * v + 1] = s1 + m * (X[3 * v + 1] - Xt[3 * v + 1]);
    g[3 * v + 2] = s2 + m * (X[3 * v + 2] - Xt[3 * v + 2]);
}

__global__ void k_inertia_energy(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                                 const double* __restrict__ mass, const double* __restrict__ X,
                                 const double* __restrict__ Xt, double* __restrict__ part) {
    Chunk c = chunks[blockIdx.x];
    double acc = 0;
    if (active[c.inst])
        for (int v = c.begin + threadIdx.x; v < c.end; v += blockDim.x) {
            double d0 = X[3 * v] - Xt[3 * v], d1 = X[3 * v + 1] - Xt[3 * v + 1], d2 = X[3 * v + 2] - Xt[3 * v + 2];
            acc += 0.5 * mass[v] * (d0 * d0 + d1 * d1 + d2 * d2);
        }
    double s = cta_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// per instance: its chunk partials summed by one warp (lane-strided, then a
// butterfly; fixed order)
__global__ void k_chunk_reduce(int nI, const int* __restrict__ coff, const double* __restrict__ part,
                               double* __restrict__ out, int accumulate) {
    const int i = (int)(((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (i >= nI) return;  // whole warp
    double s = 0;
    for (int c = coff[i] + lane; c < coff[i + 1]; c += 32) s += part[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[i] = accumulate ? out[i] + s : s;
}

__global__ void k_axpy_trial(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                             const double* __restrict__ alpha, const double* __restrict__ Xp,
                             const double* __restrict__ dir, double* __restrict__ Xo) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    int i = vinst[v];
    if (!active[i]) return;
    double a = alpha[i];
    for (int d = 0; d < 3; ++d) Xo[3 * v + d] = Xp[3 * v + d] + a * dir[3 * v + d];
}

__global__ void k_zero_dbc(long V, const unsigned char* __restrict__ dbc, double* __restrict__ g) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !dbc[v]) return;
    g[3 * v] = g[3 * v + 1] = g[3 * v + 2] = 0;
}

template <class T>
__device__ __forceinline__ void precond(long v, const T* __restrict__ dinv, const unsigned char* __restrict__ dbc,
                                        const T rv[3], T zv[3]) {
    if (dbc[v]) { zv[0] = zv[1] = zv[2] = T(0); return; }
    const T* D = dinv + 9 * v;
    zv[0] = D[0] * rv[0] + D[1] * rv[1] + D[2] * rv[2];
    zv[1] = D[3] * rv[0] + D[4] * rv[1] + D[5] * rv[2];
    zv[2] = D[6] * rv[0] + D[7] * rv[1] + D[8] * rv[2];
}

// ---- persistent PCG: one thread-block cluster runs the whole solve of one
// instance. CTA r of the cluster owns a contiguous slice of the instance's
// vertices; dot products are reduced inside each CTA (warp shuffles, then
// warp partials in order) and across the cluster through distributed shared
// memory (every CTA adds the cluster's partials in rank order, so all CTAs
// hold the same bit-identical scalar). Cluster barriers order the phases.
// Accumulation precision follows the vectors (FP32 in mixed mode).
constexpr int CL_THREADS = 512;
constexpr long kClusterCtaVertices = 160;

// y = A x over block rows [v0, v1) of one CTA: 8 lanes per row, 4 rows per
// warp in flight (lane j of a row takes blocks k0+j, k0+j+8, ...), a 3-step
// butterfly per component, then emit(v, y) on the row's first lane. The
// vector x may have been written by other CTAs of the same launch, so it is
// read through L2 (ld.cg). All lanes of every warp must call this together.
template <class T, class Emit>
__device__ __forceinline__ void spmv_rows8(int v0, int v1, const int* __restrict__ rowptr,
                                           const int* __restrict__ colidx, const T* __restrict__ val,
                                           const int* __restrict__ trp, const int* __restrict__ tcol,
                                           const T* __restrict__ tval, const unsigned char* __restrict__ dbc,
                                           const T* x, Emit&& emit) {
    const int lane = threadIdx.x & 31, l8 = lane & 7;
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = v0 + 4 * warp; base < v1; base += 4 * nw) {
        const int v = base + (lane >> 3);
        const bool act = v < v1;
        const bool fixed = act && dbc[v];
        T a0 = 0, a1 = 0, a2 = 0;
        if (act && !fixed) {
            const int k1 = rowptr[v + 1];
            for (int k = rowptr[v] + l8; k < k1; k += 8) {
                const int c = colidx[k];
                const T* m = val + 9L * k;
                const T x0 = __ldcg(x + 3 * c), x1 = __ldcg(x + 3 * c + 1), x2 = __ldcg(x + 3 * c + 2);
                a0 += m[0] * x0 + m[1] * x1 + m[2] * x2;
                a1 += m[3] * x0 + m[4] * x1 + m[5] * x2;
                a2 += m[6] * x0 + m[7] * x1 + m[8] * x2;
            }
            const int t1 = trp[v + 1];
            for (int k = trp[v] + l8; k < t1; k += 8) {
                const int c = tcol[k];
                if (dbc[c]) continue;
                const T* m = tval + 9L * k;
                const T x0 = __ldcg(x + 3 * c), x1 = __ldcg(x + 3 * c + 1), x2 = __ldcg(x + 3 * c + 2);
                a0 += m[0] * x0 + m[1] * x1 + m[2] * x2;
                a1 += m[3] * x0 + m[4] * x1 + m[5] * x2;
                a2 += m[6] * x0 + m[7] * x1 + m[8] * x2;
            }
        }
        for (int o = 4; o > 0; o >>= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        }
        if (act && l8 == 0) {
            T y[3] = {a0, a1, a2};
            if (fixed) { y[0] = __ldcg(x + 3 * v); y[1] = __ldcg(x + 3 * v + 1); y[2] = __ldcg(x + 3 * v + 2); }
            emit(v, y);
        }
    }
}

template <class T>
__device__ __forceinline__ T cta_reduce2(T a, T b, T* wsh, T& out_b) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) { wsh[2 * warp] = a; wsh[2 * warp + 1] = b; }
    __syncthreads();
    T ra = 0, rb = 0;
    for (int w = 0; w < nw; ++w) { ra += wsh[2 * w]; rb += wsh[2 * w + 1]; }
    out_b = rb;
    return ra;
}

// sum of one value over the CTA in a fixed order (result on every thread)
template <class T>
__device__ __forceinline__ T cta_sum1(T a, T* wsh) {
    T dummy;
    return cta_reduce2(a, T(0), wsh, dummy);
}

template <class T>
__device__ __forceinline__ void cluster_sum2(cg::cluster_group& cl, T a, T b, T (*slot)[2], int which, T& sa, T& sb) {
    if (threadIdx.x == 0) { slot[which][0] = a; slot[which][1] = b; }
    cl.sync();
    T ra = 0, rb = 0;
    const int n = (int)cl.num_blocks();
    for (int r = 0; r < n; ++r) {
        T* rp = cl.map_shared_rank(&slot[which][0], r);
        ra += rp[0];
        rb += rp[1];
    }
    sa = ra;
    sb = rb;
}

// contact-cluster blocks of the preconditioner, as seen by the PCG kernel
template <class T>
struct ClusterPC {
    const int* vcl;        // V: block id or -1
    const int* ioff;       // nI+1: blocks of each instance
    const int* off;        // blocks: vertex offsets
    const int* vert;       // block vertices
    const long long* doff; // dense offsets
    const int* ok;         // factorisation succeeded
    const T* Kinv;         // dense inverses
};

// z = M^{-1} r on the rows of the blocks owned by this CTA (blocks c of the
// instance with c % csize == crank): z = Y^T (Y r) with Y = L^{-1} the inverse
// Cholesky factor of the block, or 3x3 inverses when the factorisation failed.
// rc must hold 6 * kClusterCap values (r of the block, then Y r).
template <class T>
__device__ void apply_blocks(const ClusterPC<T>& pc, int inst, int crank, int csize, const T* __restrict__ dinv,
                             const unsigned char* __restrict__ dbc, const T* __restrict__ r, T* __restrict__ z,
                             T* __restrict__ p_init, T* rc) {
    T* tc = rc + 3 * kClusterCap;  // second half of the caller's shared buffer
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = pc.ioff[inst] + crank; c < pc.ioff[inst + 1]; c += csize) {
        const int o = pc.off[c], n = pc.off[c + 1] - o, N = 3 * n;
        if (!pc.ok[c]) {
            for (int li = threadIdx.x; li < n; li += blockDim.x) {
                int v = pc.vert[o + li];
                T rv[3] = {__ldcg(r + 3 * v), __ldcg(r + 3 * v + 1), __ldcg(r + 3 * v + 2)}, zv[3];
                precond(v, dinv, dbc, rv, zv);
                for (int d = 0; d < 3; ++d) {
                    z[3 * v + d] = zv[d];
                    if (p_init) p_init[3 * v + d] = zv[d];
                }
            }
            continue;
        }
        for (int a = threadIdx.x; a < N; a += blockDim.x) rc[a] = __ldcg(r + 3 * pc.vert[o + a / 3] + a % 3);
        __syncthreads();
        const T* Yc = pc.Kinv + pc.doff[c];
        // t = Y r (Y lower triangular; rows by warps, two rows per warp, every
        // load of both rows issued before the sums); t overwrites tc
        constexpr int kPer = (3 * kClusterCap + 31) / 32;
        for (int a = 2 * warp; a < N; a += 2 * nw) {
            const T* r0 = Yc + (long)a * N;
            const T* r1 = r0 + N;
            const bool two = a + 1 < N;
            T acc0 = 0, acc1 = 0;
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int bb = lane + 32 * j;
                if (bb <= a + 1 && bb < N) {
                    const T rv = rc[bb];
                    if (bb <= a) acc0 += __ldg(r0 + bb) * rv;
                    if (two) acc1 += __ldg(r1 + bb) * rv;
                }
            }
            for (int ofs = 16; ofs > 0; ofs >>= 1) {
                acc0 += __shfl_down_sync(0xffffffffu, acc0, ofs);
                acc1 += __shfl_down_sync(0xffffffffu, acc1, ofs);
            }
            if (lane == 0) {
                tc[a] = acc0;
                if (two) tc[a + 1] = acc1;
            }
        }
        __syncthreads();
        // z = Y^T t: column b of Y against t, threads over b (row k of Y is
        // read coalesced)
        for (int b = threadIdx.x; b < N; b += blockDim.x) {
            T acc = 0;
#pragma unroll 4
            for (int k = b; k < N; ++k) acc += __ldg(Yc + (long)k * N + b) * tc[k];
            const int v = pc.vert[o + b / 3];
            const T zz = dbc[v] ? T(0) : acc;
            z[3 * v + b % 3] = zz;
            if (p_init) p_init[3 * v + b % 3] = zz;
        }
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(CL_THREADS) k_pcg_cluster(
    const int* __restrict__ inst_list, const int* __restrict__ v_off, const int* __restrict__ rowptr,
    const int* __restrict__ colidx, const T* __restrict__ val, const int* __restrict__ trp, const int* __restrict__ tcol,
    const T* __restrict__ tval, const unsigned char* __restrict__ dbc, const T* __restrict__ dinv, ClusterPC<T> pc,
    const double* __restrict__ b, T* __restrict__ x, T* __restrict__ r, T* __restrict__ z, T* __restrict__ p,
    T* __restrict__ Ap, const double* __restrict__ tol_inst, double rel_tol, int max_iters,
    int* __restrict__ iters_out) {
    __shared__ T wsh[2 * (CL_THREADS / 32)];
    __shared__ T slot[4][2];
    __shared__ T rc[6 * kClusterCap];
    cg::cluster_group cl = cg::this_cluster();
    const int csize = (int)cl.num_blocks(), crank = (int)cl.block_rank();
    const int inst = inst_list[blockIdx.x / csize];
    const int iv0 = v_off[inst], iv1 = v_off[inst + 1];
    const int per = (iv1 - iv0 + csize - 1) / csize;
    const int v0 = iv0 + crank * per, v1 = min(iv1, v0 + per);
    const bool has_blocks = pc.ioff[inst + 1] > pc.ioff[inst];
    int which = 0;
    // r = b, z = M^{-1} r, p = z
    T rr_l = 0;
    for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
        T rv[3], zv[3];
        for (int d = 0; d < 3; ++d) {
            rv[d] = dbc[v] ? T(0) : (T)b[3 * v + d];
            x[3 * v + d] = T(0);
            r[3 * v + d] = rv[d];
            rr_l += rv[d] * rv[d];
        }
        if (pc.vcl[v] < 0) {
            precond(v, dinv, dbc, rv, zv);
            for (int d = 0; d < 3; ++d) {
                z[3 * v + d] = zv[d];
                p[3 * v + d] = zv[d];
            }
        }
    }
    if (has_blocks) {
        cl.sync();
        apply_blocks(pc, inst, crank, csize, dinv, dbc, r, z, p, rc);
        cl.sync();
    }
    T rz_l = 0;
    for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x)
        for (int d = 0; d < 3; ++d) rz_l += r[3 * v + d] * z[3 * v + d];
    T rr_c, rz = cta_reduce2(rz_l, rr_l, wsh, rr_c);
    T rr;
    cluster_sum2(cl, rz, rr_c, slot, which, rz, rr);
    which ^= 1;
    const double tl = tol_inst ? fmax(tol_inst[inst], rel_tol) : rel_tol;
    const T tol2 = (T)(tl * tl) * rr;
    int it = 0;
    if (rr > T(0) && rr > tol2) {
        for (it = 0; it < max_iters;) {
            cl.sync();  // every CTA's p is written before any CTA reads neighbours
            T pAp_l = 0;
            spmv_rows8<T>(v0, v1, rowptr, colidx, val, trp, tcol, tval, dbc, p, [&](int v, const T* y) {
                for (int d = 0; d < 3; ++d) {
                    Ap[3 * v + d] = y[d];
                    pAp_l += __ldcg(p + 3 * v + d) * y[d];
                }
            });
            T dummy, pAp = cta_reduce2(pAp_l, T(0), wsh, dummy);
            cluster_sum2(cl, pAp, T(0), slot, which, pAp, dummy);
            which ^= 1;
            if (!(pAp > T(0))) break;
            const T alpha = rz / pAp;
            T rrn_l = 0, rzn_l = 0;
            for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
                T rv[3], zv[3];
                for (int d = 0; d < 3; ++d) {
                    x[3 * v + d] += alpha * p[3 * v + d];
                    rv[d] = r[3 * v + d] - alpha * Ap[3 * v + d];
                    r[3 * v + d] = rv[d];
                    rrn_l += rv[d] * rv[d];
                }
                if (pc.vcl[v] < 0) {
                    precond(v, dinv, dbc, rv, zv);
                    for (int d = 0; d < 3; ++d) {
                        z[3 * v + d] = zv[d];
                        if (!has_blocks) rzn_l += rv[d] * zv[d];
                    }
                }
            }
            if (has_blocks) {
                cl.sync();
                apply_blocks(pc, inst, crank, csize, dinv, dbc, r, z, (T*)nullptr, rc);
                cl.sync();
                for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x)
                    for (int d = 0; d < 3; ++d) rzn_l += r[3 * v + d] * __ldcg(z + 3 * v + d);
            }
            T rrn_c, rzn = cta_reduce2(rzn_l, rrn_l, wsh, rrn_c);
            T rrn;
            cluster_sum2(cl, rzn, rrn_c, slot, which, rzn, rrn);
            which ^= 1;
            ++it;
            if (rrn <= tol2) break;
            const T beta = rzn / rz;
            rz = rzn;
            for (int v = v0 + threadIdx.x; v < v1; v += blockDim.x)
                for (int d = 0; d < 3; ++d) p[3 * v + d] = z[3 * v + d] + beta * p[3 * v + d];
        }
    }
    cl.sync();  // no CTA leaves while others may still read its shared memory
    if (crank == 0 && threadIdx.x == 0) iters_out[inst] = it;
}

// ---- grid-wide PCG for large instances: one cooperative launch holds every
// CTA of the wave resident; instance i owns CTAs [c0, c0+nc) (nc depends only
// on the instance's size, so results do not depend on what else is solved)
// and synchronises them through its own control block. Dot products: fixed
// in-CTA tree, then the last CTA to arrive sums the instance's CTA partials
// in CTA order and publishes the result (bit-identical scalars everywhere,
// whichever CTA arrives last). Two such rounds per iteration: the direction
// update is folded into the SpMV pass (w = A z, p = z + beta p,
// q = w + beta q with q = A p kept by recurrence). Vectors written inside
// the kernel are read through L2 (ld.cg) so no CTA sees a stale L1 line.
constexpr int GP_THREADS = 256;
constexpr int kRL = 4;  // lanes per block row in the grid PCG's SpMV (8 rows per warp step)
constexpr unsigned int kSpinLimit = 1u << 22;  // ~1 s of polling, then error
constexpr int kCtlWords = 64;                   // per instance: counter at [0], release word at [32]
constexpr int kGridSmem = 69 * 1024;            // dynamic shared memory per CTA (three CTAs per SM)

struct GridCta {
    int inst, v0, v1, c0, nc, slot;
};

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Round k (1, 2, ...) over the nc CTAs of one instance. Every CTA adds its
// partials (kRed values; thread 0's) and arrives on the counter; the CTA
// whose arrival completes the round (counter = k*nc) sums the partials in
// CTA order when `reduce` is set, stores the sums in red and releases the
// others, who spin (bounded: after kSpinLimit polls the error flag is set and
// false returned) on the release word. The counter and the release word sit
// on separate 128-byte lines so the arrivals do not queue behind the polling.
constexpr int kRed = 4;

template <class T>
__device__ __forceinline__ bool inst_round(unsigned int* ctl, T* red, T* part, int c0, int nc, unsigned int k,
                                           bool reduce, const T* a, T* ra, int* err, int* sh_i, T* sh_t) {
    if (threadIdx.x == 0) {
        if (reduce)
            for (int j = 0; j < kRed; ++j) part[kRed * blockIdx.x + j] = a[j];
        __threadfence();
        const unsigned int old = atomicAdd(ctl, 1u);
        sh_i[0] = old == k * (unsigned int)nc - 1u;
        sh_i[1] = 1;
    }
    __syncthreads();
    if (sh_i[0]) {
        if (reduce) {
            // every thread of the completing CTA loads its share of the
            // partials at once (one L2 round trip), then a fixed-order tree:
            // lanes by shuffles, warps in order
            __shared__ T wred[GP_THREADS / 32][kRed];
            __threadfence();
            T acc[kRed] = {};
            for (int c = threadIdx.x; c < nc; c += GP_THREADS)
                for (int j = 0; j < kRed; ++j) acc[j] += __ldcg(part + kRed * (c0 + c) + j);
            for (int o = 16; o > 0; o >>= 1)
                for (int j = 0; j < kRed; ++j) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
            if ((threadIdx.x & 31) == 0)
                for (int j = 0; j < kRed; ++j) wred[threadIdx.x >> 5][j] = acc[j];
            __syncthreads();
            if (threadIdx.x == 0)
                for (int j = 0; j < kRed; ++j) {
                    T t = wred[0][j];
                    for (int w = 1; w < GP_THREADS / 32; ++w) t += wred[w][j];
                    red[j] = t;
                }
        }
        if (threadIdx.x == 0) {
            __threadfence();
            atomicExch(ctl + 32, k);
        }
    } else if (threadIdx.x == 0) {
        unsigned int n = 0;
        while (*(volatile unsigned int*)(ctl + 32) < k) {
            if (++n > kSpinLimit) {
                atomicExch(err, 1);
                sh_i[1] = 0;
                break;
            }
            if (n > 256) __nanosleep(32);  // tight polling first, then back off
        }
        __threadfence();
    }
    __syncthreads();
    const bool ok = sh_i[1] != 0;
    if (reduce) {
        if (threadIdx.x < kRed) sh_t[threadIdx.x] = __ldcg(red + threadIdx.x);
        __syncthreads();
        for (int j = 0; j < kRed; ++j) ra[j] = sh_t[j];
    }
    __syncthreads();  // sh_i / sh_t are reused by the next round
    return ok;
}

// Rows of a grid-PCG CTA held in dynamic shared memory for the whole solve:
//   int srow[nv + 1]        row offsets relative to the CTA's first block
//   T   sdinv[9 nv]         3x3 block-Jacobi inverses
//   T   sval[9 ncache]      BSR values of a prefix of the CTA's blocks
//   int scol[ncache]        their block columns
// (ncache = every block when they fit, else the prefix that does; rows past
// it read the matrix from global memory). Only the vector gathers of the
// SpMV then leave the SM.
template <class T>
struct GridRows {
    int* row;
    T* dinv;
    T* val;
    int* col;
    int ncache;
};

// fixed part of the image: row offsets, the 3x3 inverses and, with the
// CTA-local polynomial preconditioner, three 3-vectors per row
__host__ __device__ inline size_t grid_smem_fixed(int nvmax, size_t tsize, bool poly) {
    size_t a = ((size_t)(nvmax + 1) * 4 + 15) & ~size_t(15);
    return a + tsize * (poly ? 18 : 9) * (size_t)nvmax;
}

template <class T>
__device__ __forceinline__ void grid_precond(const T* D, bool fixed, const T rv[3], T zv[3]) {
    if (fixed) { zv[0] = zv[1] = zv[2] = T(0); return; }
    zv[0] = D[0] * rv[0] + D[1] * rv[1] + D[2] * rv[2];
    zv[1] = D[3] * rv[0] + D[4] * rv[1] + D[5] * rv[2];
    zv[2] = D[6] * rv[0] + D[7] * rv[1] + D[8] * rv[2];
}

template <class T>
__global__ void __launch_bounds__(GP_THREADS, 3) k_pcg_grid(
    const GridCta* __restrict__ plan, int cap_blocks, int nvmax, const int* __restrict__ rowptr,
    const int* __restrict__ colidx, const T* __restrict__ val, const int* __restrict__ trp,
    const int* __restrict__ tcol, const T* __restrict__ tval, const unsigned char* __restrict__ dbc,
    const T* __restrict__ dinv, ClusterPC<T> pc, const double* __restrict__ b, T* x, T* r, T* z, T* p, T* q,
    T* u, T* w, T* sv, T* m0, T* m1, T* part, T* redbuf, unsigned int* ctlbuf, int* err,
    const double* __restrict__ tol_inst, double rel_tol, int max_iters, int* __restrict__ iters_out,
    unsigned long long* prof, int local_deg) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T wsh[2 * (GP_THREADS / 32)];
    __shared__ T sh_t[kRed];
    __shared__ int sh_i[2];
    __shared__ T rc[6 * kClusterCap];
    const GridCta me = plan[blockIdx.x];
    const int inst = me.inst, v0 = me.v0, v1 = me.v1, c0 = me.c0, nc = me.nc, rank = blockIdx.x - me.c0;
    const int nv = v1 - v0;
    unsigned int* ctl = ctlbuf + (long)kCtlWords * me.slot;
    T* red = redbuf + (long)kRed * me.slot;
    unsigned int round = 0;
    const bool has_blocks = pc.ioff[inst + 1] > pc.ioff[inst];
    const int lane = threadIdx.x & 31, l8 = lane & (kRL - 1), warp = threadIdx.x >> 5, nw = GP_THREADS / 32;
    constexpr int kRows = 32 / kRL;  // rows per warp step
    // ---- stage the CTA's rows in shared memory
    GridRows<T> S;
    S.row = reinterpret_cast<int*>(smem_raw);
    S.dinv = reinterpret_cast<T*>(smem_raw + (((size_t)(nvmax + 1) * 4 + 15) & ~size_t(15)));
    S.val = reinterpret_cast<T*>(smem_raw + grid_smem_fixed(nvmax, sizeof(T), local_deg > 0));
    S.col = reinterpret_cast<int*>(S.val + 9L * cap_blocks);
    T* ya = S.dinv + 9 * nvmax;  // polynomial preconditioner: two iterates and their sum (local_deg > 0 only)
    T* yb = ya + 3 * nvmax;
    T* yz = yb + 3 * nvmax;
    const int kb0 = rowptr[v0];
    const int nbk = rowptr[v1] - kb0;
    S.ncache = min(nbk, cap_blocks);
    for (int i = threadIdx.x; i <= nv; i += GP_THREADS) S.row[i] = rowptr[v0 + i] - kb0;
    for (int i = threadIdx.x; i < 9 * nv; i += GP_THREADS) S.dinv[i] = dinv[9L * v0 + i];
    for (int i = threadIdx.x; i < S.ncache; i += GP_THREADS) S.col[i] = colidx[kb0 + i];
    for (int i = threadIdx.x; i < 9 * S.ncache; i += GP_THREADS) S.val[i] = val[9L * kb0 + i];
    __syncthreads();
    auto barrier = [&]() {
        T none[kRed] = {};
        return inst_round<T>(ctl, red, part, c0, nc, ++round, false, none, none, err, sh_i, sh_t);
    };
    auto allreduce = [&](T a, T bb, T& ra, T& rb) {
        T in[kRed] = {a, bb}, out[kRed];
        const bool ok = inst_round<T>(ctl, red, part, c0, nc, ++round, true, in, out, err, sh_i, sh_t);
        ra = out[0];
        rb = out[1];
        return ok;
    };
    // (a0, a1, a2) = row lv of A times vin; the 8 lanes of a row group each
    // take every 8th block, the caller reduces across the group
    auto row_spmv = [&](int lv, const T* vin, T& a0, T& a1, T& a2) {
        const int v = v0 + lv;
        const int ka = S.row[lv], kz = S.row[lv + 1];
        if (kz <= S.ncache) {
#pragma unroll 4
            for (int k = ka + l8; k < kz; k += kRL) {
                const int c = S.col[k];
                const T* mm = S.val + 9 * k;
                const T x0 = __ldcg(vin + 3 * c), x1 = __ldcg(vin + 3 * c + 1), x2 = __ldcg(vin + 3 * c + 2);
                a0 += mm[0] * x0 + mm[1] * x1 + mm[2] * x2;
                a1 += mm[3] * x0 + mm[4] * x1 + mm[5] * x2;
                a2 += mm[6] * x0 + mm[7] * x1 + mm[8] * x2;
            }
        } else {
            for (int k = ka + l8; k < kz; k += kRL) {
                const int c = colidx[kb0 + k];
                const T* mm = val + 9L * (kb0 + k);
                const T x0 = __ldcg(vin + 3 * c), x1 = __ldcg(vin + 3 * c + 1), x2 = __ldcg(vin + 3 * c + 2);
                a0 += mm[0] * x0 + mm[1] * x1 + mm[2] * x2;
                a1 += mm[3] * x0 + mm[4] * x1 + mm[5] * x2;
                a2 += mm[6] * x0 + mm[7] * x1 + mm[8] * x2;
            }
        }
        const int t1e = trp[v + 1];
        for (int k = trp[v] + l8; k < t1e; k += kRL) {
            const int c = tcol[k];
            if (dbc[c]) continue;
            const T* mm = tval + 9L * k;
            const T x0 = __ldcg(vin + 3 * c), x1 = __ldcg(vin + 3 * c + 1), x2 = __ldcg(vin + 3 * c + 2);
            a0 += mm[0] * x0 + mm[1] * x1 + mm[2] * x2;
            a1 += mm[3] * x0 + mm[4] * x1 + mm[5] * x2;
            a2 += mm[6] * x0 + mm[7] * x1 + mm[8] * x2;
        }
    };
    auto group_sum3 = [&](T& a0, T& a1, T& a2) {
        for (int o = kRL / 2; o > 0; o >>= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        }
    };
    // CTA-local polynomial preconditioner: with y0 = D^-1 v in ya and yz,
    // y_{k+1} = y_k - D^-1 A_loc y_k, z = y_0 + ... + y_deg, where A_loc is
    // the matrix's blocks between this CTA's subdomain rows (block Jacobi over
    // the CTA subdomains, each block inverted by a truncated Neumann series). For an
    // even degree p(S) = sum_k (I - S)^k > 0 for every S = D^-1/2 A_loc D^-1/2
    // > 0, so M^-1 = p(D^-1 A_loc) D^-1 is symmetric positive definite. The
    // result z is written to dst (global) for the instance's next SpMV.
    // The subdomain is the CTA's rows whose blocks all sit in shared memory
    // (a prefix [0, nloc) of its rows); a row past it is its own block
    // (A_loc = D there, so its Neumann terms vanish and it keeps y0 = D^-1 v).
    int nloc = 0;
    if (local_deg > 0) {
        if (threadIdx.x == 0) {
            int lo = 0, hi = nv;  // largest r with S.row[r] <= S.ncache
            while (lo < hi) {
                const int mid = (lo + hi + 1) / 2;
                if (S.row[mid] <= S.ncache) lo = mid;
                else hi = mid - 1;
            }
            sh_i[0] = lo;
        }
        __syncthreads();
        nloc = sh_i[0];
        __syncthreads();
    }
    auto local_poly = [&](T* dst) {
        __syncthreads();
        T* yin = ya;
        T* yout = yb;
        for (int pass = 0; pass < local_deg; ++pass) {
            for (int base = kRows * warp; base < nv; base += kRows * nw) {
                const int lv = base + lane / kRL;
                const bool act = lv < nv;
                const bool inside = lv < nloc;
                const int v = v0 + (act ? lv : 0);
                const bool fixed = act && dbc[v];
                T a0 = 0, a1 = 0, a2 = 0;
                if (inside && !fixed) {
                    const int ka = S.row[lv], kz = S.row[lv + 1];
#pragma unroll 4
                    for (int k = ka + l8; k < kz; k += kRL) {
                        const unsigned lc = (unsigned)(S.col[k] - v0);
                        if (lc >= (unsigned)nloc) continue;
                        const T* mm = S.val + 9 * k;
                        const T x0 = yin[3 * lc], x1 = yin[3 * lc + 1], x2 = yin[3 * lc + 2];
                        a0 += mm[0] * x0 + mm[1] * x1 + mm[2] * x2;
                        a1 += mm[3] * x0 + mm[4] * x1 + mm[5] * x2;
                        a2 += mm[6] * x0 + mm[7] * x1 + mm[8] * x2;
                    }
                }
                group_sum3(a0, a1, a2);
                if (act && l8 < 3) {
                    const T* D = S.dinv + 9 * lv;
                    const T yn = (fixed || !inside)
                                     ? T(0)
                                     : yin[3 * lv + l8] - (D[3 * l8] * a0 + D[3 * l8 + 1] * a1 + D[3 * l8 + 2] * a2);
                    yout[3 * lv + l8] = yn;
                    yz[3 * lv + l8] += yn;
                }
            }
            __syncthreads();
            T* t = yin;
            yin = yout;
            yout = t;
        }
        for (int i = threadIdx.x; i < 3 * nv; i += GP_THREADS) dst[3 * v0 + i] = yz[i];
    };
    if (!has_blocks) {
        // ---- pipelined PCG (Ghysels & Vanroose): one reduction round per
        // iteration, which also publishes the vector the next SpMV gathers.
        // Recurrences: w = A u, m = M w, z = A q, q = M s, s = A p; m is
        // double-buffered because neighbours gather it while it is updated.
        for (int lv = threadIdx.x; lv < nv; lv += GP_THREADS) {
            const int v = v0 + lv;
            const bool fixed = dbc[v];
            T rv[3], uv[3];
            for (int d = 0; d < 3; ++d) rv[d] = fixed ? T(0) : (T)b[3 * v + d];
            grid_precond(S.dinv + 9 * lv, fixed, rv, uv);
            for (int d = 0; d < 3; ++d) {
                const int i3 = 3 * v + d;
                x[i3] = T(0);
                r[i3] = rv[d];
                u[i3] = uv[d];
                z[i3] = T(0);
                q[i3] = T(0);
                sv[i3] = T(0);
                p[i3] = T(0);
                if (local_deg > 0) {  // ya/yz overlay the cached values otherwise
                    ya[3 * lv + d] = uv[d];
                    yz[3 * lv + d] = uv[d];
                }
            }
        }
        if (local_deg > 0) local_poly(u);  // u = M r
        if (!barrier()) return;
        // w = A u, m = M w; partials gamma = r.u, delta = w.u, rho = r.r
        T gam_l = 0, del_l = 0, rho_l = 0;
        for (int base = kRows * warp; base < nv; base += kRows * nw) {
            const int lv = base + lane / kRL;
            const bool act = lv < nv;
            const int v = v0 + (act ? lv : 0);
            const bool fixed = act && dbc[v];
            T a0 = 0, a1 = 0, a2 = 0;
            if (act && !fixed) row_spmv(lv, u, a0, a1, a2);
            group_sum3(a0, a1, a2);
            T wn = 0;
            if (act && l8 < 3) {
                const int i3 = 3 * v + l8;
                const T uo = u[i3], ro = r[i3];
                wn = fixed ? T(0) : (l8 == 0 ? a0 : (l8 == 1 ? a1 : a2));
                w[i3] = wn;
                gam_l += ro * uo;
                del_l += wn * uo;
                rho_l += ro * ro;
            }
            const int gb = lane & ~(kRL - 1);
            const T w0 = __shfl_sync(0xffffffffu, wn, gb), w1 = __shfl_sync(0xffffffffu, wn, gb + 1),
                    w2 = __shfl_sync(0xffffffffu, wn, gb + 2);
            if (act && l8 < 3) {
                const T* D = S.dinv + 9 * lv;
                const T mv = fixed ? T(0) : D[3 * l8] * w0 + D[3 * l8 + 1] * w1 + D[3 * l8 + 2] * w2;
                m0[3 * v + l8] = mv;
                if (local_deg > 0) {
                    ya[3 * lv + l8] = mv;
                    yz[3 * lv + l8] = mv;
                }
            }
        }
        if (local_deg > 0) local_poly(m0);  // m = M w
        T red3[kRed];
        {
            T in[kRed] = {cta_sum1(gam_l, wsh), cta_sum1(del_l, wsh), cta_sum1(rho_l, wsh), T(0)};
            if (!inst_round<T>(ctl, red, part, c0, nc, ++round, true, in, red3, err, sh_i, sh_t)) return;
        }
        T gam = red3[0], del = red3[1];
        const T rho0 = red3[2];
        const double tl = tol_inst ? fmax(tol_inst[inst], rel_tol) : rel_tol;
        const T tol2 = (T)(tl * tl) * rho0;
        int it = 0;
        T* mc = m0;
        T* mn_ = m1;
        T gam_prev = 0, alpha_prev = 0;
        if (rho0 > T(0) && rho0 > tol2) {
            const bool timed = prof && blockIdx.x == 0 && threadIdx.x == 0;
            unsigned long long t0 = timed ? gtimer() : 0, t1;
            for (it = 0; it < max_iters;) {
                T beta = 0, alpha;
                if (it == 0) {
                    alpha = gam / del;
                } else {
                    beta = gam / gam_prev;
                    alpha = gam / (del - beta * gam / alpha_prev);
                }
                if (!(alpha > T(0)) || !(alpha < T(INFINITY))) break;  // breakdown: keep the current x
                gam_l = del_l = rho_l = 0;
                for (int base = kRows * warp; base < nv; base += kRows * nw) {
                    const int lv = base + lane / kRL;
                    const bool act = lv < nv;
                    const int v = v0 + (act ? lv : 0);
                    const bool fixed = act && dbc[v];
                    T mo = 0, zo = 0, qo = 0, so = 0, po = 0, uo = 0, wo = 0, xo = 0, ro = 0;
                    if (act && l8 < 3) {
                        const int i3 = 3 * v + l8;
                        mo = __ldcg(mc + i3);
                        zo = z[i3]; qo = q[i3]; so = sv[i3]; po = p[i3];
                        uo = u[i3]; wo = w[i3]; xo = x[i3]; ro = r[i3];
                    }
                    T a0 = 0, a1 = 0, a2 = 0;
                    if (act && !fixed) row_spmv(lv, mc, a0, a1, a2);
                    group_sum3(a0, a1, a2);
                    T wn = 0;
                    if (act && l8 < 3) {
                        const int i3 = 3 * v + l8;
                        const T n = fixed ? T(0) : (l8 == 0 ? a0 : (l8 == 1 ? a1 : a2));
                        const T zn = n + beta * zo, qn = mo + beta * qo, sn = wo + beta * so, pn = uo + beta * po;
                        const T xn = xo + alpha * pn, rn = ro - alpha * sn, un = uo - alpha * qn;
                        wn = wo - alpha * zn;
                        z[i3] = zn; q[i3] = qn; sv[i3] = sn; p[i3] = pn;
                        x[i3] = xn; r[i3] = rn; u[i3] = un; w[i3] = wn;
                        gam_l += rn * un;
                        del_l += wn * un;
                        rho_l += rn * rn;
                    }
                    const int gb = lane & ~(kRL - 1);
                    const T w0 = __shfl_sync(0xffffffffu, wn, gb), w1 = __shfl_sync(0xffffffffu, wn, gb + 1),
                            w2 = __shfl_sync(0xffffffffu, wn, gb + 2);
                    if (act && l8 < 3) {
                        const T* D = S.dinv + 9 * lv;
                        const T mv = fixed ? T(0) : D[3 * l8] * w0 + D[3 * l8 + 1] * w1 + D[3 * l8 + 2] * w2;
                        mn_[3 * v + l8] = mv;
                        if (local_deg > 0) {
                            ya[3 * lv + l8] = mv;
                            yz[3 * lv + l8] = mv;
                        }
                    }
                }
                if (local_deg > 0) local_poly(mn_);  // m = M w
                T in[kRed] = {cta_sum1(gam_l, wsh), cta_sum1(del_l, wsh), cta_sum1(rho_l, wsh), T(0)};
                if (timed) { t1 = gtimer(); prof[0] += t1 - t0; t0 = t1; }
                if (!inst_round<T>(ctl, red, part, c0, nc, ++round, true, in, red3, err, sh_i, sh_t)) return;
                if (timed) { t1 = gtimer(); prof[1] += t1 - t0; t0 = t1; prof[4] += 1; }
                ++it;
                if (red3[2] <= tol2) break;
                T* tmp = mc;
                mc = mn_;
                mn_ = tmp;
                gam_prev = gam;
                alpha_prev = alpha;
                gam = red3[0];
                del = red3[1];
            }
        }
        if (rank == 0 && threadIdx.x == 0) iters_out[inst] = it;
        return;
    }
    // r = b, x = 0, z = M^{-1} r, p = q = 0
    T rr_l = 0, rz_l = 0;
    for (int lv = threadIdx.x; lv < nv; lv += GP_THREADS) {
        const int v = v0 + lv;
        const bool fixed = dbc[v];
        T rv[3], zv[3];
        for (int d = 0; d < 3; ++d) {
            rv[d] = fixed ? T(0) : (T)b[3 * v + d];
            x[3 * v + d] = T(0);
            r[3 * v + d] = rv[d];
            p[3 * v + d] = T(0);
            q[3 * v + d] = T(0);
            rr_l += rv[d] * rv[d];
        }
        if (pc.vcl[v] < 0) {
            grid_precond(S.dinv + 9 * lv, fixed, rv, zv);
            for (int d = 0; d < 3; ++d) {
                z[3 * v + d] = zv[d];
                if (!has_blocks) rz_l += rv[d] * zv[d];
            }
        }
    }
    if (has_blocks) {
        if (!barrier()) return;
        apply_blocks(pc, inst, rank, nc, dinv, dbc, r, z, (T*)nullptr, rc);
        if (!barrier()) return;
        for (int lv = threadIdx.x; lv < nv; lv += GP_THREADS)
            for (int d = 0; d < 3; ++d) rz_l += r[3 * (v0 + lv) + d] * __ldcg(z + 3 * (v0 + lv) + d);
    }
    T rr_c, rz_c = cta_reduce2(rz_l, rr_l, wsh, rr_c);
    T rz, rr0;
    if (!allreduce(rz_c, rr_c, rz, rr0)) return;
    const double tl = tol_inst ? fmax(tol_inst[inst], rel_tol) : rel_tol;
    const T tol2 = (T)(tl * tl) * rr0;
    T beta = 0;
    int it = 0;
    if (rr0 > T(0) && rr0 > tol2) {
        const bool timed = prof && blockIdx.x == 0 && threadIdx.x == 0;
        unsigned long long t0 = timed ? gtimer() : 0, t1;
        for (it = 0; it < max_iters;) {
            // w = A z on this CTA's rows (8 lanes per row, 4 rows per warp);
            // lane d < 3 of each row then forms p = z + beta p, q = w + beta q
            // for component d
            T pq_l = 0;
            for (int base = kRows * warp; base < nv; base += kRows * nw) {
                const int lv = base + lane / kRL;
                const bool act = lv < nv;
                const int v = v0 + (act ? lv : 0);
                const bool fixed = act && dbc[v];
                T zo = 0, po = 0, qo = 0;
                if (act && l8 < 3) {
                    zo = __ldcg(z + 3 * v + l8);
                    po = p[3 * v + l8];
                    qo = q[3 * v + l8];
                }
                T a0 = 0, a1 = 0, a2 = 0;
                if (act && !fixed) {
                    const int ka = S.row[lv], kz = S.row[lv + 1];
                    if (kz <= S.ncache) {
                        for (int k = ka + l8; k < kz; k += kRL) {
                            const int c = S.col[k];
                            const T* m = S.val + 9 * k;
                            const T x0 = __ldcg(z + 3 * c), x1 = __ldcg(z + 3 * c + 1), x2 = __ldcg(z + 3 * c + 2);
                            a0 += m[0] * x0 + m[1] * x1 + m[2] * x2;
                            a1 += m[3] * x0 + m[4] * x1 + m[5] * x2;
                            a2 += m[6] * x0 + m[7] * x1 + m[8] * x2;
                        }
                    } else {
                        for (int k = ka + l8; k < kz; k += kRL) {
                            const int c = colidx[kb0 + k];
                            const T* m = val + 9L * (kb0 + k);
                            const T x0 = __ldcg(z + 3 * c), x1 = __ldcg(z + 3 * c + 1), x2 = __ldcg(z + 3 * c + 2);
                            a0 += m[0] * x0 + m[1] * x1 + m[2] * x2;
                            a1 += m[3] * x0 + m[4] * x1 + m[5] * x2;
                            a2 += m[6] * x0 + m[7] * x1 + m[8] * x2;
                        }
                    }
                    const int t1e = trp[v + 1];
                    for (int k = trp[v] + l8; k < t1e; k += kRL) {
                        const int c = tcol[k];
                        if (dbc[c]) continue;
                        const T* m = tval + 9L * k;
                        const T x0 = __ldcg(z + 3 * c), x1 = __ldcg(z + 3 * c + 1), x2 = __ldcg(z + 3 * c + 2);
                        a0 += m[0] * x0 + m[1] * x1 + m[2] * x2;
                        a1 += m[3] * x0 + m[4] * x1 + m[5] * x2;
                        a2 += m[6] * x0 + m[7] * x1 + m[8] * x2;
                    }
                }
                for (int o = kRL / 2; o > 0; o >>= 1) {
                    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
                    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
                    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
                }
                if (act && l8 < 3) {
                    // DBC rows: A is the identity there, so w = z
                    const T w = fixed ? zo : (l8 == 0 ? a0 : (l8 == 1 ? a1 : a2));
                    const T pn = zo + beta * po;
                    const T qn = w + beta * qo;
                    p[3 * v + l8] = pn;
                    q[3 * v + l8] = qn;
                    pq_l += pn * qn;
                }
            }
            T d0, pq_c = cta_reduce2(pq_l, T(0), wsh, d0);
            if (timed) { t1 = gtimer(); prof[0] += t1 - t0; t0 = t1; }
            T pq;
            if (!allreduce(pq_c, T(0), pq, d0)) return;
            if (timed) { t1 = gtimer(); prof[1] += t1 - t0; t0 = t1; }
            if (!(pq > T(0))) break;
            const T alpha = rz / pq;
            // x += alpha p; r -= alpha q; z = M^{-1} r (r.z in the same pass
            // unless contact blocks write z of other CTAs' rows)
            T rrn_l = 0, rzn_l = 0;
            for (int lv = threadIdx.x; lv < nv; lv += GP_THREADS) {
                const int v = v0 + lv;
                T rv[3], zv[3];
                for (int d = 0; d < 3; ++d) {
                    x[3 * v + d] += alpha * p[3 * v + d];
                    rv[d] = r[3 * v + d] - alpha * q[3 * v + d];
                    r[3 * v + d] = rv[d];
                    rrn_l += rv[d] * rv[d];
                }
                if (pc.vcl[v] < 0) {
                    grid_precond(S.dinv + 9 * lv, dbc[v] != 0, rv, zv);
                    for (int d = 0; d < 3; ++d) {
                        z[3 * v + d] = zv[d];
                        if (!has_blocks) rzn_l += rv[d] * zv[d];
                    }
                }
            }
            if (has_blocks) {
                if (!barrier()) return;
                apply_blocks(pc, inst, rank, nc, dinv, dbc, r, z, (T*)nullptr, rc);
                if (!barrier()) return;
                for (int lv = threadIdx.x; lv < nv; lv += GP_THREADS)
                    for (int d = 0; d < 3; ++d) rzn_l += r[3 * (v0 + lv) + d] * __ldcg(z + 3 * (v0 + lv) + d);
            }
            T rrn_c, rzn_c = cta_reduce2(rzn_l, rrn_l, wsh, rrn_c);
            if (timed) { t1 = gtimer(); prof[2] += t1 - t0; t0 = t1; }
            T rzn, rrn;
            if (!allreduce(rzn_c, rrn_c, rzn, rrn)) return;
            if (timed) { t1 = gtimer(); prof[3] += t1 - t0; t0 = t1; prof[4] += 1; }
            ++it;
            if (rrn <= tol2) break;
            beta = rzn / rz;
            rz = rzn;
        }
    }
    if (rank == 0 && threadIdx.x == 0) iters_out[inst] = it;
}

}  // namespace

// ---------------------------------------------------------------- host side
int chunk_reduce_off(Arena& A, const int* coff, const double* part, double* out, bool accumulate, cudaStream_t s) {
    (::idp::count_launch(), k_chunk_reduce<<<grid_for(32L * A.nI), kBlock, 0, s>>>(A.nI, coff, part, out, accumulate ? 1 : 0));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int chunk_reduce(Arena& A, Work& W, const Chunk* chunks, int nchunks, const double* part, double* out, cudaStream_t s) {
    (void)W;
    (void)nchunks;
    const int* coff = (chunks == A.tet_chunks) ? A.tet_chunk_off : A.vert_chunk_off;
    return chunk_reduce_off(A, coff, part, out, false, s);
}

int vec_inertia(Arena& A, Work& W, const double* X, double* inst_E, double* g, cudaStream_t s) {
    (void)g;
    if (W[W_CHUNK_SUM].ensure(sizeof(double) * (A.n_vert_chunks + A.n_tet_chunks + 2))) return IDP_ERR_CUDA;
    double* part = W[W_CHUNK_SUM].as<double>();
    (::idp::count_launch(), k_inertia_energy<<<A.n_vert_chunks, kBlock, 0, s>>>(A.vert_chunks, A.active, A.mass, X, A.Xtilde, part));
    return chunk_reduce_off(A, A.vert_chunk_off, part, inst_E, false, s);
}

int grad_gather_tet(Arena& A, Work& W, const double* X, double* g, cudaStream_t s) {
    (::idp::count_launch(), k_grad_gather_tet<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.vert_corner_ptr, A.vert_corner,
                                                       W[W_TET_GRAD].as<double>(), A.mass, X, A.Xtilde, g));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int vec_axpy_trial(Arena& A, const double* Xprev, const double* dir, double* Xout, cudaStream_t s) {
    (::idp::count_launch(), k_axpy_trial<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.alpha, Xprev, dir, Xout));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int vec_zero_dbc(Arena& A, double* g, cudaStream_t s) {
    (::idp::count_launch(), k_zero_dbc<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.dbc, g));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int assemble(Arena& A, Work& W, const ContactSet& cs, bool fp64, cudaStream_t s) {
    (void)cs;
    size_t el = fp64 ? sizeof(double) : sizeof(float);
    if (W[W_BSR_VAL].ensure(el * 9 * (A.B + 1)) || W[W_DIAG_INV].ensure(el * 9 * (A.V + 1))) return IDP_ERR_CUDA;
    const int* trp = W[W_TAIL_ROWPTR].as<int>();
    const int* tcol = W[W_TAIL_COL].as<int>();
    if (fp64) {
        (::idp::count_launch(), k_assemble_tet<double><<<grid_for(A.B), kBlock, 0, s>>>(A.B, A.src_ptr, A.src, W[W_TET_HESS].as<double>(), A.brow,
                                                                A.colidx, A.mass, A.dbc, A.vinst, A.active, A.fvol, A.h, A.dstiff, A.dbc_excl,
                                                                W[W_BSR_VAL].as<double>()));
        (::idp::count_launch(), k_diag_inv<double><<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.diagblk, W[W_BSR_VAL].as<double>(), trp, tcol,
                                                            W[W_TAIL_VAL].as<double>(), A.dbc, A.vinst, A.active,
                                                            W[W_DIAG_INV].as<double>()));
    } else {
        (::idp::count_launch(), k_assemble_tet<float><<<grid_for(A.B), kBlock, 0, s>>>(A.B, A.src_ptr, A.src, W[W_TET_HESS].as<float>(), A.brow,
                                                               A.colidx, A.mass, A.dbc, A.vinst, A.active, A.fvol, A.h, A.dstiff, A.dbc_excl,
                                                               W[W_BSR_VAL].as<float>()));
        (::idp::count_launch(), k_diag_inv<float><<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.diagblk, W[W_BSR_VAL].as<float>(), trp, tcol,
                                                           W[W_TAIL_VAL].as<float>(), A.dbc, A.vinst, A.active,
                                                           W[W_DIAG_INV].as<float>()));
    }
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int hessian_apply(Arena& A, Work& W, bool fp64, const double* x, double* y, cudaStream_t s) {
    const int* trp = W[W_TAIL_ROWPTR].as<int>();
    const int* tcol = W[W_TAIL_COL].as<int>();
    if (fp64)
        (::idp::count_launch(), k_spmv_plain<double><<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.rowptr, A.colidx,
                                                              W[W_BSR_VAL].as<double>(), trp, tcol,
                                                              W[W_TAIL_VAL].as<double>(), A.dbc, x, y));
    else
        (::idp::count_launch(), k_spmv_plain<float><<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.rowptr, A.colidx,
                                                             W[W_BSR_VAL].as<float>(), trp, tcol,
                                                             W[W_TAIL_VAL].as<float>(), A.dbc, x, y));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

// PCG on b (FP64 rhs), result added to nothing: x (type T) holds the solution
template <class T>
static int pcg_inner(Arena& A, Work& W, const double* b, double rel_tol, int max_iters, std::vector<int>& iters,
                     T** xout, cudaStream_t s) {
    const int nI = A.nI;
    long n3 = 3 * A.V;
    if (W[W_PCG_VEC].ensure(sizeof(T) * 10 * (n3 + 4))) return IDP_ERR_CUDA;
    T* base = W[W_PCG_VEC].as<T>();
    T *x = base, *r = base + n3 + 4, *z = r + n3 + 4, *p = z + n3 + 4, *Ap = p + n3 + 4;
    T *pu = Ap + n3 + 4, *pw = pu + n3 + 4, *psv = pw + n3 + 4, *pm0 = psv + n3 + 4, *pm1 = pm0 + n3 + 4;
    const T* val = W[W_BSR_VAL].as<T>();
    const T* dinv = W[W_DIAG_INV].as<T>();
    const int* trp = W[W_TAIL_ROWPTR].as<int>();
    const int* tcol = W[W_TAIL_COL].as<int>();
    const T* tval = W[W_TAIL_VAL].as<T>();
    // instances up to W.grid_min_v vertices: one thread-block cluster each,
    // grouped by cluster size (one launch per size); larger ones: grid PCG
    std::vector<unsigned char> act(nI), small(nI, 0), large(nI, 0);
    IDP_CUDA_TRY(cudaMemcpyAsync(act.data(), A.active, nI, cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaStreamSynchronize(s));
    bool any_small = false, any_large = false;
    std::vector<int> by_size[5];  // cluster sizes 1, 2, 4, 8, 16
    for (int i = 0; i < nI; ++i) {
        if (!act[i]) continue;
        long vi = A.v_off[i + 1] - A.v_off[i];
        if (vi > W.grid_min_v) { large[i] = 1; any_large = true; continue; }
        small[i] = 1;
        any_small = true;
        // cluster size from the instance's own size only (one CTA per ~160
        // vertices, at most 16), so its reduction order, hence its result,
        // does not depend on what else is solved in the launch
        int k = 0;
        while (k < 4 && (1L << k) * kClusterCtaVertices < vi) ++k;
        by_size[k].push_back(i);
    }
    if (W[W_MISC2].ensure(sizeof(int) * (2 * nI + 64))) return IDP_ERR_CUDA;
    int* d_list = W[W_MISC2].as<int>();
    int* d_iters = d_list + nI + 32;
    iters.assign(nI, 0);
    if (any_small) {
        std::vector<int> flat;
        for (int k = 0; k < 5; ++k) flat.insert(flat.end(), by_size[k].begin(), by_size[k].end());
        IDP_CUDA_TRY(cudaMemcpyAsync(d_list, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice, s));
        static std::atomic<bool> attr_set{false};  // one per instantiation
        if (!attr_set.load()) {
            cudaFuncSetAttribute(k_pcg_cluster<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            attr_set.store(true);
        }
        ClusterPC<T> pcb;
        pcb.vcl = W.cl.vcl;
        pcb.ioff = W.cl.ioff;
        pcb.off = W.cl.off;
        pcb.vert = W.cl.vert;
        pcb.doff = W.cl.doff;
        pcb.ok = W.cl.ok;
        pcb.Kinv = W.cl.n > 0 ? W[W_CL_DENSE].as<T>() + W.cl.dense : nullptr;
        W.timer.start(PhaseTimer::PCG, s);
        int base = 0;
        for (int k = 0; k < 5; ++k) {
            int n = (int)by_size[k].size();
            if (!n) continue;
            int cs = 1 << k;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(n * cs);
            cfg.blockDim = dim3(CL_THREADS);
            cfg.stream = s;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = cs;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            const int* lst = d_list + base;
            ::idp::count_launch();
            IDP_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_pcg_cluster<T>, lst, (const int*)A.d_v_off, (const int*)A.rowptr,
                                            (const int*)A.colidx, val, trp, tcol, tval, (const unsigned char*)A.dbc,
                                            dinv, pcb, b, x, r, z, p, Ap, (const double*)W.tol_inst, rel_tol,
                                            max_iters, d_iters));
            W.stats.pcg_launches += 1;
            base += n;
        }
        W.timer.stop(s);
        std::vector<int> hit(nI);
        IDP_CUDA_TRY(cudaMemcpyAsync(hit.data(), d_iters, sizeof(int) * nI, cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        for (int i = 0; i < nI; ++i)
            if (small[i]) iters[i] = hit[i];
    }
    auto account = [&](const std::vector<unsigned char>& which) {
        for (int i = 0; i < nI; ++i)
            if (which[i]) {
                W.stats.pcg_iters += iters[i];
                if ((int)W.pcg_bytes_per_iter.size() == nI)
                    W.stats.pcg_bytes += (double)iters[i] * W.pcg_bytes_per_iter[i] * (sizeof(T) / 4.0);
            }
    };
    account(small);
    if (!any_large) {
        *xout = x;
        return IDP_OK;
    }
    // large instances: grid-wide PCG, in waves of at most gmax CTAs
    static std::atomic<int> gmax_cache{0};  // one per instantiation
    int gmax = gmax_cache.load();
    if (!gmax) {
        int dev = 0, nsm = 0, per = 0;
        IDP_CUDA_TRY(cudaGetDevice(&dev));
        IDP_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        IDP_CUDA_TRY(cudaFuncSetAttribute(k_pcg_grid<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGridSmem));
        IDP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcg_grid<T>, GP_THREADS, kGridSmem));
        gmax = nsm * per;
        if (gmax <= 0) return IDP_ERR_CUDA;
        gmax_cache.store(gmax);
    }
    const long vper = W.grid_vper;
    std::vector<GridCta> plan;
    std::vector<std::vector<GridCta>> waves;
    int slot = 0;
    for (int i = 0; i < nI; ++i) {
        if (!large[i]) continue;
        const int iv0 = A.v_off[i], iv1 = A.v_off[i + 1];
        const long vi = iv1 - iv0;
        int ncta = (int)std::min<long>((vi + vper - 1) / vper, (long)gmax);
        if ((int)plan.size() + ncta > gmax) {
            waves.push_back(plan);
            plan.clear();
            slot = 0;
        }
        const int c0 = (int)plan.size();
        const long per = (vi + ncta - 1) / ncta;
        for (int k = 0; k < ncta; ++k) {
            GridCta g;
            g.inst = i;
            g.v0 = (int)std::min<long>(iv1, iv0 + k * per);
            g.v1 = (int)std::min<long>(iv1, iv0 + (k + 1) * per);
            g.c0 = c0;
            g.nc = ncta;
            g.slot = slot;
            plan.push_back(g);
        }
        ++slot;
    }
    if (!plan.empty()) waves.push_back(plan);
    // W_PCG_GRID: plan | partials (kRed per CTA) | sums (kRed per instance) | control words | error flag
    const size_t o_part = sizeof(GridCta) * gmax;
    const size_t o_red = o_part + sizeof(T) * kRed * (size_t)gmax;
    const size_t o_ctl = (o_red + sizeof(T) * kRed * (size_t)(nI + 1) + 255) & ~size_t(255);
    const size_t o_err = o_ctl + sizeof(unsigned int) * kCtlWords * (size_t)(nI + 1);
    if (W[W_PCG_GRID].ensure(o_err + 256)) return IDP_ERR_CUDA;
    // phase timers of CTA 0 (spmv, first reduction, update, second reduction, iterations) when profiling
    static const bool profiling = std::getenv("IDP_PROFILE") != nullptr;
    unsigned long long* d_prof = profiling ? reinterpret_cast<unsigned long long*>(W[W_PCG_GRID].as<char>() + o_err + 64)
                                           : nullptr;
    char* gb = W[W_PCG_GRID].as<char>();
    GridCta* d_plan = reinterpret_cast<GridCta*>(gb);
    T* d_part = reinterpret_cast<T*>(gb + o_part);
    T* d_red = reinterpret_cast<T*>(gb + o_red);
    unsigned int* d_ctl = reinterpret_cast<unsigned int*>(gb + o_ctl);
    int* d_err = reinterpret_cast<int*>(gb + o_err);
    ClusterPC<T> pcb;
    pcb.vcl = W.cl.vcl;
    pcb.ioff = W.cl.ioff;
    pcb.off = W.cl.off;
    pcb.vert = W.cl.vert;
    pcb.doff = W.cl.doff;
    pcb.ok = W.cl.ok;
    pcb.Kinv = W.cl.n > 0 ? W[W_CL_DENSE].as<T>() + W.cl.dense : nullptr;
    W.timer.start(PhaseTimer::PCG, s);
    IDP_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    if (d_prof && !W.grid_prof_init) {
        IDP_CUDA_TRY(cudaMemsetAsync(d_prof, 0, 5 * sizeof(unsigned long long), s));
        W.grid_prof_init = true;
    }
    for (auto& wv : waves) {
        const int G = (int)wv.size();
        int nvmax = 1;
        for (const GridCta& g : wv) nvmax = std::max(nvmax, g.v1 - g.v0);
        // the polynomial preconditioner's vectors when they leave room for
        // at least half of the rows' blocks, else block Jacobi for this wave
        long nbmax = 0;
        for (const GridCta& g : wv) nbmax = std::max<long>(nbmax, (long)(A.rowptr_h[g.v1] - A.rowptr_h[g.v0]));
        int deg = W.local_deg;
        long fixed = (long)grid_smem_fixed(nvmax, sizeof(T), deg > 0);
        if (deg > 0 && (kGridSmem - fixed) / (long)(9 * sizeof(T) + 4) < nbmax / 2) {
            deg = 0;
            fixed = (long)grid_smem_fixed(nvmax, sizeof(T), false);
        }
        const int cap_blocks = (int)((kGridSmem - fixed) / (long)(9 * sizeof(T) + 4));
        if (cap_blocks < 0) return IDP_ERR_CAPACITY;  // rows per CTA beyond the shared-memory image
        IDP_CUDA_TRY(cudaMemcpyAsync(d_plan, wv.data(), sizeof(GridCta) * G, cudaMemcpyHostToDevice, s));
        IDP_CUDA_TRY(cudaMemsetAsync(d_ctl, 0, sizeof(unsigned int) * kCtlWords * (nI + 1), s));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(G);
        cfg.blockDim = dim3(GP_THREADS);
        cfg.dynamicSmemBytes = kGridSmem;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        ::idp::count_launch();
        IDP_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_pcg_grid<T>, (const GridCta*)d_plan, cap_blocks, nvmax,
                                        (const int*)A.rowptr,
                                        (const int*)A.colidx, val, trp, tcol, tval, (const unsigned char*)A.dbc, dinv,
                                        pcb, b, x, r, z, p, Ap, pu, pw, psv, pm0, pm1, d_part, d_red, d_ctl, d_err,
                                        (const double*)W.tol_inst, rel_tol, max_iters, d_iters, d_prof, deg));
        W.stats.pcg_launches += 1;
    }
    W.timer.stop(s);
    int herr = 0;
    std::vector<int> hit(nI);
    IDP_CUDA_TRY(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(hit.data(), d_iters, sizeof(int) * nI, cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr) return IDP_ERR_CUDA;  // a barrier wait ran out (never expected)
    if (d_prof) {
        unsigned long long hp[5];
        IDP_CUDA_TRY(cudaMemcpy(hp, d_prof, sizeof(hp), cudaMemcpyDeviceToHost));
        IDP_CUDA_TRY(cudaMemset(d_prof, 0, sizeof(hp)));
        for (int k = 0; k < 5; ++k) W.grid_prof[k] += hp[k];
    }
    for (int i = 0; i < nI; ++i)
        if (large[i]) iters[i] = hit[i];
    account(large);
    *xout = x;
    return IDP_OK;
}

int pcg_solve(Arena& A, Work& W, const ContactSet& cs, bool fp64, const double* rhs, double* sol, double rel_tol,
              int max_iters, std::vector<int>& iters_out, std::vector<double>& relres_out, cudaStream_t s,
              const double* tol_host) {
    (void)cs;
    const int nI = A.nI;
    long n3 = 3 * A.V;
    iters_out.assign(nI, 0);
    relres_out.assign(nI, 0.0);
    if (W[W_PCG_VEC64].ensure(sizeof(double) * (n3 + 4)) ||
        W[W_INST_SUM].ensure(sizeof(double) * 8 * (nI + 1)) || W[W_MISC].ensure(sizeof(double) * (A.n_vert_chunks + 2)))
        return IDP_ERR_CUDA;
    double* res = W[W_PCG_VEC64].as<double>();
    double* inst_rr = W[W_INST_SUM].as<double>();
    double* part = W[W_MISC].as<double>();
    const int* trp = W[W_TAIL_ROWPTR].as<int>();
    const int* tcol = W[W_TAIL_COL].as<int>();
    // only the active instances' solutions are reset: a later solve of some
    // instances (FP64 fallback) must not disturb the others' directions
    (::idp::count_launch(), k_zero_masked<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, sol));
    std::vector<double> b2(nI, 0.0), hrr(nI);
    std::vector<unsigned char> act(nI), act0(nI);
    IDP_CUDA_TRY(cudaMemcpyAsync(act0.data(), A.active, nI, cudaMemcpyDeviceToHost, s));
    // FP64 residual res = b - A sol and its squared norm per instance; the
    // norms are copied to pinned host memory, valid after the next
    // synchronisation of the stream (sync = true waits here)
    double* hres = W.pinned_doubles(nI);
    if (!hres) return IDP_ERR_CUDA;
    auto residual_async = [&]() -> int {
        if (fp64)
            (::idp::count_launch(), k_residual64<double><<<grid_for(A.V, 64), 64, 0, s>>>(A.V, A.vinst, A.active, A.rowptr, A.colidx,
                                                                    W[W_BSR_VAL].as<double>(), trp, tcol,
                                                                    W[W_TAIL_VAL].as<double>(), A.dbc, rhs, sol, res));
        else
            (::idp::count_launch(), k_residual64<float><<<grid_for(A.V, 64), 64, 0, s>>>(A.V, A.vinst, A.active, A.rowptr, A.colidx,
                                                                   W[W_BSR_VAL].as<float>(), trp, tcol,
                                                                   W[W_TAIL_VAL].as<float>(), A.dbc, rhs, sol, res));
        (::idp::count_launch(), k_norm2_chunks<<<A.n_vert_chunks, kBlock, 0, s>>>(A.vert_chunks, A.active, res, part));
        if (chunk_reduce_off(A, A.vert_chunk_off, part, inst_rr, false, s)) return IDP_ERR_CUDA;
        IDP_CUDA_TRY(cudaMemcpyAsync(hres, inst_rr, sizeof(double) * nI, cudaMemcpyDeviceToHost, s));
        return IDP_OK;
    };
    auto residual = [&](std::vector<double>& out) -> int {
        int r = residual_async();
        if (r) return r;
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        out.assign(hres, hres + nI);
        return IDP_OK;
    };
    // |b|^2 (x = 0 gives res = b); read after the first sweep, whose own
    // synchronisation brings it back (every active instance runs sweep 0)
    int rc = residual_async();
    if (rc) return rc;
    bool b2_pending = true;
    bool hrr_current = false;
    const int max_refine = fp64 ? 1 : 8;
    const double inner_tol = fp64 ? rel_tol : std::max(rel_tol, 2e-3);
    std::vector<double> prev(nI, 0.0);
    for (int ref = 0; ref < max_refine; ++ref) {
        // instances whose FP64 residual is already small, or that stopped
        // improving (the FP32 operator cannot resolve them), stop refining
        bool any = false;
        if (ref > 0) {
            if (b2_pending) {  // the first sweep synchronised the stream
                b2.assign(hres, hres + nI);
                b2_pending = false;
                for (int i = 0; i < nI; ++i) prev[i] = b2[i];
            }
            rc = residual(hrr);
            if (rc) return rc;
            hrr_current = true;
            for (int i = 0; i < nI; ++i) {
                const double ti = tol_host ? std::max(rel_tol, tol_host[i]) : rel_tol;
                const bool stalled = act[i] && hrr[i] > 0.25 * prev[i];
                act[i] = act[i] && b2[i] > 0 && hrr[i] > ti * ti * b2[i] && !stalled;
                relres_out[i] = b2[i] > 0 ? std::sqrt(hrr[i] / b2[i]) : 0.0;
                prev[i] = hrr[i];
                any |= act[i] != 0;
            }
        } else {
            for (int i = 0; i < nI; ++i) {
                act[i] = act0[i];
                any |= act[i] != 0;
            }
        }
        if (!any) break;
        hrr_current = false;
        IDP_CUDA_TRY(cudaMemcpyAsync(A.active, act.data(), nI, cudaMemcpyHostToDevice, s));
        std::vector<int> its;
        if (fp64) {
            double* e = nullptr;
            rc = pcg_inner<double>(A, W, res, inner_tol, max_iters, its, &e, s);
            if (rc) break;
            (::idp::count_launch(), k_add_correction<double><<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, e, sol));
        } else {
            float* e = nullptr;
            rc = pcg_inner<float>(A, W, res, inner_tol, max_iters, its, &e, s);
            if (rc) break;
            (::idp::count_launch(), k_add_correction<float><<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, e, sol));
        }
        for (int i = 0; i < nI; ++i)
            if (act[i]) iters_out[i] += its[i];
    }
    IDP_CUDA_TRY(cudaMemcpyAsync(A.active, act0.data(), nI, cudaMemcpyHostToDevice, s));
    if (rc) return rc;
    if (b2_pending) {
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        b2.assign(hres, hres + nI);
    }
    if (!hrr_current) {
        rc = residual(hrr);
        if (rc) return rc;
    }
    for (int i = 0; i < nI; ++i) relres_out[i] = b2[i] > 0 ? std::sqrt(hrr[i] / b2[i]) : 0.0;
    return IDP_OK;
}

}  // namespace idp
