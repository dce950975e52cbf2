// Neo-Hookean tet kernels: energy and inversion check (FP64), first
// Piola-Kirchhoff gradient (FP64) and the PSD-projected 12x12 element Hessian
// (FP32 in mixed mode, FP64 in the plain path).
//
// Reference: Physics/NEOHOOKEAN.h:78-300 (Compute_Psi, Compute_E, PK1,
// Compute_DP_Div_DF), FEM/DEFORMATION_GRADIENT.h:112-144 (F = Ds * IB),
// FEM/ELEM_TO_NODE.h:90-257 (scatter of P * IB^T and of the 12x12 blocks),
// FEM/Shell/INC_POTENTIAL.h:97-109 (det F <= 0 rejects the iterate).
//
// The projected Hessian is assembled from its eigen-modes: the 3x3 block of
// d2E/dsigma2 (projected by its own eigen-decomposition) and, for every
// singular-value pair (i, j), the flip mode (U_i V_j^T + U_j V_i^T)/sqrt2 with
// eigenvalue 2*left and the twist mode (U_i V_j^T - U_j V_i^T)/sqrt2 with
// eigenvalue 2*right — the eigen-decomposition of the reference's 2x2 B
// blocks [[l+r, l-r], [l-r, l+r]]. Each mode Q contributes
// lambda * g g^T with g = dF/dx^T vec(Q), computed as Q * IB^T.
#include <mutex>
#include <cuda.h>
#include "engine.hpp"
#include "prims.cuh"

namespace idp {

namespace {

__device__ __forceinline__ void load_F(const double* __restrict__ X, int4 t, const double* __restrict__ IB, double F[9]) {
    D3 x0 = ld3(X, t.x), x1 = ld3(X, t.y), x2 = ld3(X, t.z), x3 = ld3(X, t.w);
    double Ds[9] = {x1.x - x0.x, x2.x - x0.x, x3.x - x0.x, x1.y - x0.y, x2.y - x0.y, x3.y - x0.y,
                    x1.z - x0.z, x2.z - x0.z, x3.z - x0.z};
    double B[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) B[k] = IB[k];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F[i * 3 + j] = Ds[i * 3 + 0] * B[0 * 3 + j] + Ds[i * 3 + 1] * B[1 * 3 + j] + Ds[i * 3 + 2] * B[2 * 3 + j];
}

template <class T>
__device__ __forceinline__ T det3(const T F[9]) {
    return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) + F[2] * (F[3] * F[7] - F[4] * F[6]);
}

__device__ double block_sum(double v) {
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

// one CTA per chunk of tets of one instance
__global__ void k_tet_energy(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                             const double* __restrict__ X, const int4* __restrict__ tet, const double* __restrict__ IB,
                             const double* __restrict__ vol, const double* __restrict__ lam,
                             const double* __restrict__ mu, double w, double* __restrict__ chunk_E,
                             int* __restrict__ inst_bad) {
    Chunk c = chunks[blockIdx.x];
    if (!active[c.inst]) {
        if (threadIdx.x == 0) chunk_E[blockIdx.x] = 0.0;
        return;
    }
    double acc = 0.0;
    int bad = 0;
    for (int t = c.begin + threadIdx.x; t < c.end; t += blockDim.x) {
        double F[9];
        load_F(X, tet[t], IB + 9 * (long)t, F);
        double J = det3(F);
        if (J <= 0) { bad = 1; continue; }
        double f2 = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k) f2 += F[k] * F[k];
        double lJ = log(J);
        double m = mu[t], l = lam[t];
        acc += w * vol[t] * (m / 2.0 * (f2 - 3.0) - (m - l / 2.0 * lJ) * lJ);
    }
    double s = block_sum(acc);
    if (bad) inst_bad[c.inst] = 1;
    if (threadIdx.x == 0) chunk_E[blockIdx.x] = s;
}

// PK1 stress times IB^T per corner (12 doubles per tet)
__global__ void k_tet_gradient(long T, const int* __restrict__ tinst, const unsigned char* __restrict__ active,
                               const double* __restrict__ X, const int4* __restrict__ tet,
                               const double* __restrict__ IB, const double* __restrict__ vol,
                               const double* __restrict__ lam, const double* __restrict__ mu, double w,
                               double* __restrict__ out) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    if (tinst && !active[tinst[t]]) return;
    double F[9];
    const double* B = IB + 9 * t;
    load_F(X, tet[t], B, F);
    double J = det3(F);
    double C[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8], F[3] * F[7] - F[4] * F[6],
                   F[2] * F[7] - F[1] * F[8], F[0] * F[8] - F[2] * F[6], F[1] * F[6] - F[0] * F[7],
                   F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5], F[0] * F[4] - F[1] * F[3]};
    double lJ = log(J), invJ = 1.0 / J;
    double wv = w * vol[t], m = mu[t], l = lam[t];
    double P[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        double FinvT = C[k] * invJ;
        P[k] = wv * (m * (F[k] - FinvT) + l * lJ * FinvT);
    }
    double r[12];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) r[3 * (a + 1) + d] = B[a * 3 + 0] * P[d * 3 + 0] + B[a * 3 + 1] * P[d * 3 + 1] + B[a * 3 + 2] * P[d * 3 + 2];
#pragma unroll
    for (int d = 0; d < 3; ++d) r[d] = -r[3 + d] - r[6 + d] - r[9 + d];
    double* o = out + 12 * t;
#pragma unroll
    for (int k = 0; k < 12; ++k) o[k] = r[k];
}

// ---- 3x3 symmetric eigen-decomposition by cyclic Jacobi (fixed sweeps)
template <class T>
__device__ __forceinline__ void rot(T A[9], T V[9], int p, int q) {
    T apq = A[p * 3 + q];
    if (apq == T(0)) return;
    T app = A[p * 3 + p], aqq = A[q * 3 + q];
    T theta = (aqq - app) / (T(2) * apq);
    T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
    T c = T(1) / sqrt(t * t + T(1)), s = t * c;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T akp = A[k * 3 + p], akq = A[k * 3 + q];
        A[k * 3 + p] = c * akp - s * akq;
        A[k * 3 + q] = s * akp + c * akq;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T apk = A[p * 3 + k], aqk = A[q * 3 + k];
        A[p * 3 + k] = c * apk - s * aqk;
        A[q * 3 + k] = s * apk + c * aqk;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T vkp = V[k * 3 + p], vkq = V[k * 3 + q];
        V[k * 3 + p] = c * vkp - s * vkq;
        V[k * 3 + q] = s * vkp + c * vkq;
    }
}

template <class T>
__device__ void eig3(T A[9], T w[3], T V[9]) {
#pragma unroll
    for (int k = 0; k < 9; ++k) V[k] = (k % 4 == 0) ? T(1) : T(0);
    for (int sweep = 0; sweep < 8; ++sweep) {
        T off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
        T dia = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
        if (off <= T(1e-30) * dia || off == T(0)) break;
        rot(A, V, 0, 1);
        rot(A, V, 0, 2);
        rot(A, V, 1, 2);
    }
    w[0] = A[0];
    w[1] = A[4];
    w[2] = A[8];
}

// SVD with det U = det V = 1 via the eigen-decomposition of F^T F
template <class T>
__device__ void svd3(const T F[9], T U[9], T S[3], T V[9]) {
    T A[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) A[i * 3 + j] = F[i] * F[j] + F[3 + i] * F[3 + j] + F[6 + i] * F[6 + j];
    T w[3], Ve[9];
    eig3(A, w, Ve);
    // sort descending
    int o0 = 0, o1 = 1, o2 = 2;
    if (w[o0] < w[o1]) { int t = o0; o0 = o1; o1 = t; }
    if (w[o1] < w[o2]) { int t = o1; o1 = o2; o2 = t; }
    if (w[o0] < w[o1]) { int t = o0; o0 = o1; o1 = t; }
    int ord[3] = {o0, o1, o2};
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) V[r * 3 + c] = Ve[r * 3 + ord[c]];
    if (det3(V) < T(0))
#pragma unroll
        for (int r = 0; r < 3; ++r) V[r * 3 + 2] = -V[r * 3 + 2];
    T FV[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) FV[r * 3 + c] = F[r * 3] * V[c] + F[r * 3 + 1] * V[3 + c] + F[r * 3 + 2] * V[6 + c];
    Vec3<T> u0 = mk3(FV[0], FV[3], FV[6]), u1 = mk3(FV[1], FV[4], FV[7]);
    T n0 = sqrt(sqn(u0));
    u0 = (T(1) / n0) * u0;
    u1 = u1 - dot(u1, u0) * u0;
    T n1 = sqrt(sqn(u1));
    if (n1 > T(1e-30)) {
        u1 = (T(1) / n1) * u1;
    } else {
        Vec3<T> tt = fabs(u0.x) < T(0.9) ? mk3(T(1), T(0), T(0)) : mk3(T(0), T(1), T(0));
        u1 = cross(u0, tt);
        u1 = (T(1) / sqrt(sqn(u1))) * u1;
    }
    Vec3<T> u2 = cross(u0, u1);
    U[0] = u0.x; U[1] = u1.x; U[2] = u2.x;
    U[3] = u0.y; U[4] = u1.y; U[5] = u2.y;
    U[6] = u0.z; U[7] = u1.z; U[8] = u2.z;
#pragma unroll
    for (int c = 0; c < 3; ++c) S[c] = U[c] * FV[c] + U[3 + c] * FV[3 + c] + U[6 + c] * FV[6 + c];
}

// rank-1 update of the 10 upper 3x3 blocks with lambda * g g^T
template <class T>
__device__ __forceinline__ void rank1(T H[90], T lambda, const T g[12]) {
    if (lambda <= T(0)) return;
    int k = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = a; b < 4; ++b) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                T ga = lambda * g[3 * a + d];
#pragma unroll
                for (int e = 0; e < 3; ++e) H[k * 9 + d * 3 + e] += ga * g[3 * b + e];
            }
            ++k;
        }
}

// g = dF/dx^T vec(Q) for Q = U * C * V^T given as a dense 3x3
template <class T>
__device__ __forceinline__ void mode_grad(const T Q[9], const T B[9], T g[12]) {
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int d = 0; d < 3; ++d) g[3 * (m + 1) + d] = Q[d * 3] * B[m * 3] + Q[d * 3 + 1] * B[m * 3 + 1] + Q[d * 3 + 2] * B[m * 3 + 2];
#pragma unroll
    for (int d = 0; d < 3; ++d) g[d] = -g[3 + d] - g[6 + d] - g[9 + d];
}

template <class T>
__global__ void k_tet_hessian(long T_, const int* __restrict__ tinst, const unsigned char* __restrict__ active,
                              const double* __restrict__ X, const int4* __restrict__ tet,
                              const double* __restrict__ IB, const double* __restrict__ vol,
                              const double* __restrict__ lam, const double* __restrict__ mu, double w,
                              T* __restrict__ out) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T_) return;
    if (tinst && !active[tinst[t]]) return;
    double Fd[9];
    load_F(X, tet[t], IB + 9 * t, Fd);
    T F[9], B[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) { F[k] = (T)Fd[k]; B[k] = (T)IB[9 * t + k]; }
    T U[9], S[3], V[9];
    svd3(F, U, S, V);
    T u = (T)mu[t], l = (T)lam[t], wv = (T)(w * vol[t]);
    T lp = log(S[0] * S[1] * S[2]);
    T dE[3], A[9];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T inv = T(1) / S[i];
        dE[i] = u * (S[i] - inv) + l * inv * lp;
        T inv2 = inv * inv;
        A[i * 4] = u * (T(1) + inv2) - l * inv2 * (lp - T(1));
    }
    A[1] = A[3] = l / (S[0] * S[1]);
    A[5] = A[7] = l / (S[1] * S[2]);
    A[2] = A[6] = l / (S[2] * S[0]);
    T aw[3], aV[9];
    eig3(A, aw, aV);
    T H[90];
#pragma unroll
    for (int k = 0; k < 90; ++k) H[k] = T(0);
    T Q[9], g[12];
    // A-block modes: Q = U diag(e) V^T
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        T e0 = aV[0 * 3 + m], e1 = aV[1 * 3 + m], e2 = aV[2 * 3 + m];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Q[i * 3 + j] = U[i * 3] * e0 * V[j * 3] + U[i * 3 + 1] * e1 * V[j * 3 + 1] + U[i * 3 + 2] * e2 * V[j * 3 + 2];
        mode_grad(Q, B, g);
        rank1(H, wv * aw[m], g);
    }
    // pair modes (i, j) = (0,1), (1,2), (2,0)
    const T middle = u - l * lp;
    const T rs2 = T(0.70710678118654752440);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        int i = c, j = (c + 1) % 3;
        T left = (u + middle / S[i] / S[j]) / T(2);
        T ss = S[i] + S[j];
        T right = (dE[i] + dE[j]) / (T(2) * (ss < T(1e-6) ? T(1e-6) : ss));
#pragma unroll
        for (int sgn = 0; sgn < 2; ++sgn) {
            T lamk = sgn == 0 ? T(2) * left : T(2) * right;
            if (lamk <= T(0)) continue;
            T sj = sgn == 0 ? T(1) : T(-1);
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int q = 0; q < 3; ++q) Q[r * 3 + q] = rs2 * (U[r * 3 + i] * V[q * 3 + j] + sj * U[r * 3 + j] * V[q * 3 + i]);
            mode_grad(Q, B, g);
            rank1(H, wv * lamk, g);
        }
    }
    T* o = out + 90 * t;
#pragma unroll
    for (int k = 0; k < 90; ++k) o[k] = H[k];
}

}  // namespace

int tet_energy(Arena& A, Work& W, const double* X, double w_h2, double* inst_E, int* inst_bad, cudaStream_t s) {
    if (W[W_CHUNK_SUM].ensure(sizeof(double) * (A.n_tet_chunks + 1))) return IDP_ERR_CUDA;
    (::idp::count_launch(), k_tet_energy<<<A.n_tet_chunks, kBlock, 0, s>>>(A.tet_chunks, A.active, X, A.tet, A.IB, A.vol, A.lam, A.mu, w_h2,
                                                     W[W_CHUNK_SUM].as<double>(), inst_bad));
    return chunk_reduce(A, W, A.tet_chunks, A.n_tet_chunks, W[W_CHUNK_SUM].as<double>(), inst_E, s);
}

int tet_gradient(Arena& A, Work& W, const double* X, double w_h2, double* g_corners_unused, cudaStream_t s) {
    (void)g_corners_unused;
    if (W[W_TET_GRAD].ensure(sizeof(double) * 12 * (A.T + 1))) return IDP_ERR_CUDA;
    (::idp::count_launch(), k_tet_gradient<<<grid_for(A.T), kBlock, 0, s>>>(A.T, nullptr, A.active, X, A.tet, A.IB, A.vol, A.lam, A.mu, w_h2,
                                                     W[W_TET_GRAD].as<double>()));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int tet_hessian(Arena& A, Work& W, const double* X, double w_h2, bool fp64, cudaStream_t s) {
    size_t el = fp64 ? sizeof(double) : sizeof(float);
    // element blocks: 10 per tet, then 6 per elastic-shell face and 10 per hinge
    if (W[W_TET_HESS].ensure(el * 9 * (10 * (A.T + 1) + 6 * A.Fm + 10 * A.Hn))) return IDP_ERR_CUDA;
    if (fp64)
        (::idp::count_launch(), k_tet_hessian<double><<<grid_for(A.T, 128), 128, 0, s>>>(A.T, nullptr, A.active, X, A.tet, A.IB, A.vol, A.lam,
                                                                  A.mu, w_h2, W[W_TET_HESS].as<double>()));
    else
        (::idp::count_launch(), k_tet_hessian<float><<<grid_for(A.T, 128), 128, 0, s>>>(A.T, nullptr, A.active, X, A.tet, A.IB, A.vol, A.lam,
                                                                 A.mu, w_h2, W[W_TET_HESS].as<float>()));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int tet_detcheck(Arena& A, Work& W, const double* X, int* inst_bad, cudaStream_t s) {
    // the energy kernel performs the same det F <= 0 test
    if (W[W_INST_SUM].ensure(sizeof(double) * 8 * (A.nI + 1))) return IDP_ERR_CUDA;
    return tet_energy(A, W, X, 0.0, W[W_INST_SUM].as<double>() + 4 * A.nI, inst_bad, s);
}

namespace {

// ---- allocation-free elastic energy (exported as idp_tet_energy_noalloc)
//
// Some callers cannot allocate device memory while they run: a host
// application that reserves the whole GPU budget up front and hands the
// library only its own buffers (a DCC plug-in or engine fixing one animation
// frame after another), or a latency-bound loop that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree imply. For them this entry
// point evaluates w * sum_t vol_t * Psi(F_t) over caller-owned device arrays
// with the same per-tet arithmetic and the same reduction order as the
// arena path (CTA tree per 1024-tet chunk, then the chunk sums in order),
// using only the fixed scratch below for the chunk sums and the inversion
// flag.
constexpr int kNoAllocMaxChunks = 16384;  // => at most 16,777,216 tets per call
constexpr size_t kNoAllocScratchBytes = sizeof(double) * kNoAllocMaxChunks + 256;
// Held by every GPU that loads the library, until exit (128 KB + 256 B).
// Every call shares it and the last call's contents stay: the flag word is
// cleared at the start of each call, the chunk sums are overwritten.
static __device__ __align__(256) unsigned char g_tet_energy_scratch[kNoAllocScratchBytes];

__global__ void k_tet_energy_noalloc(int T, const int4* __restrict__ tet, const double* __restrict__ X,
                                     const double* __restrict__ IB, const double* __restrict__ vol,
                                     const double* __restrict__ lam, const double* __restrict__ mu, double w,
                                     unsigned char* __restrict__ scratch) {
    double* chunk_E = reinterpret_cast<double*>(scratch);
    int* bad_flag = reinterpret_cast<int*>(scratch + sizeof(double) * kNoAllocMaxChunks);
    const int begin = blockIdx.x * kChunk, end = min(T, begin + kChunk);
    double acc = 0.0;
    int bad = 0;
    for (int t = begin + threadIdx.x; t < end; t += blockDim.x) {
        double F[9];
        load_F(X, tet[t], IB + 9 * (long)t, F);
        double J = det3(F);
        if (J <= 0) { bad = 1; continue; }
        double f2 = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k) f2 += F[k] * F[k];
        double lJ = log(J);
        double m = mu[t], l = lam[t];
        acc += w * vol[t] * (m / 2.0 * (f2 - 3.0) - (m - l / 2.0 * lJ) * lJ);
    }
    double s = block_sum(acc);
    if (bad) *bad_flag = 1;
    if (threadIdx.x == 0) chunk_E[blockIdx.x] = s;
}

__global__ void k_tet_energy_noalloc_sum(int nchunks, const unsigned char* __restrict__ scratch,
                                         double* __restrict__ energy, int* __restrict__ inverted) {
    const double* chunk_E = reinterpret_cast<const double*>(scratch);
    const int* bad_flag = reinterpret_cast<const int*>(scratch + sizeof(double) * kNoAllocMaxChunks);
    double s = 0;
    for (int c = 0; c < nchunks; ++c) s += chunk_E[c];
    *energy = s;
    *inverted = *bad_flag;
}

// Device address of the scratch array, looked up once per device and
// context: a context that is destroyed and re-created (cudaDeviceReset, or a
// primary context released and retained again) reloads the module, so the
// cached address is keyed on the driver's unique id of the current context
// (cuCtxGetId), reached through the runtime's driver entry-point query so
// that the library needs no link to libcuda.
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_addr[kNoAllocMaxDevices] = {};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// unique id of the calling thread's current context + 1 (0: none current, or
// the driver entry points are unavailable); call with g_noalloc_mu held
unsigned long long current_context_key() {
    static bool looked_up = false;
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    if (!looked_up) {
        looked_up = true;
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(f);
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id + 1;
}

}  // namespace

}  // namespace idp

extern "C" int idp_tet_energy_noalloc(int T, const int32_t* tets, const double* X, const double* IB,
                                      const double* vol, const double* lam, const double* mu, double weight,
                                      double* energy, int32_t* inverted, void* stream) {
    using namespace idp;
    if (T < 0 || !energy || !inverted) return IDP_ERR_INVALID_ARG;
    if (T > 0 && (!tets || !X || !IB || !vol || !lam || !mu)) return IDP_ERR_INVALID_ARG;
    if ((long)T > (long)kNoAllocMaxChunks * kChunk) return IDP_ERR_CAPACITY;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return IDP_ERR_CUDA;
    unsigned char* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        const unsigned long long key = current_context_key();
        if (!g_noalloc_addr[dev] || key == 0 || key != g_noalloc_ctx[dev]) {
            // set-up, the first call on this device and context: the
            // symbol's device address (the name itself is only a host-side
            // stand-in); the lookup also makes the device's primary context
            // current when no context was yet
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_tet_energy_scratch) != cudaSuccess || !p) return IDP_ERR_CUDA;
            g_noalloc_addr[dev] = static_cast<unsigned char*>(p);
            g_noalloc_ctx[dev] = current_context_key();
        }
        scratch = g_noalloc_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nchunks = (T + kChunk - 1) / kChunk;
    if (cudaMemsetAsync(scratch + sizeof(double) * kNoAllocMaxChunks, 0, sizeof(int), s) != cudaSuccess)
        return IDP_ERR_CUDA;
    if (nchunks > 0)
        (::idp::count_launch(),
         k_tet_energy_noalloc<<<nchunks, kBlock, 0, s>>>(T, reinterpret_cast<const int4*>(tets), X, IB, vol, lam, mu,
                                                         weight, scratch));
    (::idp::count_launch(), k_tet_energy_noalloc_sum<<<1, 1, 0, s>>>(nchunks, scratch, energy, inverted));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}
