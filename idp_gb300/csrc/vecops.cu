// Small per-vertex and per-constraint kernels of the Newton loop.
#include "engine.hpp"
#include "geom.cuh"

namespace idp {

namespace {

__global__ void k_fill_value(long n, double v, double* __restrict__ a) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

__global__ void k_neg(long n, const double* __restrict__ a, double* __restrict__ o) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) o[i] = -a[i];
}

__global__ void k_copy_masked(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ mask,
                              const double* __restrict__ src, double* __restrict__ dst) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !mask[vinst[v]]) return;
    dst[3 * v] = src[3 * v];
    dst[3 * v + 1] = src[3 * v + 1];
    dst[3 * v + 2] = src[3 * v + 2];
}

__global__ void k_dir_norm2(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                            const double* __restrict__ dir, double* __restrict__ part) {
    __shared__ double sh[kBlock];
    Chunk c = chunks[blockIdx.x];
    double acc = 0;
    if (active[c.inst])
        for (int v = c.begin + threadIdx.x; v < c.end; v += blockDim.x)
            for (int d = 0; d < 3; ++d) acc += dir[3 * v + d] * dir[3 * v + d];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = kBlock / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_velocity(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                           const double* __restrict__ X, const double* __restrict__ Xn, double h, double* __restrict__ v) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V || !active[vinst[i]]) return;
    for (int d = 0; d < 3; ++d) v[3 * i + d] = (X[3 * i + d] - Xn[3 * i + d]) / h;
}

__global__ void k_xtilde(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                         const double* __restrict__ X, const double* __restrict__ v, double h,
                         double* __restrict__ Xt) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V || !active[vinst[i]]) return;
    for (int d = 0; d < 3; ++d) Xt[3 * i + d] = X[3 * i + d] + h * v[3 * i + d];
}

// with a body force (IMPLICIT_EULER.h:195-216): x_tilde = x + (h v + h^2 a),
// a = M^-1 b, each operation rounded on its own in the reference's order
__global__ void k_xtilde_b(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                           const double* __restrict__ X, const double* __restrict__ v, const double* __restrict__ a,
                           double h, double* __restrict__ Xt) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V || !active[vinst[i]]) return;
    const double h2 = __dmul_rn(h, h);
    for (int d = 0; d < 3; ++d)
        Xt[3 * i + d] = __dadd_rn(X[3 * i + d], __dadd_rn(__dmul_rn(h, v[3 * i + d]), __dmul_rn(h2, a[3 * i + d])));
}

// kappa adaptation test of IMPLICIT_EULER.h:566-595 over the previous set
__global__ void k_kappa_check(long C, const int4* __restrict__ cons, const int* __restrict__ cinst,
                              const unsigned char* __restrict__ active, const double* __restrict__ X,
                              const double* __restrict__ d2prev, int* __restrict__ flag) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    int inst = cinst[i];
    if (!active[inst]) return;
    double prev = d2prev[i];
    if (!(prev < 1e-18)) return;
    double cur = geo::stencil_dist2(geo::decode(cons[i]), X);
    if (cur < prev) flag[inst] = 1;
}

// out[v] = in[vsrc[v]] (device order from the caller's), or the reverse
__global__ void k_perm3(long v0, long n, const int* __restrict__ vsrc, const double* __restrict__ in,
                        double* __restrict__ out, int to_device) {
    long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long v = v0 + k, src = vsrc[v];
    if (to_device) {
        out[3 * v] = in[3 * src];
        out[3 * v + 1] = in[3 * src + 1];
        out[3 * v + 2] = in[3 * src + 2];
    } else {
        out[3 * src] = in[3 * v];
        out[3 * src + 1] = in[3 * v + 1];
        out[3 * src + 2] = in[3 * v + 2];
    }
}

}  // namespace

int perm_to_device(Arena& A, long v0, long n, const double* in, double* out, cudaStream_t s) {
    if (n <= 0) return IDP_OK;
    (::idp::count_launch(), k_perm3<<<grid_for(n), kBlock, 0, s>>>(v0, n, A.vsrc, in, out, 1));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int perm_to_caller(Arena& A, long v0, long n, const double* in, double* out, cudaStream_t s) {
    if (n <= 0) return IDP_OK;
    (::idp::count_launch(), k_perm3<<<grid_for(n), kBlock, 0, s>>>(v0, n, A.vsrc, in, out, 0));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int vec_fill(double* a, long n, double v, cudaStream_t s) {
    if (n <= 0) return IDP_OK;
    (::idp::count_launch(), k_fill_value<<<grid_for(n), kBlock, 0, s>>>(n, v, a));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int vec_neg(long n, const double* a, double* out, cudaStream_t s) {
    (::idp::count_launch(), k_neg<<<grid_for(n), kBlock, 0, s>>>(n, a, out));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int vec_copy_masked(Arena& A, const unsigned char* mask, const double* src, double* dst, cudaStream_t s) {
    (::idp::count_launch(), k_copy_masked<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, mask, src, dst));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int vec_dir_norm2(Arena& A, Work& W, const double* dir, double* inst_out, cudaStream_t s) {
    if (W[W_CHUNK_SUM].ensure(sizeof(double) * (A.n_vert_chunks + A.n_tet_chunks + 2))) return IDP_ERR_CUDA;
    double* part = W[W_CHUNK_SUM].as<double>();
    (::idp::count_launch(), k_dir_norm2<<<A.n_vert_chunks, kBlock, 0, s>>>(A.vert_chunks, A.active, dir, part));
    return chunk_reduce_off(A, A.vert_chunk_off, part, inst_out, false, s);
}

int vec_velocity(Arena& A, const double* X, const double* Xn, double h, double* v, cudaStream_t s) {
    (::idp::count_launch(), k_velocity<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, X, Xn, h, v));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int vec_xtilde(Arena& A, const double* X, const double* v, double h, double* Xt, cudaStream_t s, const double* acc) {
    if (acc)
        (::idp::count_launch(), k_xtilde_b<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, X, v, acc, h, Xt));
    else
        (::idp::count_launch(), k_xtilde<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, X, v, h, Xt));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int kappa_check(Arena& A, Work& W, const double* X, const int4* cons, const int* cinst, const double* d2prev, long C,
                int* inst_flag, cudaStream_t s) {
    (void)W;
    if (C <= 0) return IDP_OK;
    (::idp::count_launch(), k_kappa_check<<<grid_for(C), kBlock, 0, s>>>(C, cons, cinst, A.active, X, d2prev, inst_flag));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

}  // namespace idp
