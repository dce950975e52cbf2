// Flow energy of triangle shells (Advance_One_Step_IE_Flow,
// FEM/Shell/DISCRETE_SHELL.h:1113): E = -h/2 x^T L x with, per face f and
// corner i, (L x)_i += vol_f / 6 (x_{i+1} + x_{i+2} - 2 x_i)
// (FEM/Shell/INC_POTENTIAL.h:53-73), gradient -h L x (:191-211) and the
// constant Hessian -h L (:323-339, assembled with the tet blocks in
// solver.cu). The energy is evaluated in its equal edge form
// h/12 sum_f vol_f (|x0-x1|^2 + |x1-x2|^2 + |x2-x0|^2), which avoids the
// cancellation of the x^T L x form (every term is non-negative); the gradient
// per vertex is h/6 sum_f vol_f (2 x_i - x_{i+1} - x_{i+2}) over its faces in
// a fixed order. FP64 throughout.
#include "engine.hpp"

namespace idp {
namespace {

__device__ double block_sum_flow(double v) {
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

__device__ __forceinline__ double sq3(const double* a, const double* b) {
    const double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
    return d0 * d0 + d1 * d1 + d2 * d2;
}

// one CTA per chunk of faces of one instance; fixed tree per chunk
__global__ void k_flow_energy(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                              const double* __restrict__ X, const int* __restrict__ face,
                              const double* __restrict__ fvol, double h, double* __restrict__ part) {
    const Chunk c = chunks[blockIdx.x];
    double acc = 0.0;
    if (active[c.inst])
        for (int f = c.begin + threadIdx.x; f < c.end; f += blockDim.x) {
            const double* x0 = X + 3L * face[3L * f];
            const double* x1 = X + 3L * face[3L * f + 1];
            const double* x2 = X + 3L * face[3L * f + 2];
            acc += h / 12.0 * fvol[f] * (sq3(x0, x1) + sq3(x1, x2) + sq3(x2, x0));
        }
    const double s = block_sum_flow(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// per vertex: its incident faces in ascending order
__global__ void k_flow_gradient(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                                const int* __restrict__ vfp, const int* __restrict__ vf, const int* __restrict__ face,
                                const double* __restrict__ fvol, const double* __restrict__ X, double h,
                                double* __restrict__ g) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    const int k0 = vfp[v], k1 = vfp[v + 1];
    if (k0 == k1) return;
    double s0 = 0, s1 = 0, s2 = 0;
    const double* xv = X + 3 * v;
    for (int k = k0; k < k1; ++k) {
        const int code = vf[k];  // face * 3 + corner
        const int f = code / 3, i = code - 3 * f;
        const double w = h * fvol[f] / 6.0;
        const double* xa = X + 3L * face[3L * f + (i + 1) % 3];
        const double* xb = X + 3L * face[3L * f + (i + 2) % 3];
        s0 += w * (2.0 * xv[0] - xa[0] - xb[0]);
        s1 += w * (2.0 * xv[1] - xa[1] - xb[1]);
        s2 += w * (2.0 * xv[2] - xa[2] - xb[2]);
    }
    g[3 * v] += s0;
    g[3 * v + 1] += s1;
    g[3 * v + 2] += s2;
}

}  // namespace

int flow_energy(Arena& A, Work& W, const double* X, double* inst_E, cudaStream_t s) {
    if (A.F == 0) return IDP_OK;
    if (W[W_CHUNK_SUM].ensure(sizeof(double) * (A.n_face_chunks + A.n_tet_chunks + A.n_vert_chunks + 2)))
        return IDP_ERR_CUDA;
    double* part = W[W_CHUNK_SUM].as<double>();
    (::idp::count_launch(),
     k_flow_energy<<<A.n_face_chunks, kBlock, 0, s>>>(A.face_chunks, A.active, X, A.face, A.fvol, A.h, part));
    return chunk_reduce_off(A, A.face_chunk_off, part, inst_E, true, s);
}

int flow_gradient(Arena& A, const double* X, double* g, cudaStream_t s) {
    if (A.F == 0) return IDP_OK;
    (::idp::count_launch(), k_flow_gradient<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.vert_face_ptr,
                                                                              A.vert_face, A.face, A.fvol, X, A.h, g));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

}  // namespace idp
