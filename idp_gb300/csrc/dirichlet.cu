// Moving Dirichlet conditions of the Newton step: the augmented Lagrangian of
// Advance_One_Step_IE_Discrete_Shell (FEM/Shell/IMPLICIT_EULER.h:305-401,
// 701-757) with the penalty of FEM/Shell/DIRICHLET.h. A DBC vertex whose
// target equals its position at the step's start is fixed (projected); the
// others are moved to their targets at once when the CCD step of the
// displacement allows it (alpha = 1), else pulled there by the penalty
// stiff/2 sum m |t - x|^2, whose stiffness the Newton loop doubles until the
// vertices have covered 99 % of the way.
#include "engine.hpp"

namespace idp {
namespace {

// displacement to the target on the DBC vertices of the masked instances
// (zero elsewhere), whether the vertex is already there, and a per-instance
// flag when some DBC vertex has to move (IMPLICIT_EULER.h:309-328)
__global__ void k_dbc_classify(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                               const unsigned char* __restrict__ excl, const double* __restrict__ X,
                               const double* __restrict__ tgt, double* __restrict__ dir,
                               unsigned char* __restrict__ fixed, int* __restrict__ moving) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]]) return;
    double d0 = 0, d1 = 0, d2 = 0;
    unsigned char f = 0;
    if (excl[v]) {
        d0 = tgt[3 * v] - X[3 * v];
        d1 = tgt[3 * v + 1] - X[3 * v + 1];
        d2 = tgt[3 * v + 2] - X[3 * v + 2];
        f = (d0 == 0 && d1 == 0 && d2 == 0) ? 1 : 0;
        if (!f) moving[vinst[v]] = 1;
    }
    dir[3 * v] = d0;
    dir[3 * v + 1] = d1;
    dir[3 * v + 2] = d2;
    fixed[v] = f;
}

// x = target on every DBC vertex of the masked instances (IMPLICIT_EULER.h:385-394)
__global__ void k_dbc_snap(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                           const unsigned char* __restrict__ excl, const double* __restrict__ tgt,
                           double* __restrict__ X) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !active[vinst[v]] || !excl[v]) return;
    X[3 * v] = tgt[3 * v];
    X[3 * v + 1] = tgt[3 * v + 1];
    X[3 * v + 2] = tgt[3 * v + 2];
}

// per vertex chunk of the masked instances whose penalty is on: sum m |t - x|^2
// (Compute_DBC_Energy before its stiff/2 factor, DIRICHLET.h:26-45) and
// sum |t - x|^2 (Compute_DBC_Dist2, :6-24)
__global__ void k_dbc_sums(const Chunk* __restrict__ chunks, const unsigned char* __restrict__ active,
                           const double* __restrict__ stiff, const unsigned char* __restrict__ excl,
                           const double* __restrict__ mass, const double* __restrict__ X,
                           const double* __restrict__ tgt, double* __restrict__ part_w, double* __restrict__ part_d) {
    __shared__ double sw[kBlock], sd[kBlock];
    Chunk c = chunks[blockIdx.x];
    double aw = 0, ad = 0;
    if (active[c.inst] && stiff[c.inst] > 0)
        for (int v = c.begin + threadIdx.x; v < c.end; v += blockDim.x) {
            if (!excl[v]) continue;
            double q = 0;
            for (int d = 0; d < 3; ++d) {
                const double e = tgt[3 * v + d] - X[3 * v + d];
                q += e * e;
            }
            aw += q * mass[v];
            ad += q;
        }
    sw[threadIdx.x] = aw;
    sd[threadIdx.x] = ad;
    __syncthreads();
    for (int st = kBlock / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            sw[threadIdx.x] += sw[threadIdx.x + st];
            sd[threadIdx.x] += sd[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part_w[blockIdx.x] = sw[0];
        part_d[blockIdx.x] = sd[0];
    }
}

// g += stiff m (x - t) on the DBC vertices (Compute_DBC_Gradient, DIRICHLET.h:47-70)
__global__ void k_dbc_grad(long V, const int* __restrict__ vinst, const unsigned char* __restrict__ active,
                           const double* __restrict__ stiff, const unsigned char* __restrict__ excl,
                           const double* __restrict__ mass, const double* __restrict__ X,
                           const double* __restrict__ tgt, double* __restrict__ g) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || !excl[v]) return;
    const int i = vinst[v];
    if (!active[i] || !(stiff[i] > 0)) return;
    const double k = stiff[i] * mass[v];
    for (int d = 0; d < 3; ++d) g[3 * v + d] += k * (X[3 * v + d] - tgt[3 * v + d]);
}

}  // namespace

int dbc_classify(Arena& A, const double* X, double* dir, int* moving, cudaStream_t s) {
    if (!A.dtgt || !A.dfix) return IDP_ERR_STATE;
    (::idp::count_launch(), k_dbc_classify<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.dbc_excl, X,
                                                                          A.dtgt, dir, A.dfix, moving));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int dbc_snap(Arena& A, double* X, cudaStream_t s) {
    if (!A.dtgt) return IDP_ERR_STATE;
    (::idp::count_launch(), k_dbc_snap<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.dbc_excl, A.dtgt, X));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

int dbc_sums(Arena& A, Work& W, const double* X, double* inst_w, double* inst_d, cudaStream_t s) {
    if (!A.dtgt) return IDP_ERR_STATE;
    if (W[W_CHUNK_SUM].ensure(sizeof(double) * (2 * A.n_vert_chunks + 2))) return IDP_ERR_CUDA;
    double* pw = W[W_CHUNK_SUM].as<double>();
    double* pd = pw + A.n_vert_chunks;
    (::idp::count_launch(), k_dbc_sums<<<A.n_vert_chunks, kBlock, 0, s>>>(A.vert_chunks, A.active, A.dstiff, A.dbc_excl,
                                                                        A.mass, X, A.dtgt, pw, pd));
    int rc = chunk_reduce_off(A, A.vert_chunk_off, pw, inst_w, false, s);
    if (!rc) rc = chunk_reduce_off(A, A.vert_chunk_off, pd, inst_d, false, s);
    return rc;
}

int dbc_gradient(Arena& A, const double* X, double* g, cudaStream_t s) {
    if (!A.dtgt) return IDP_ERR_STATE;
    (::idp::count_launch(), k_dbc_grad<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, A.active, A.dstiff, A.dbc_excl,
                                                                       A.mass, X, A.dtgt, g));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

}  // namespace idp
