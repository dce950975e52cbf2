// Normal-flow predictor: every surface vertex is pushed along its
// area-weighted outward normal, interior vertices are held in place.
// Normal formula: Update_Normal_Flow_Neumann, FEM/Shell/DISCRETE_SHELL.h:359-395
// (sum over incident surface triangles of cross(X2-X1, X3-X1), normalised).
// The reference applies it as a body force b = magnitude * m_i * n_i, whose
// predictor shift h^2 M^-1 b is h^2 * magnitude * n_i; here the shift `step`
// is given directly and stored as a velocity (x_tilde = x + h v).
// Compiled with --fmad=false: the per-vertex sums run in triangle order with
// the same operations as the oracle, so velocities are bit-identical.
#include "engine.hpp"

namespace idp {

namespace {

__global__ void k_normal_flow(long V, const int* __restrict__ vinst, int sel, const double* __restrict__ X,
                              const int* __restrict__ stri, const int* __restrict__ vtri_ptr,
                              const int* __restrict__ vtri, double step, double h, double* __restrict__ vel) {
    long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    if (sel >= 0 && vinst[v] != sel) return;
    double n0 = 0, n1 = 0, n2 = 0;
    for (int k = vtri_ptr[v]; k < vtri_ptr[v + 1]; ++k) {
        const int f = vtri[k];
        const int a = stri[3 * f], b = stri[3 * f + 1], c = stri[3 * f + 2];
        const double e1x = X[3 * b] - X[3 * a], e1y = X[3 * b + 1] - X[3 * a + 1], e1z = X[3 * b + 2] - X[3 * a + 2];
        const double e2x = X[3 * c] - X[3 * a], e2y = X[3 * c + 1] - X[3 * a + 1], e2z = X[3 * c + 2] - X[3 * a + 2];
        n0 += e1y * e2z - e1z * e2y;
        n1 += e1z * e2x - e1x * e2z;
        n2 += e1x * e2y - e1y * e2x;
    }
    double w = 0;
    const double sq = n0 * n0 + n1 * n1 + n2 * n2;
    if (vtri_ptr[v + 1] > vtri_ptr[v] && sq > 0) w = step / sqrt(sq);
    vel[3 * v] = w * n0 / h;
    vel[3 * v + 1] = w * n1 / h;
    vel[3 * v + 2] = w * n2 / h;
}

}  // namespace

int normal_flow_velocity(Arena& A, int sel, double step, double h, double* vel, cudaStream_t s) {
    if (A.V <= 0) return IDP_OK;
    (::idp::count_launch(),
     k_normal_flow<<<grid_for(A.V), kBlock, 0, s>>>(A.V, A.vinst, sel, A.X, A.stri, A.vtri_ptr, A.vtri, step, h, vel));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

}  // namespace idp
