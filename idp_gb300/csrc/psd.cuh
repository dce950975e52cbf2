// PSD projection of a small symmetric matrix (n <= 12), following the
// reference's makePD (Math/UTILS.h:10-27: eigen-decompose, clamp negative
// eigenvalues to zero, recompose): a per-thread Cholesky test first (a
// positive definite matrix is left unchanged, chol_pd), else cyclic Jacobi
// rotations by one warp until the off-diagonal part is negligible
// (psd_warp_project).
#pragma once
#include "common.cuh"

namespace idp {
namespace {

template <class T>
__device__ bool chol_pd(const T* A, int n) {
    T L[78];
    for (int j = 0; j < n; ++j) {
        T s = A[j * n + j];
        for (int k = 0; k < j; ++k) s -= L[j * (j + 1) / 2 + k] * L[j * (j + 1) / 2 + k];
        if (!(s > T(0))) return false;
        T ljj = sqrt(s);
        L[j * (j + 1) / 2 + j] = ljj;
        for (int i = j + 1; i < n; ++i) {
            T t = A[i * n + j];
            for (int k = 0; k < j; ++k) t -= L[i * (i + 1) / 2 + k] * L[j * (j + 1) / 2 + k];
            L[i * (i + 1) / 2 + j] = t / ljj;
        }
    }
    return true;
}

// Cyclic Jacobi sweeps run by one warp on an n x n matrix A in shared
// memory (n <= 12), Vm holding the identity. Each rotation of a pair (p, q)
// uses theta = (a_qq - a_pp) / (2 a_pq), t = sign(theta) / (|theta| +
// sqrt(theta^2 + 1)), c = 1 / sqrt(t^2 + 1), s = t c; a sweep visits every
// pair in round-robin (tournament) order, so each step rotates n/2 disjoint
// pairs at once (an odd n gets a dummy index), the rotations' column, row
// and eigenvector updates spread over the lanes. Sweeps stop once the
// squared off-diagonal part is at most 1e-14 (FP32) or 1e-30 (FP64) of the
// squared total, after 20 at most. On return A holds the projection
// V max(Lambda, 0) V^T, symmetric. cs, pq and wv are the warp's scratch (6
// rotations, 12 eigenvalues).
constexpr int kPsdWarps = 8;  // warps per CTA of the warp-per-matrix kernels

template <class T>
__device__ void psd_warp_project(T* A, T* Vm, int n, T (*cs)[2], int (*pq)[2], T* wv, int lane) {
    const int m = n + (n & 1);  // players of the tournament
    const int P = m / 2;         // rotations per step
    for (int sweep = 0; sweep < 20; ++sweep) {
        T off = 0, tot = 0;
        for (int k = lane; k < n * n; k += 32) {
            const T a = A[k];
            tot += a * a;
            if (k / n != k % n) off += a * a;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        if (off <= (sizeof(T) == 4 ? T(1e-14) : T(1e-30)) * tot || off == T(0)) break;
        for (int r = 0; r < m - 1; ++r) {
            if (lane < P) {
                int p = lane == 0 ? r : (r + lane) % (m - 1);
                int q = lane == 0 ? m - 1 : (r - lane + (m - 1)) % (m - 1);
                if (p > q) { const int t = p; p = q; q = t; }
                T c = T(1), sn = T(0);
                if (q < n) {
                    const T apq = A[p * n + q];
                    if (apq != T(0)) {
                        const T app = A[p * n + p], aqq = A[q * n + q];
                        const T theta = (aqq - app) / (T(2) * apq);
                        const T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
                        c = T(1) / sqrt(t * t + T(1));
                        sn = t * c;
                    }
                }
                pq[lane][0] = p;
                pq[lane][1] = q;
                cs[lane][0] = c;
                cs[lane][1] = sn;
            }
            __syncwarp();
            // columns of A and of V: A <- A J, V <- V J
            for (int t = lane; t < 2 * P * n; t += 32) {
                T* M = t < P * n ? A : Vm;
                const int u = t < P * n ? t : t - P * n;
                const int j = u / n, k = u % n;
                const int p = pq[j][0], q = pq[j][1];
                if (q >= n) continue;
                const T c = cs[j][0], sn = cs[j][1];
                const T mp = M[k * n + p], mq = M[k * n + q];
                M[k * n + p] = c * mp - sn * mq;
                M[k * n + q] = sn * mp + c * mq;
            }
            __syncwarp();
            // rows of A: A <- J^T A
            for (int t = lane; t < P * n; t += 32) {
                const int j = t / n, k = t % n;
                const int p = pq[j][0], q = pq[j][1];
                if (q >= n) continue;
                const T c = cs[j][0], sn = cs[j][1];
                const T ap = A[p * n + k], aq = A[q * n + k];
                A[p * n + k] = c * ap - sn * aq;
                A[q * n + k] = sn * ap + c * aq;
            }
            __syncwarp();
        }
    }
    if (lane < n) wv[lane] = A[lane * n + lane] > T(0) ? A[lane * n + lane] : T(0);
    __syncwarp();
    for (int t = lane; t < n * n; t += 32) {
        const int a = t / n, b = t % n;
        T acc = 0;
        for (int k = 0; k < n; ++k) acc += Vm[a * n + k] * wv[k] * Vm[b * n + k];
        A[t] = acc;
    }
    __syncwarp();
    // symmetric by construction up to rounding: mirror the upper triangle
    for (int t = lane; t < n * n; t += 32) {
        const int a = t / n, b = t % n;
        if (a > b) A[t] = A[b * n + a];
    }
    __syncwarp();
}

}  // namespace
}  // namespace idp
