// PSD projection of a small symmetric matrix (n <= 12), following the
// reference's makePD (Math/UTILS.h:10-27: eigen-decompose, clamp negative
// eigenvalues to zero, recompose): a Cholesky test first (a positive definite
// matrix is left unchanged), else cyclic Jacobi rotations until the
// off-diagonal part is negligible. One thread per matrix.
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

template <class T>
__device__ void make_pd(T* A, int n) {
    if (chol_pd(A, n)) return;
    T V[144];
    for (int i = 0; i < n * n; ++i) V[i] = T(0);
    for (int i = 0; i < n; ++i) V[i * n + i] = T(1);
    for (int sweep = 0; sweep < 20; ++sweep) {
        T off = 0, tot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                T a = A[i * n + j];
                tot += a * a;
                if (i != j) off += a * a;
            }
        if (off <= (sizeof(T) == 4 ? T(1e-14) : T(1e-30)) * tot || off == T(0)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                T apq = A[p * n + q];
                if (apq == T(0)) continue;
                T app = A[p * n + p], aqq = A[q * n + q];
                T theta = (aqq - app) / (T(2) * apq);
                T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
                T c = T(1) / sqrt(t * t + T(1)), s = t * c;
                for (int k = 0; k < n; ++k) {
                    T akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    T apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    T vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    T w[12];
    for (int i = 0; i < n; ++i) w[i] = A[i * n + i] > T(0) ? A[i * n + i] : T(0);
    for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
            T s = 0;
            for (int k = 0; k < n; ++k) s += V[i * n + k] * w[k] * V[j * n + k];
            A[i * n + j] = s;
            A[j * n + i] = s;
        }
}

}  // namespace
}  // namespace idp
