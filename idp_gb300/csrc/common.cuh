// Shared device/host definitions for the GB300 injective-deformation engine.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#define IDP_CUDA_TRY(expr)                                                           \
    do {                                                                             \
        cudaError_t _e = (expr);                                                     \
        if (_e != cudaSuccess) {                                                     \
            std::fprintf(stderr, "idp: CUDA error %s at %s:%d\n", cudaGetErrorString(_e), \
                         __FILE__, __LINE__);                                        \
            return IDP_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)

namespace idp {

constexpr int kBlock = 256;

// host-side count of kernel launches made by this library (every launch
// site is written as (count_launch(), kernel<<<...>>>(...)))
extern thread_local long long g_launch_count;  // per host thread (one thread drives a context at a time)
inline void count_launch() { ++g_launch_count; }

inline int grid_for(long n, int block = kBlock) {
    long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 2147483647L) g = 2147483647L;
    return (int)g;
}

// Chunk of a per-instance element range. Element loops that reduce per
// instance launch one CTA per chunk; chunks never straddle two instances, so
// every per-instance sum is taken in a fixed order that does not depend on
// which other instances share the launch.
struct Chunk {
    int inst;
    int begin;
    int end;
};
constexpr int kChunk = 1024;
// vertices per dense contact-cluster block of the preconditioner (576 x 576)
constexpr int kClusterCap = 192;

// ---- small vector math (templated so FP32 and FP64 paths share code)
template <class T>
struct Vec3 {
    T x, y, z;
};
template <class T>
__host__ __device__ inline Vec3<T> mk3(T a, T b, T c) { return {a, b, c}; }
template <class T>
__host__ __device__ inline Vec3<T> operator-(Vec3<T> a, Vec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T>
__host__ __device__ inline Vec3<T> operator+(Vec3<T> a, Vec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T>
__host__ __device__ inline Vec3<T> operator*(T s, Vec3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T>
__host__ __device__ inline T dot(Vec3<T> a, Vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T>
__host__ __device__ inline T sqn(Vec3<T> a) { return dot(a, a); }
template <class T>
__host__ __device__ inline Vec3<T> cross(Vec3<T> a, Vec3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T>
__host__ __device__ inline T comp(Vec3<T> a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

typedef Vec3<double> D3;
typedef Vec3<float> F3;

__device__ inline D3 ld3(const double* p, int v) { return {p[3 * v], p[3 * v + 1], p[3 * v + 2]}; }
__device__ inline F3 tof(D3 a) { return {(float)a.x, (float)a.y, (float)a.z}; }

// non-negative doubles order like their bit patterns
__device__ inline void atomic_min_nonneg(double* addr, double v) {
    atomicMin(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

}  // namespace idp
