// Contact-cluster blocks of the PCG preconditioner.
//
// Barrier Hessians couple the 2-4 vertices of a constraint with stiffness
// many orders above the elastic and inertial terms, and 3x3 block-Jacobi
// cannot see those couplings. Vertices linked through constraints are grouped
// (union-find over the constraint stencils, groups larger than kClusterCap
// split in breadth-first order so coupled vertices stay together); every
// group's dense block of the system matrix is gathered and factored
// (Cholesky, then the inverse factor) on the device, one CTA per group, and
// the PCG applies the block inverse to the group's rows. All other vertices keep their 3x3
// block-Jacobi inverse. A block whose factorisation fails falls back to the
// 3x3 inverses of its vertices.
#include <algorithm>
#include <deque>
#include <numeric>
#include <vector>
#include <atomic>
#include "engine.hpp"

namespace idp {

namespace {

template <class T>
__global__ void k_cl_gather(int ncl, const int* __restrict__ off, const int* __restrict__ vert,
                            const int* __restrict__ vcl, const int* __restrict__ vloc,
                            const long long* __restrict__ doff, const int* __restrict__ rowptr,
                            const int* __restrict__ colidx, const T* __restrict__ val, const int* __restrict__ trp,
                            const int* __restrict__ tcol, const T* __restrict__ tval,
                            const unsigned char* __restrict__ dbc, T* __restrict__ K) {
    int c = blockIdx.x;
    int n = off[c + 1] - off[c], N = 3 * n;
    T* Kc = K + doff[c];
    for (long i = threadIdx.x; i < (long)N * N; i += blockDim.x) Kc[i] = T(0);
    __syncthreads();
    for (int li = threadIdx.x; li < n; li += blockDim.x) {
        int v = vert[off[c] + li];
        if (dbc[v]) {
            for (int a = 0; a < 3; ++a) Kc[(long)(3 * li + a) * N + 3 * li + a] = T(1);
            continue;
        }
        for (int k = rowptr[v]; k < rowptr[v + 1]; ++k) {
            int col = colidx[k];
            if (vcl[col] != c) continue;
            int lj = vloc[col];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) Kc[(long)(3 * li + a) * N + 3 * lj + b] += val[9 * (long)k + 3 * a + b];
        }
        for (int k = trp[v]; k < trp[v + 1]; ++k) {
            int col = tcol[k];
            if (dbc[col] || vcl[col] != c) continue;
            int lj = vloc[col];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) Kc[(long)(3 * li + a) * N + 3 * lj + b] += tval[9 * (long)k + 3 * a + b];
        }
    }
}

// Factor every block, one CTA per block, in 32-wide panels:
//  Cholesky K_c = L L^T (right-looking, in place): the diagonal 32x32 tile is
//  factored by one warp in shared memory, the panel below it is solved row by
//  row (thread per row) into shared memory, and the trailing lower triangle
//  takes the rank-32 update from the staged panel (padded rows, no bank
//  conflicts);
//  Y = L^{-1} by block rows: for rows i0..i0+31 every thread owns a column and
//  keeps the 32 row sums in registers while streaming the column of the rows
//  above, then solves with the diagonal tile.
// The PCG applies K_c^{-1} = Y^T Y as z = Y^T (Y r). ok[c] = 0 when a pivot is
// not positive (the block then falls back to 3x3 inverses).
constexpr int kInvThreads = 256;
constexpr int kTB = 32;
constexpr int kNMax = 3 * kClusterCap;

template <class T>
size_t invert_smem_bytes() {
    const size_t pan = (size_t)kNMax * (kTB + 1), rows = (size_t)kTB * (kNMax + 1);
    return sizeof(T) * ((pan > rows ? pan : rows) + (size_t)kTB * (kTB + 1)) + 64;
}

template <class T>
__global__ void __launch_bounds__(kInvThreads) k_cl_invert(int ncl, const int* __restrict__ off,
                                                           const long long* __restrict__ doff, T* __restrict__ K,
                                                           T* __restrict__ Ybuf, int* __restrict__ ok) {
    extern __shared__ __align__(16) unsigned char inv_smem[];
    T* big = reinterpret_cast<T*>(inv_smem);                                  // panel or row tile
    T* dsm = big + (kNMax * (kTB + 1) > kTB * (kNMax + 1) ? kNMax * (kTB + 1) : kTB * (kNMax + 1));  // TB x (TB+1)
    __shared__ int fail;
    const int c = blockIdx.x;
    const int N = 3 * (off[c + 1] - off[c]);
    T* L = K + doff[c];
    T* Y = Ybuf + doff[c];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = kInvThreads / 32;
    if (tid == 0) fail = 0;
    __syncthreads();
    // ---- Cholesky
    for (int k0 = 0; k0 < N; k0 += kTB) {
        const int kw = min(kTB, N - k0);
        for (int e = tid; e < kw * kw; e += kInvThreads) {
            const int r = e / kw, q = e % kw;
            dsm[r * (kTB + 1) + q] = L[(long)(k0 + r) * N + k0 + q];
        }
        __syncthreads();
        if (warp == 0) {
            for (int j = 0; j < kw; ++j) {
                const T d = dsm[j * (kTB + 1) + j];
                if (!(d > T(0))) {
                    if (lane == 0) fail = 1;
                    break;
                }
                const T ljj = sqrt(d);
                __syncwarp();
                if (lane == j) dsm[j * (kTB + 1) + j] = ljj;
                if (lane > j && lane < kw) dsm[lane * (kTB + 1) + j] /= ljj;
                __syncwarp();
                if (lane > j && lane < kw) {
                    const T lij = dsm[lane * (kTB + 1) + j];
                    for (int q = j + 1; q <= lane; ++q) dsm[lane * (kTB + 1) + q] -= lij * dsm[q * (kTB + 1) + j];
                }
                __syncwarp();
            }
        }
        __syncthreads();
        if (fail) {
            if (tid == 0) ok[c] = 0;
            return;
        }
        for (int e = tid; e < kw * kw; e += kInvThreads) {
            const int r = e / kw, q = e % kw;
            if (q <= r) L[(long)(k0 + r) * N + k0 + q] = dsm[r * (kTB + 1) + q];
        }
        // panel rows below: x L_kk^T = a, staged in big[(i - k0 - kw) * (kTB + 1) + q]
        const int m0 = k0 + kw, m = N - m0;
        for (int ri = tid; ri < m; ri += kInvThreads) {
            const long i = m0 + ri;
            T x[kTB];
#pragma unroll
            for (int q = 0; q < kTB; ++q) {
                if (q < kw) {
                    T a = L[i * N + k0 + q];
                    for (int t = 0; t < q; ++t) a -= x[t] * dsm[q * (kTB + 1) + t];
                    x[q] = a / dsm[q * (kTB + 1) + q];
                    big[ri * (kTB + 1) + q] = x[q];
                    L[i * N + k0 + q] = x[q];
                }
            }
        }
        __syncthreads();
        // trailing lower triangle: A[i][j] -= panel_i . panel_j
        for (int ri = warp; ri < m; ri += nw) {
            const T* pi = big + ri * (kTB + 1);
            T* Ai = L + (long)(m0 + ri) * N + m0;
            for (int rj = lane; rj <= ri; rj += 32) {
                const T* pj = big + rj * (kTB + 1);
                T acc = 0;
#pragma unroll 8
                for (int q = 0; q < kw; ++q) acc += pi[q] * pj[q];
                Ai[rj] -= acc;
            }
        }
        __syncthreads();
    }
    // ---- Y = L^{-1}, block row by block row
    for (int i0 = 0; i0 < N; i0 += kTB) {
        const int iw = min(kTB, N - i0);
        const int ncol = i0 + iw;
        // rows i0..i0+iw of L (columns < i0) and the diagonal tile
        for (int e = tid; e < iw * ncol; e += kInvThreads) {
            const int r = e / ncol, k = e % ncol;
            const T v = L[(long)(i0 + r) * N + k];
            if (k < i0) big[r * (kNMax + 1) + k] = v;
            else dsm[r * (kTB + 1) + (k - i0)] = v;
        }
        __syncthreads();
        for (int col = tid; col < ncol; col += kInvThreads) {
            T acc[kTB];
#pragma unroll
            for (int r = 0; r < kTB; ++r) acc[r] = T(0);
            for (int k = col; k < i0; ++k) {
                const T ykc = Y[(long)k * N + col];
#pragma unroll
                for (int r = 0; r < kTB; ++r) acc[r] += big[r * (kNMax + 1) + k] * ykc;
            }
#pragma unroll
            for (int r = 0; r < kTB; ++r) {
                if (r < iw) {
                    T v = (col == i0 + r ? T(1) : T(0)) - acc[r];
                    for (int t = 0; t < r; ++t) v -= dsm[r * (kTB + 1) + t] * acc[t];
                    v /= dsm[r * (kTB + 1) + r];
                    acc[r] = v;  // acc[r] now holds y(i0 + r, col)
                    Y[(long)(i0 + r) * N + col] = col <= i0 + r ? v : T(0);
                }
            }
        }
        // columns right of the tile stay zero (Y is lower triangular)
        for (int e = tid; e < iw * (N - ncol); e += kInvThreads) {
            const int r = e / (N - ncol), q = ncol + e % (N - ncol);
            Y[(long)(i0 + r) * N + q] = T(0);
        }
        __syncthreads();
    }
    if (tid == 0) ok[c] = 1;
}

struct DSU {
    std::vector<int> p;
    explicit DSU(int n) : p(n) { std::iota(p.begin(), p.end(), 0); }
    int find(int a) {
        while (p[a] != a) a = p[a] = p[p[a]];
        return a;
    }
    void unite(int a, int b) {
        a = find(a);
        b = find(b);
        if (a != b) p[a < b ? b : a] = a < b ? a : b;
    }
};

}  // namespace

int build_contact_clusters(Arena& A, Work& W, const ContactSet& cs, bool fp64, cudaStream_t s) {
    Work::Clusters& cl = W.cl;
    cl.n = 0;
    cl.nvert = 0;
    const long C = cs.C;
    const int nI = A.nI;
    if (W[W_CL_INT].ensure(sizeof(int) * (2 * A.V + 8 * (nI + 1) + 64))) return IDP_ERR_CUDA;
    int* base = W[W_CL_INT].as<int>();
    if (C <= 0) {
        cl.vcl = base;
        IDP_CUDA_TRY(cudaMemsetAsync(cl.vcl, 0xff, sizeof(int) * A.V, s));
        cl.ioff = base + A.V;
        IDP_CUDA_TRY(cudaMemsetAsync(cl.ioff, 0, sizeof(int) * (nI + 1), s));
        return IDP_OK;
    }
    // constraints to the host (C x 20 bytes)
    std::vector<int4> hc(C);
    std::vector<int> hi(C);
    IDP_CUDA_TRY(cudaMemcpyAsync(hc.data(), W[W_CONS].p, sizeof(int4) * C, cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(hi.data(), W[W_CONS_INST].p, sizeof(int) * C, cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaStreamSynchronize(s));
    // stencil vertices of each constraint (sign encoding of FEM/IPC.h:202-250)
    auto stencil = [](int4 c, int* v) {
        if (c.x >= 0) {
            v[0] = c.x;
            v[1] = c.y;
            v[2] = c.z >= 0 ? c.z : -c.z - 1;
            v[3] = c.w >= 0 ? c.w : -c.w - 1;
            return 4;
        }
        v[0] = -c.x - 1;
        v[1] = c.y;
        if (c.w >= 0) { v[2] = c.z; v[3] = c.w; return 4; }
        if (c.z >= 0) { v[2] = c.z; return 3; }
        return 2;
    };
    // compact the vertices that appear in constraints
    std::vector<int> gid;
    gid.reserve(4 * C);
    for (long k = 0; k < C; ++k) {
        int v[4];
        int nv = stencil(hc[k], v);
        for (int a = 0; a < nv; ++a) gid.push_back(v[a]);
    }
    std::sort(gid.begin(), gid.end());
    gid.erase(std::unique(gid.begin(), gid.end()), gid.end());
    const int m = (int)gid.size();
    auto lid = [&](int v) { return (int)(std::lower_bound(gid.begin(), gid.end(), v) - gid.begin()); };
    DSU dsu(m);
    std::vector<std::vector<int>> adj(m);
    for (long k = 0; k < C; ++k) {
        int v[4];
        int nv = stencil(hc[k], v);
        int l[4];
        for (int a = 0; a < nv; ++a) l[a] = lid(v[a]);
        for (int a = 1; a < nv; ++a) dsu.unite(l[0], l[a]);
        for (int a = 0; a < nv; ++a)
            for (int b = 0; b < nv; ++b)
                if (a != b) adj[l[a]].push_back(l[b]);
    }
    for (auto& a : adj) {
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
    }
    // components in order of their smallest vertex, split breadth-first
    std::vector<std::vector<int>> comps;
    {
        std::vector<int> rootc(m, -1);
        for (int i = 0; i < m; ++i) {
            int r = dsu.find(i);
            if (rootc[r] < 0) {
                rootc[r] = (int)comps.size();
                comps.emplace_back();
            }
            comps[rootc[r]].push_back(i);
        }
    }
    std::vector<std::vector<int>> blocks;
    std::vector<char> taken(m, 0);
    for (auto& comp : comps) {
        if ((int)comp.size() < 2) continue;
        if ((int)comp.size() <= W.cl_cap) {
            blocks.push_back(comp);
            continue;
        }
        for (int st : comp) {
            if (taken[st]) continue;
            std::vector<int> blk;
            std::deque<int> q{st};
            taken[st] = 1;
            while (!q.empty() && (int)blk.size() < W.cl_cap) {
                int u = q.front();
                q.pop_front();
                blk.push_back(u);
                for (int w : adj[u])
                    if (!taken[w] && (int)(blk.size() + q.size()) < W.cl_cap) {
                        taken[w] = 1;
                        q.push_back(w);
                    }
            }
            for (int u : q) taken[u] = 0;  // not placed: left for the next block
            if (blk.size() >= 2) blocks.push_back(blk);
        }
    }
    // sort blocks by instance; device arrays
    std::vector<int> vinst_h(blocks.size());
    {
        // instance of a global vertex from the arena offsets
        for (size_t b = 0; b < blocks.size(); ++b) {
            int v = gid[blocks[b][0]];
            vinst_h[b] = (int)(std::upper_bound(A.v_off.begin(), A.v_off.end(), v) - A.v_off.begin()) - 1;
        }
    }
    std::vector<int> order(blocks.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return vinst_h[a] < vinst_h[b]; });
    std::vector<int> off(1, 0), vert, ioff(nI + 1, 0), vcl(A.V, -1), vloc(A.V, 0);
    std::vector<long long> doff(1, 0);
    int maxn = 0;
    for (int bi = 0; bi < (int)order.size(); ++bi) {
        auto& blk = blocks[order[bi]];
        std::vector<int> vs;
        for (int l : blk) vs.push_back(gid[l]);
        std::sort(vs.begin(), vs.end());
        for (size_t k = 0; k < vs.size(); ++k) {
            vcl[vs[k]] = bi;
            vloc[vs[k]] = (int)k;
        }
        vert.insert(vert.end(), vs.begin(), vs.end());
        off.push_back((int)vert.size());
        long long N = 3LL * (long long)vs.size();
        doff.push_back(doff.back() + N * N);
        ioff[vinst_h[order[bi]] + 1]++;
        maxn = std::max(maxn, (int)vs.size());
    }
    for (int i = 0; i < nI; ++i) ioff[i + 1] += ioff[i];
    const int ncl = (int)order.size();
    cl.n = ncl;
    cl.nvert = (long)vert.size();
    cl.dense = doff.back();
    cl.max_n = maxn;
    // int buffer layout: vcl[V] vloc[V] ioff[nI+1] off[ncl+1] vert[nvert] ok[ncl] | doff (8-byte aligned)
    size_t ints = 2 * (size_t)A.V + (nI + 1) + (ncl + 1) + vert.size() + ncl + 8;
    size_t bytes = sizeof(int) * ints + sizeof(long long) * (ncl + 2) + 64;
    if (W[W_CL_INT].ensure(bytes)) return IDP_ERR_CUDA;
    base = W[W_CL_INT].as<int>();
    cl.vcl = base;
    cl.vloc = cl.vcl + A.V;
    cl.ioff = cl.vloc + A.V;
    cl.off = cl.ioff + (nI + 1);
    cl.vert = cl.off + (ncl + 1);
    int* okp = cl.vert + vert.size();
    cl.ok = okp;
    size_t used = (size_t)(okp + ncl - base);
    used = (used + 1) / 2 * 2;
    cl.doff = reinterpret_cast<long long*>(base + used);
    IDP_CUDA_TRY(cudaMemcpyAsync(cl.vcl, vcl.data(), sizeof(int) * A.V, cudaMemcpyHostToDevice, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(cl.vloc, vloc.data(), sizeof(int) * A.V, cudaMemcpyHostToDevice, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(cl.ioff, ioff.data(), sizeof(int) * (nI + 1), cudaMemcpyHostToDevice, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(cl.off, off.data(), sizeof(int) * (ncl + 1), cudaMemcpyHostToDevice, s));
    if (!vert.empty())
        IDP_CUDA_TRY(cudaMemcpyAsync(cl.vert, vert.data(), sizeof(int) * vert.size(), cudaMemcpyHostToDevice, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(cl.doff, doff.data(), sizeof(long long) * (ncl + 1), cudaMemcpyHostToDevice, s));
    if (ncl == 0) {
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        return IDP_OK;
    }
    size_t el = fp64 ? sizeof(double) : sizeof(float);
    if (W[W_CL_DENSE].ensure(el * 2 * (size_t)(cl.dense + 1))) return IDP_ERR_CUDA;
    const int* trp = W[W_TAIL_ROWPTR].as<int>();
    const int* tcol = W[W_TAIL_COL].as<int>();
    if (fp64) {
        double* K = W[W_CL_DENSE].as<double>();
        (::idp::count_launch(), k_cl_gather<double><<<ncl, 256, 0, s>>>(ncl, cl.off, cl.vert, cl.vcl, cl.vloc, cl.doff, A.rowptr, A.colidx,
                                                  W[W_BSR_VAL].as<double>(), trp, tcol, W[W_TAIL_VAL].as<double>(),
                                                  A.dbc, K));
        static std::atomic<bool> attr_d{false};
        if (!attr_d.load()) {
            IDP_CUDA_TRY(cudaFuncSetAttribute(k_cl_invert<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)invert_smem_bytes<double>()));
            attr_d.store(true);
        }
        (::idp::count_launch(), k_cl_invert<double><<<ncl, kInvThreads, invert_smem_bytes<double>(), s>>>(
                                    ncl, cl.off, cl.doff, K, K + cl.dense, okp));
    } else {
        float* K = W[W_CL_DENSE].as<float>();
        (::idp::count_launch(), k_cl_gather<float><<<ncl, 256, 0, s>>>(ncl, cl.off, cl.vert, cl.vcl, cl.vloc, cl.doff, A.rowptr, A.colidx,
                                                 W[W_BSR_VAL].as<float>(), trp, tcol, W[W_TAIL_VAL].as<float>(), A.dbc,
                                                 K));
        static std::atomic<bool> attr_f{false};
        if (!attr_f.load()) {
            IDP_CUDA_TRY(cudaFuncSetAttribute(k_cl_invert<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)invert_smem_bytes<float>()));
            attr_f.store(true);
        }
        (::idp::count_launch(), k_cl_invert<float><<<ncl, kInvThreads, invert_smem_bytes<float>(), s>>>(
                                    ncl, cl.off, cl.doff, K, K + cl.dense, okp));
    }
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

}  // namespace idp
