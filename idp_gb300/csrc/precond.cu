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

// Factor every block: K_c = L L^T (right-looking Cholesky in place, the
// pivot column staged in shared memory, each warp updating whole rows of the
// trailing triangle with coalesced accesses), then Y = L^{-1} into Ybuf by
// forward substitution on the identity, all columns in lock-step (thread c
// owns column c; row k of Y is read coalesced, L[i][k] is a broadcast).
// The PCG applies K_c^{-1} = Y^T Y as z = Y^T (Y r). ok[c] = 0 when a pivot
// is not positive (the block then falls back to 3x3 inverses).
constexpr int kInvThreads = 1024;

template <class T>
__global__ void __launch_bounds__(kInvThreads) k_cl_invert(int ncl, const int* __restrict__ off,
                                                           const long long* __restrict__ doff, T* __restrict__ K,
                                                           T* __restrict__ Ybuf, int* __restrict__ ok) {
    __shared__ T colj[3 * kClusterCap];
    const int c = blockIdx.x;
    const int N = 3 * (off[c + 1] - off[c]);
    T* L = K + doff[c];
    T* Y = Ybuf + doff[c];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < N; ++j) {
        const T d = L[(long)j * N + j];
        if (!(d > T(0))) {  // every thread sees the same pivot
            if (threadIdx.x == 0) ok[c] = 0;
            return;
        }
        const T ljj = sqrt(d);
        for (int i = j + threadIdx.x; i < N; i += blockDim.x) {
            const T v = i == j ? ljj : L[(long)i * N + j] / ljj;
            L[(long)i * N + j] = v;
            colj[i] = v;
        }
        __syncthreads();
        for (int i = j + 1 + warp; i < N; i += nw) {
            const T lij = colj[i];
            T* Li = L + (long)i * N;
            for (int k = j + 1 + lane; k <= i; k += 32) Li[k] -= lij * colj[k];
        }
        __syncthreads();
    }
    // Y = L^{-1}: row i of Y from rows k < i (columns c <= k are nonzero)
    for (int i = 0; i < N; ++i) {
        const T* Li = L + (long)i * N;
        const T inv = T(1) / Li[i];
        for (int col = threadIdx.x; col < N; col += blockDim.x) {
            T acc = col == i ? T(1) : T(0);
            for (int k = col; k < i; ++k) acc -= Li[k] * Y[(long)k * N + col];
            Y[(long)i * N + col] = col <= i ? acc * inv : T(0);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) ok[c] = 1;
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
        (::idp::count_launch(), k_cl_invert<double><<<ncl, kInvThreads, 0, s>>>(ncl, cl.off, cl.doff, K, K + cl.dense, okp));
    } else {
        float* K = W[W_CL_DENSE].as<float>();
        (::idp::count_launch(), k_cl_gather<float><<<ncl, 256, 0, s>>>(ncl, cl.off, cl.vert, cl.vcl, cl.vloc, cl.doff, A.rowptr, A.colidx,
                                                 W[W_BSR_VAL].as<float>(), trp, tcol, W[W_TAIL_VAL].as<float>(), A.dbc,
                                                 K));
        (::idp::count_launch(), k_cl_invert<float><<<ncl, kInvThreads, 0, s>>>(ncl, cl.off, cl.doff, K, K + cl.dense, okp));
    }
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

}  // namespace idp
