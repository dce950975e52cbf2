// Surface extraction of a tet mesh on the device, in the reference's order
// (Find_Surface_TriMesh, Utils/MESHIO.h:485-544, and the edge and node lists
// of Find_Surface_Primitives_And_Compute_Area, MESHIO.h:768-834), with the
// same result as the host extraction in engine.cpp:
//   1. every tet face (the reference's four oriented faces per tet) keyed by
//      its sorted vertex triple packed in 63 bits, stably radix-sorted, so
//      equal triples are adjacent in face order;
//   2. a face is on the surface unless a face with the same triple and the
//      opposite orientation parity exists;
//   3. surface faces sorted by their oriented triple, duplicates dropped;
//   4. every triangle's three directed edges (triangles in order, then
//      (k0,k1), (k1,k2), (k2,k0)) stably sorted by their unordered pair: the
//      first of each run gives the edge's orientation; the edges are then
//      sorted by that oriented pair;
//   5. the nodes are the vertices of the triangles, ascending.
// Vertex ids must be below 2^21 (the packing); larger meshes use the host.
#include <vector>

#include "engine.hpp"
#include "prims.cuh"

namespace idp {
namespace {

__device__ __forceinline__ uint64_t pack3(uint64_t a, uint64_t b, uint64_t c) { return (a << 42) | (b << 21) | c; }

__global__ void k_tet_faces(long T, const int* __restrict__ tets, int* __restrict__ fk, uint64_t* __restrict__ key,
                            uint32_t* __restrict__ val, unsigned char* __restrict__ par) {
    const long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= 4 * T) return;
    const int* e = tets + 4 * (f >> 2);
    int k0, k1, k2;
    switch (f & 3) {
        case 0: k0 = e[0]; k1 = e[2]; k2 = e[1]; break;
        case 1: k0 = e[0]; k1 = e[3]; k2 = e[2]; break;
        case 2: k0 = e[0]; k1 = e[1]; k2 = e[3]; break;
        default: k0 = e[1]; k1 = e[2]; k2 = e[3]; break;
    }
    fk[3 * f] = k0;
    fk[3 * f + 1] = k1;
    fk[3 * f + 2] = k2;
    int s0 = min(k0, min(k1, k2)), s2 = max(k0, max(k1, k2)), s1 = k0 + k1 + k2 - s0 - s2;
    key[f] = pack3((uint64_t)s0, (uint64_t)s1, (uint64_t)s2);
    val[f] = (uint32_t)f;
    par[f] = (unsigned char)(((k0 > k1) + (k0 > k2) + (k1 > k2)) & 1);
}

// flag[i] = 1 when sorted face i has no twin of opposite parity among the
// faces with its triple (a run of equal keys around i)
__global__ void k_face_surface(long n, const uint64_t* __restrict__ key, const uint32_t* __restrict__ val,
                               const unsigned char* __restrict__ par, uint32_t* __restrict__ flag) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = key[i];
    const unsigned char p = par[val[i]];
    bool twin = false;
    for (long j = i - 1; j >= 0 && key[j] == k && !twin; --j) twin = par[val[j]] != p;
    for (long j = i + 1; j < n && key[j] == k && !twin; ++j) twin = par[val[j]] != p;
    flag[i] = twin ? 0u : 1u;
}

// surface faces: key = oriented triple, value = face index
__global__ void k_surface_keys(long n, const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                               const uint32_t* __restrict__ val, const int* __restrict__ fk,
                               uint64_t* __restrict__ okey, uint32_t* __restrict__ oval) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const uint32_t f = val[i], o = pos[i];
    okey[o] = pack3((uint64_t)fk[3L * f], (uint64_t)fk[3L * f + 1], (uint64_t)fk[3L * f + 2]);
    oval[o] = f;
}

__global__ void k_first_of_run(long n, const uint64_t* __restrict__ key, uint32_t* __restrict__ flag) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

__global__ void k_write_tris(long n, const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                             const uint32_t* __restrict__ val, const int* __restrict__ fk, int* __restrict__ tris) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const uint32_t f = val[i], o = pos[i];
    tris[3L * o] = fk[3L * f];
    tris[3L * o + 1] = fk[3L * f + 1];
    tris[3L * o + 2] = fk[3L * f + 2];
}

// directed edges of the triangles in order: key = unordered pair, value = 3j + l
__global__ void k_tri_edges(long nt, const int* __restrict__ tris, uint64_t* __restrict__ key,
                            uint32_t* __restrict__ val) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nt) return;
    const long j = i / 3;
    const int l = (int)(i - 3 * j);
    const int a = tris[3 * j + l], b = tris[3 * j + (l + 1) % 3];
    key[i] = ((uint64_t)min(a, b) << 21) | (uint64_t)max(a, b);
    val[i] = (uint32_t)i;
}

// the first directed edge of each unordered pair, keyed by its oriented pair
__global__ void k_edge_keys(long n, const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                            const uint32_t* __restrict__ val, const int* __restrict__ tris, uint64_t* __restrict__ okey,
                            uint32_t* __restrict__ oval) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const long e = val[i], j = e / 3;
    const int l = (int)(e - 3 * j);
    const int a = tris[3 * j + l], b = tris[3 * j + (l + 1) % 3];
    okey[pos[i]] = ((uint64_t)a << 21) | (uint64_t)b;
    oval[pos[i]] = 0;
}

__global__ void k_mark_nodes(long n3, const int* __restrict__ tris, uint32_t* __restrict__ used) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n3) used[tris[i]] = 1u;
}

__global__ void k_write_nodes(long V, const uint32_t* __restrict__ used, const uint32_t* __restrict__ pos,
                              int* __restrict__ nodes) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < V && used[v]) nodes[pos[v]] = (int)v;
}

struct DevMem {
    std::vector<void*> p;
    ~DevMem() {
        for (void* q : p) cudaFree(q);
    }
    template <class T>
    T* get(size_t n) {
        void* q = nullptr;
        if (cudaMalloc(&q, sizeof(T) * (n + 1)) != cudaSuccess) return nullptr;
        p.push_back(q);
        return static_cast<T*>(q);
    }
};

}  // namespace

int extract_surface_device(int V, const std::vector<int>& tets, std::vector<int>& tris, std::vector<int>& edges,
                           std::vector<int>& nodes, cudaStream_t s) {
    const long T = (long)tets.size() / 4, n = 4 * T;
    if (V <= 0 || V > (1 << 21) || T <= 0 || n > 0xffffffffL) return IDP_ERR_INVALID_ARG;
    DevMem m;
    int* d_tets = m.get<int>(4 * T);
    int* fk = m.get<int>(3 * n);
    uint64_t *key = m.get<uint64_t>(n), *key_alt = m.get<uint64_t>(n);
    uint32_t *val = m.get<uint32_t>(n), *val_alt = m.get<uint32_t>(n);
    unsigned char* par = m.get<unsigned char>(n);
    uint32_t *flag = m.get<uint32_t>(n), *pos = m.get<uint32_t>(n), *total = m.get<uint32_t>(1);
    const size_t scr = std::max(radix_sort_scratch_bytes(n), scan_scratch_bytes(n));
    void* scratch = m.get<unsigned char>(scr);
    if (!d_tets || !fk || !key || !key_alt || !val || !val_alt || !par || !flag || !pos || !total || !scratch)
        return IDP_ERR_CUDA;
    auto grid = [](long k) { return (unsigned)((k + kBlock - 1) / kBlock); };
    uint32_t cnt = 0;
    auto read_total = [&]() -> int {
        IDP_CUDA_TRY(cudaMemcpyAsync(&cnt, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        return IDP_OK;
    };
    IDP_CUDA_TRY(cudaMemcpyAsync(d_tets, tets.data(), sizeof(int) * 4 * T, cudaMemcpyHostToDevice, s));
    // 1-2: faces by sorted triple, surface flags
    (::idp::count_launch(), k_tet_faces<<<grid(n), kBlock, 0, s>>>(T, d_tets, fk, key, val, par));
    IDP_CUDA_TRY(radix_sort_pairs(key, val, key_alt, val_alt, n, 63, scratch, s));
    (::idp::count_launch(), k_face_surface<<<grid(n), kBlock, 0, s>>>(n, key, val, par, flag));
    IDP_CUDA_TRY(scan_exclusive(flag, pos, n, total, scratch, s));
    int rc = read_total();
    if (rc) return rc;
    const long nb = cnt;
    if (nb == 0) return IDP_ERR_INVALID_ARG;  // a closed tet mesh has surface faces
    // 3: surface faces by oriented triple, duplicates dropped
    (::idp::count_launch(), k_surface_keys<<<grid(n), kBlock, 0, s>>>(n, flag, pos, val, fk, key_alt, val_alt));
    IDP_CUDA_TRY(radix_sort_pairs(key_alt, val_alt, key, val, nb, 63, scratch, s));
    (::idp::count_launch(), k_first_of_run<<<grid(nb), kBlock, 0, s>>>(nb, key_alt, flag));
    IDP_CUDA_TRY(scan_exclusive(flag, pos, nb, total, scratch, s));
    if ((rc = read_total())) return rc;
    const long nt = cnt;
    int* d_tris = m.get<int>(3 * nt);
    if (!d_tris) return IDP_ERR_CUDA;
    (::idp::count_launch(), k_write_tris<<<grid(nb), kBlock, 0, s>>>(nb, flag, pos, val_alt, fk, d_tris));
    // 4: edges, first orientation, sorted by it (buffers sized for 3 nt
    // directed edges, which can exceed the face count of a tiny mesh)
    const long ne3 = 3 * nt;
    uint64_t *ek0 = m.get<uint64_t>(ne3), *ek1 = m.get<uint64_t>(ne3);
    uint32_t *ev0 = m.get<uint32_t>(ne3), *ev1 = m.get<uint32_t>(ne3);
    uint32_t *eflag = m.get<uint32_t>(ne3), *epos = m.get<uint32_t>(ne3);
    uint32_t *used = m.get<uint32_t>(V), *npos = m.get<uint32_t>(V);
    const size_t scr2 = std::max(radix_sort_scratch_bytes(ne3), scan_scratch_bytes(std::max<long>(ne3, V)));
    void* scratch2 = m.get<unsigned char>(scr2);
    if (!ek0 || !ek1 || !ev0 || !ev1 || !eflag || !epos || !used || !npos || !scratch2) return IDP_ERR_CUDA;
    (::idp::count_launch(), k_tri_edges<<<grid(ne3), kBlock, 0, s>>>(nt, d_tris, ek0, ev0));
    IDP_CUDA_TRY(radix_sort_pairs(ek0, ev0, ek1, ev1, ne3, 42, scratch2, s));
    (::idp::count_launch(), k_first_of_run<<<grid(ne3), kBlock, 0, s>>>(ne3, ek0, eflag));
    IDP_CUDA_TRY(scan_exclusive(eflag, epos, ne3, total, scratch2, s));
    if ((rc = read_total())) return rc;
    const long ne = cnt;
    (::idp::count_launch(), k_edge_keys<<<grid(ne3), kBlock, 0, s>>>(ne3, eflag, epos, ev0, d_tris, ek1, ev1));
    IDP_CUDA_TRY(radix_sort_pairs(ek1, ev1, ek0, ev0, ne, 42, scratch2, s));
    // 5: nodes ascending
    IDP_CUDA_TRY(cudaMemsetAsync(used, 0, sizeof(uint32_t) * V, s));
    (::idp::count_launch(), k_mark_nodes<<<grid(ne3), kBlock, 0, s>>>(ne3, d_tris, used));
    IDP_CUDA_TRY(scan_exclusive(used, npos, V, total, scratch2, s));
    if ((rc = read_total())) return rc;
    const long nn = cnt;
    int* d_nodes = m.get<int>(nn);
    if (!d_nodes) return IDP_ERR_CUDA;
    (::idp::count_launch(), k_write_nodes<<<grid(V), kBlock, 0, s>>>(V, used, npos, d_nodes));
    std::vector<uint64_t> ek(ne);
    tris.resize(3 * nt);
    nodes.resize(nn);
    IDP_CUDA_TRY(cudaMemcpyAsync(tris.data(), d_tris, sizeof(int) * 3 * nt, cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(ek.data(), ek1, sizeof(uint64_t) * ne, cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaMemcpyAsync(nodes.data(), d_nodes, sizeof(int) * nn, cudaMemcpyDeviceToHost, s));
    IDP_CUDA_TRY(cudaStreamSynchronize(s));
    edges.resize(2 * ne);
    for (long e = 0; e < ne; ++e) {
        edges[2 * e] = (int)(ek[e] >> 21);
        edges[2 * e + 1] = (int)(ek[e] & ((1u << 21) - 1));
    }
    return IDP_OK;
}

}  // namespace idp
