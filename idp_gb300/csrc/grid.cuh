// Uniform-grid broad phase shared by the constraint-set builder and the CCD:
// every primitive is binned into the cells its integer box covers, the
// (instance, cell) keys are radix-sorted, and each query (one warp) walks the
// cells of its own box, binary-searching each cell in the sorted table.
// Candidate pairs are compacted warp-cooperatively (ballot + popc) into a
// global list.
#pragma once
#include "common.cuh"

namespace idp {

struct GridP {
    double lo[3];
    double inv;
    int n[3];      // cells per axis (indices clamped to [0, n])
    long s1, s2;   // linear strides: cell = x + y*s1 + z*s2
};

struct BoxI {
    int lo[3], hi[3];
};

// order-preserving map of doubles to u64 (for exact atomic min/max)
__device__ __forceinline__ unsigned long long ord_enc(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_dec(unsigned long long u) {
    unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ int clampi(int v, int a, int b) { return v < a ? a : (v > b ? b : v); }

__device__ __forceinline__ int vox(double x, double lo, double inv) { return (int)floor((x - lo) * inv); }

__device__ __forceinline__ uint64_t cell_key(int inst, const GridP& g, int x, int y, int z) {
    return ((uint64_t)inst << 32) | (uint64_t)((long)x + (long)y * g.s1 + (long)z * g.s2);
}

__device__ __forceinline__ int lower_bound_u64(const uint64_t* __restrict__ a, int n, uint64_t key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// warp-per-query walk: the whole warp visits the cells of box qb in order;
// for every occupied cell, lanes take the cell's entries 32 at a time and
// call test(entry, cell) -> emit?; emitted values are compacted with one
// ballot per 32 entries. All lanes of the warp must call this together.
template <class V, class Test>
__device__ __forceinline__ void warp_walk_emit(const BoxI& qb, int inst, const GridP& g, const uint64_t* __restrict__ ckey,
                                               const uint32_t* __restrict__ cstart, int ncell,
                                               const uint32_t* __restrict__ entries, V* __restrict__ out,
                                               unsigned int* counter, long cap, Test&& test);

// lowest corner cell of the intersection of the query box and box b
__device__ __forceinline__ bool is_first_shared(const BoxI& q, const BoxI& b, int cx, int cy, int cz) {
    int c[3] = {cx, cy, cz};
    for (int d = 0; d < 3; ++d) {
        if (b.lo[d] > q.hi[d] || b.hi[d] < q.lo[d]) return false;
        int m = q.lo[d] > b.lo[d] ? q.lo[d] : b.lo[d];
        if (m != c[d]) return false;
    }
    return true;
}

// warp-cooperative append: lanes with emit=true write v to out[] in a block
// reserved by one atomicAdd per warp. Writes beyond cap are dropped (the
// counter still counts them so the caller can grow and retry).
template <class V>
__device__ __forceinline__ void warp_emit(bool emit, const V& v, V* __restrict__ out, unsigned int* counter, long cap) {
    unsigned int m = __ballot_sync(0xffffffffu, emit);
    if (!m) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned int)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (emit) {
        unsigned int pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < cap) out[pos] = v;
    }
}

template <class V, class Test>
__device__ __forceinline__ void warp_walk_emit(const BoxI& qb, int inst, const GridP& g, const uint64_t* __restrict__ ckey,
                                               const uint32_t* __restrict__ cstart, int ncell,
                                               const uint32_t* __restrict__ entries, V* __restrict__ out,
                                               unsigned int* counter, long cap, Test&& test) {
    const int lane = threadIdx.x & 31;
    for (int z = qb.lo[2]; z <= qb.hi[2]; ++z)
        for (int y = qb.lo[1]; y <= qb.hi[1]; ++y)
            for (int x = qb.lo[0]; x <= qb.hi[0]; ++x) {
                uint64_t key = cell_key(inst, g, x, y, z);
                int k = lower_bound_u64(ckey, ncell, key);
                if (k >= ncell || ckey[k] != key) continue;
                uint32_t e0 = cstart[k], e1 = cstart[k + 1];
                for (uint32_t base = e0; base < e1; base += 32) {
                    uint32_t e = base + lane;
                    V v;
                    bool emit = false;
                    if (e < e1) emit = test(entries[e], x, y, z, v);
                    warp_emit(emit, v, out, counter, cap);
                }
            }
}

// ---- host-side builder (contact.cu): sorted (instance, cell) entry table
struct BoxGrid {
    uint64_t* cell_keys = nullptr;       // sorted unique keys
    uint32_t* cell_start = nullptr;      // cells + 1
    uint32_t* entries = nullptr;         // primitive ids, grouped by cell
    const uint32_t* d_ncell = nullptr;   // device: number of cells
    long nent = 0;
};

struct Work;
// Bins nprim boxes (box[i], instance inst[i]; skipped when active[inst]==0)
// into their cells, in two steps so several grids share one host round trip:
// box_grid_count writes the number of (box, cell) entries to *h_total (pinned
// host memory, valid after the stream is synchronised); box_grid_finish then
// emits, sorts and tabulates them. slot selects one of two buffer sets so a
// triangle grid and an edge grid can coexist.
int box_grid_count(Work& W, int slot, const BoxI* boxes, const int* inst, const unsigned char* active, long nprim,
                   uint32_t* h_total, cudaStream_t s);
int box_grid_finish(Work& W, int slot, const BoxI* boxes, const int* inst, const unsigned char* active, long nprim,
                    const GridP* gp, int nI, long ne, BoxGrid& out, cudaStream_t s);

}  // namespace idp
