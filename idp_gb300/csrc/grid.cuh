// Uniform-grid broad phase shared by the constraint-set builder and the CCD:
// every primitive is binned into the cells its integer box covers, the
// (instance, cell) keys are radix-sorted, and each query (one warp) walks the
// cells of its own box, binary-searching each cell in the sorted table.
// Candidate pairs are compacted warp-cooperatively (ballot + popc) into a
// global list.
#pragma once
#include "common.cuh"

namespace idp {

// lanes per broad-phase query: constraint-set cells (edge-length sized) hold
// a handful of primitives; CCD cells (one or more reference voxels) hold more
constexpr int kQueryLanes = 8;
constexpr int kCcdQueryLanes = 16;

struct GridP {
    double lo[3];
    double inv;
    int n[3];      // cells per axis (indices clamped to [0, n])
    int coarse;    // CCD candidate grid: reference voxels per cell along each axis
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

// Block-wide min (lo) / max (hi) of order-encoded coordinates into bb[6*inst]:
// when every valid thread of the block belongs to the same instance (the
// usual case: primitives are stored instance by instance) one atomic per
// value per block, else one per thread. Every thread of the block must call
// this (valid = false for threads without an element).
__device__ __forceinline__ void bbox_block_update(bool valid, int inst, int inst_first, const unsigned long long lo[3],
                                                  const unsigned long long hi[3], unsigned long long* bb) {
    __shared__ unsigned long long s_v[6][32];
    const bool uni = __syncthreads_and(!valid || inst == inst_first);
    const bool any = __syncthreads_or(valid);
    if (!any) return;
    if (!uni) {
        if (valid)
            for (int d = 0; d < 3; ++d) {
                atomicMin(bb + 6 * inst + d, lo[d]);
                atomicMax(bb + 6 * inst + 3 + d, hi[d]);
            }
        return;
    }
    unsigned long long v[6];
    for (int d = 0; d < 3; ++d) {
        v[d] = valid ? lo[d] : ~0ull;
        v[3 + d] = valid ? hi[d] : 0ull;
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int d = 0; d < 3; ++d) {
            unsigned long long a = __shfl_xor_sync(0xffffffffu, v[d], o);
            unsigned long long b = __shfl_xor_sync(0xffffffffu, v[3 + d], o);
            v[d] = a < v[d] ? a : v[d];
            v[3 + d] = b > v[3 + d] ? b : v[3 + d];
        }
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 6; ++d) s_v[d][warp] = v[d];
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        unsigned long long r = s_v[d][0];
        for (int w = 1; w < nw; ++w) r = d < 3 ? (s_v[d][w] < r ? s_v[d][w] : r) : (s_v[d][w] > r ? s_v[d][w] : r);
        if (d < 3) atomicMin(bb + 6 * inst_first + d, r);
        else atomicMax(bb + 6 * inst_first + d, r);
    }
}

__device__ __forceinline__ int clampi(int v, int a, int b) { return v < a ? a : (v > b ? b : v); }

__device__ __forceinline__ int vox(double x, double lo, double inv) { return (int)floor((x - lo) * inv); }

__device__ __forceinline__ uint64_t cell_key(int inst, const GridP& g, int x, int y, int z) {
    return ((uint64_t)inst << 32) | (uint64_t)((long)x + (long)y * g.s1 + (long)z * g.s2);
}


// open-addressing hash from (instance, cell) key to the cell's index in the
// sorted cell table (linear probing, table at most half full)
constexpr unsigned long long kHashEmpty = ~0ull;

// cell lookup of a box grid: either a dense table (cell id = first cell of
// the instance + linear cell index) or, when the grids would hold too many
// cells, an open-addressing hash of the occupied cells
struct CellHash {
    int dense = 0;
    const uint32_t* cbase = nullptr;  // dense: first cell of every instance
    uint32_t cap = 0xffffffffu;        // dense: cells in the table (lookups past it miss)
    uint32_t ent_cap = 0xffffffffu;    // entries in the table
    const unsigned long long* key = nullptr;
    const uint32_t* val = nullptr;
    uint32_t mask = 0;
};

// dense tables up to this many cells (all instances of a grid together)
constexpr unsigned long long kDenseMaxCells = 1ull << 25;

__device__ __forceinline__ uint32_t cell_hash(uint64_t key, uint32_t mask) {
    uint64_t h = key * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
    return (uint32_t)h & mask;
}

__device__ __forceinline__ int cell_find(const CellHash& t, int inst, const GridP& g, int x, int y, int z);

__device__ __forceinline__ int cell_find_key(const CellHash& t, uint64_t key) {
    uint32_t h = cell_hash(key, t.mask);
    for (uint32_t probe = 0; probe <= t.mask; ++probe) {
        const unsigned long long k = t.key[h];
        if (k == key) return (int)t.val[h];
        if (k == kHashEmpty) return -1;
        h = (h + 1) & t.mask;
    }
    return -1;
}

__device__ __forceinline__ int cell_find(const CellHash& t, int inst, const GridP& g, int x, int y, int z) {
    if (t.dense) {
        if (x < 0 || y < 0 || z < 0 || x > g.n[0] || y > g.n[1] || z > g.n[2]) return -1;
        const uint32_t c = t.cbase[inst] + (uint32_t)((long)x + (long)y * g.s1 + (long)z * g.s2);
        return c < t.cap ? (int)c : -1;
    }
    return cell_find_key(t, cell_key(inst, g, x, y, z));
}

// group-per-query walk: the G lanes of a group (G divides 32, groups aligned
// in the warp) visit the cells of box qb in order; for every occupied cell
// they take the cell's entries G at a time and call
// test(entry, cx, cy, cz, value) -> emit?; emitted values are compacted with
// one ballot per G entries. All lanes of the group must call this together.
template <int G, class V, class Test>
__device__ __forceinline__ void group_walk_emit(const BoxI& qb, int inst, const GridP& g, const CellHash& cells,
                                                const uint32_t* __restrict__ cstart,
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

// group-cooperative append: lanes with emit=true write v to out[] in a block
// reserved by one atomicAdd per group. Writes beyond cap are dropped (the
// counter still counts them so the caller can grow and retry).
template <int G, class V>
__device__ __forceinline__ void group_emit(bool emit, const V& v, V* __restrict__ out, unsigned int* counter, long cap) {
    const int lane = threadIdx.x & 31;
    const unsigned int gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const unsigned int m = __ballot_sync(gmask, emit) & gmask;
    if (!m) return;
    const int leader = __ffs(m) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned int)__popc(m));
    base = __shfl_sync(gmask, base, leader);
    if (emit) {
        unsigned int pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < cap) out[pos] = v;
    }
}

template <int G, class V, class Test>
__device__ __forceinline__ void group_walk_emit(const BoxI& qb, int inst, const GridP& g, const CellHash& cells,
                                                const uint32_t* __restrict__ cstart,
                                                const uint32_t* __restrict__ entries, V* __restrict__ out,
                                                unsigned int* counter, long cap, Test&& test) {
    const int gl = threadIdx.x & (G - 1);
    for (int z = qb.lo[2]; z <= qb.hi[2]; ++z)
        for (int y = qb.lo[1]; y <= qb.hi[1]; ++y)
            for (int x = qb.lo[0]; x <= qb.hi[0]; ++x) {
                const int k = cell_find(cells, inst, g, x, y, z);
                if (k < 0) continue;
                const uint32_t e0 = cstart[k], e1 = min(cstart[k + 1], cells.ent_cap);
                for (uint32_t base = e0; base < e1; base += G) {
                    const uint32_t e = base + gl;
                    V v;
                    bool emit = false;
                    if (e < e1) emit = test(entries[e], x, y, z, v);
                    group_emit<G>(emit, v, out, counter, cap);
                }
            }
}

// ---- host-side builder (contact.cu): sorted (instance, cell) entry table
struct BoxGrid {
    uint32_t* cell_start = nullptr;      // cells + 1
    uint32_t* entries = nullptr;         // primitive ids, grouped by cell
    CellHash cells;                      // (instance, cell) key -> cell index
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
                    const GridP* gp, int nI, long ne, unsigned long long ncells, BoxGrid& out, cudaStream_t s);
// Triangle (gt) and edge (ge) grids of one broad phase (set 0: constraint
// set, 1: CCD). Once a set has been built with a host round trip, later
// builds reuse its table capacities without one: the kernels record in
// *d_flag (bit 0: more cells, bit 1: more entries than the capacities) what
// did not fit, and the caller, at its next synchronisation, calls
// grids_overflowed and rebuilds when it returns true.
int grids_build(Work& W, int set, const BoxI* tbox, long nt, const int* tinst, const BoxI* ebox, long ne,
                const int* einst, const unsigned char* active, const GridP* gp, int nI, unsigned int* d_flag,
                BoxGrid& gt, BoxGrid& ge, cudaStream_t s);
bool grids_overflowed(Work& W, int set, unsigned int flag);
// first cell of every instance of a grid and the total cell count (written
// to *h_cells, pinned host memory, valid after the stream is synchronised)
int grid_cell_bases(Work& W, const GridP* gp, int nI, unsigned long long* h_cells, cudaStream_t s);

}  // namespace idp
