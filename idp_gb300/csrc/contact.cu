// Constraint-set builder (compiled with --fmad=false): GPU restatement of
// Compute_Constraint_Set, 3D branch (FEM/IPC.h:143-661).
//
//   1. per-instance grid over the surface (cell = rest mean edge length,
//      origin = min surface-node position), triangles and edges binned into
//      the cells their integer boxes cover, (instance, cell) radix-sorted;
//   2. point-triangle and edge-edge queries walk their +-dHat box, report each
//      candidate once (lowest shared cell) after the reference's exclusions and
//      AABB test (CCD.h:149-185), compacted warp-cooperatively;
//   3. narrow phase: FP64 distance type + squared distance, d < dHat^2, and the
//      sign-tagged int4 encoding of IPC.h:202-250 / 434-554;
//   4. records sorted by (instance, c0, c1, c2, c3); duplicate regular PP/PE
//      records merged with multiplicity -count in slot 3 (IPC.h:599-654).
// The grid is only a conservative filter; membership is decided by the same
// FP64 tests the reference applies, so the set does not depend on the cell
// size. The output order is the sort order, independent of thread timing.
#include "engine.hpp"
#include "grid.cuh"
#include "geom.cuh"
#include "predicates.cuh"
#include "prims.cuh"

namespace idp {

using namespace geo;

namespace {

__global__ void k_bbox(long n, const int* __restrict__ nodes, const int* __restrict__ ninst,
                       const unsigned char* __restrict__ active, const double* __restrict__ X,
                       unsigned long long* __restrict__ bb) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int inst = i < n ? ninst[i] : 0;
    const int inst_first = ninst[(long)blockIdx.x * blockDim.x];
    const bool valid = i < n && active[inst];
    unsigned long long lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (valid) {
        D3 p = ld3(X, nodes[i]);
        lo[0] = hi[0] = ord_enc(p.x);
        lo[1] = hi[1] = ord_enc(p.y);
        lo[2] = hi[2] = ord_enc(p.z);
    }
    bbox_block_update(valid, inst, inst_first, lo, hi, bb);
}

__global__ void k_bbox_init(int nI, unsigned long long* bb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nI) return;
    bb[i] = (i % 6) < 3 ? 0xffffffffffffffffull : 0ull;
}

// grid parameters of the constraint-set grid
__global__ void k_grid_params(int nI, const unsigned long long* __restrict__ bb, const double* __restrict__ cell,
                              const double* __restrict__ dHat2, const double* __restrict__ thick,
                              const unsigned char* __restrict__ active, GridP* __restrict__ gp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nI) return;
    GridP g;
    double r = sqrt(dHat2[i]) + thick[i];
    double h = cell[i];
    double ext[3];
    for (int d = 0; d < 3; ++d) {
        double lo = ord_dec(bb[6 * i + d]), hi = ord_dec(bb[6 * i + 3 + d]);
        if (!active[i] || !(hi >= lo)) { lo = 0; hi = 0; }
        g.lo[d] = lo - 2 * r;
        ext[d] = (hi - lo) + 4 * r;
    }
    if (!(h > 0)) h = 1.0;
    // keep the cell count per instance below 2^31
    for (int it = 0; it < 64; ++it) {
        double c = (floor(ext[0] / h) + 2) * (floor(ext[1] / h) + 2) * (floor(ext[2] / h) + 2);
        if (c < 2.0e9) break;
        h *= 1.5;
    }
    g.inv = 1.0 / h;
    for (int d = 0; d < 3; ++d) g.n[d] = (int)floor(ext[d] * g.inv) + 1;
    g.s1 = (long)g.n[0] + 1;
    g.s2 = g.s1 * ((long)g.n[1] + 1);
    gp[i] = g;
}

__device__ __forceinline__ void vox3(const GridP& g, D3 p, int o[3]) {
    o[0] = clampi(vox(p.x, g.lo[0], g.inv), 0, g.n[0]);
    o[1] = clampi(vox(p.y, g.lo[1], g.inv), 0, g.n[1]);
    o[2] = clampi(vox(p.z, g.lo[2], g.inv), 0, g.n[2]);
}

template <int K>
__global__ void k_prim_boxes(long n, const int* __restrict__ verts, const int* __restrict__ pinst,
                             const unsigned char* __restrict__ active, const double* __restrict__ X,
                             const GridP* __restrict__ gp, BoxI* __restrict__ boxes) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int inst = pinst[i];
    BoxI b;
    if (!active[inst]) {
        for (int d = 0; d < 3; ++d) { b.lo[d] = 1; b.hi[d] = 0; }
        boxes[i] = b;
        return;
    }
    GridP g = gp[inst];
    int o[3];
    vox3(g, ld3(X, verts[K * i]), o);
    for (int d = 0; d < 3; ++d) b.lo[d] = b.hi[d] = o[d];
    for (int k = 1; k < K; ++k) {
        vox3(g, ld3(X, verts[K * i + k]), o);
        for (int d = 0; d < 3; ++d) {
            b.lo[d] = min(b.lo[d], o[d]);
            b.hi[d] = max(b.hi[d], o[d]);
        }
    }
    boxes[i] = b;
}

// ---- generic grid build
__global__ void k_box_count(long n, const BoxI* __restrict__ boxes, const int* __restrict__ pinst,
                            const unsigned char* __restrict__ active, uint32_t* __restrict__ cnt) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BoxI b = boxes[i];
    uint32_t c = 0;
    if (active[pinst[i]] && b.lo[0] <= b.hi[0] && b.lo[1] <= b.hi[1] && b.lo[2] <= b.hi[2])
        c = (uint32_t)(b.hi[0] - b.lo[0] + 1) * (uint32_t)(b.hi[1] - b.lo[1] + 1) * (uint32_t)(b.hi[2] - b.lo[2] + 1);
    cnt[i] = c;
}

__global__ void k_box_emit(long n, const BoxI* __restrict__ boxes, const int* __restrict__ pinst,
                           const unsigned char* __restrict__ active, const GridP* __restrict__ gp,
                           const uint32_t* __restrict__ off, uint64_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int inst = pinst[i];
    if (!active[inst]) return;
    BoxI b = boxes[i];
    GridP g = gp[inst];
    uint32_t o = off[i];
    for (int z = b.lo[2]; z <= b.hi[2]; ++z)
        for (int y = b.lo[1]; y <= b.hi[1]; ++y)
            for (int x = b.lo[0]; x <= b.hi[0]; ++x) {
                keys[o] = cell_key(inst, g, x, y, z);
                vals[o] = (uint32_t)i;
                ++o;
            }
}

// first cell of every instance (prefix of the per-instance cell counts) and
// the total; one thread, instances are few
__global__ void k_cell_bases(int nI, const GridP* __restrict__ gp, uint32_t* __restrict__ cbase,
                             unsigned long long* __restrict__ total, unsigned long long cap,
                             unsigned int* __restrict__ flag) {
    unsigned long long acc = 0;
    for (int i = 0; i < nI; ++i) {
        cbase[i] = (uint32_t)(acc < 0xffffffffull ? acc : 0xffffffffull);
        const GridP g = gp[i];
        acc += (unsigned long long)g.s2 * (unsigned long long)(g.n[2] + 1);
    }
    cbase[nI] = (uint32_t)(acc < 0xffffffffull ? acc : 0xffffffffull);
    *total = acc;
    if (flag && acc > cap) atomicOr(flag, 1u);
}

// both grids of a broad phase in one pass (boxes [0, nt) are triangles,
// [nt, nt + ne) edges); cell tables side by side: grid g's cell c is slot
// g * (cap + 1) + c. Cells past the capacity are skipped (the build is redone).
__device__ __forceinline__ bool dense2_box(long i, long nt, const BoxI* __restrict__ tbox, const int* __restrict__ tinst,
                                           const BoxI* __restrict__ ebox, const int* __restrict__ einst,
                                           const unsigned char* __restrict__ active, BoxI& b, int& inst, int& grid) {
    grid = i < nt ? 0 : 1;
    inst = grid ? einst[i - nt] : tinst[i];
    if (!active[inst]) return false;
    b = grid ? ebox[i - nt] : tbox[i];
    return true;
}

__global__ void k_dense_count2(long nt, long ne, const BoxI* __restrict__ tbox, const int* __restrict__ tinst,
                               const BoxI* __restrict__ ebox, const int* __restrict__ einst,
                               const unsigned char* __restrict__ active, const GridP* __restrict__ gp,
                               const uint32_t* __restrict__ cbase, uint32_t cap, uint32_t* __restrict__ ccount) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt + ne) return;
    BoxI b;
    int inst, grid;
    if (!dense2_box(i, nt, tbox, tinst, ebox, einst, active, b, inst, grid)) return;
    const GridP g = gp[inst];
    const uint32_t c0 = cbase[inst];
    uint32_t* cnt = ccount + (size_t)grid * (cap + 1);
    const int zl = max(b.lo[2], 0), zh = min(b.hi[2], g.n[2]), yl = max(b.lo[1], 0), yh = min(b.hi[1], g.n[1]);
    const int xl = max(b.lo[0], 0), xh = min(b.hi[0], g.n[0]);
    for (int z = zl; z <= zh; ++z)
        for (int y = yl; y <= yh; ++y)
            for (int x = xl; x <= xh; ++x) {
                const uint32_t c = c0 + (uint32_t)((long)x + (long)y * g.s1 + (long)z * g.s2);
                if (c < cap) atomicAdd(cnt + c, 1u);
            }
}

__global__ void k_dense_fill2(long nt, long ne, const BoxI* __restrict__ tbox, const int* __restrict__ tinst,
                              const BoxI* __restrict__ ebox, const int* __restrict__ einst,
                              const unsigned char* __restrict__ active, const GridP* __restrict__ gp,
                              const uint32_t* __restrict__ cbase, uint32_t cap, const uint32_t* __restrict__ cstart,
                              uint32_t* __restrict__ ccount, uint32_t* __restrict__ entries, long ent_cap,
                              unsigned int* __restrict__ flag) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt + ne) return;
    BoxI b;
    int inst, grid;
    if (!dense2_box(i, nt, tbox, tinst, ebox, einst, active, b, inst, grid)) return;
    const GridP g = gp[inst];
    const uint32_t c0 = cbase[inst];
    const size_t base = (size_t)grid * (cap + 1);
    const int zl = max(b.lo[2], 0), zh = min(b.hi[2], g.n[2]), yl = max(b.lo[1], 0), yh = min(b.hi[1], g.n[1]);
    const int xl = max(b.lo[0], 0), xh = min(b.hi[0], g.n[0]);
    const uint32_t prim = (uint32_t)(grid ? i - nt : i);
    for (int z = zl; z <= zh; ++z)
        for (int y = yl; y <= yh; ++y)
            for (int x = xl; x <= xh; ++x) {
                const uint32_t c = c0 + (uint32_t)((long)x + (long)y * g.s1 + (long)z * g.s2);
                if (c >= cap) continue;
                const uint32_t pos = cstart[base + c] + atomicSub(ccount + base + c, 1u) - 1u;
                if (pos < ent_cap) entries[pos] = prim;
                else atomicOr(flag, 2u);
            }
}

// dense table: occupancy count per cell, then each box's cells take a slot
// (the order of the entries inside a cell is immaterial to every consumer:
// constraint records are sorted afterwards and CCD keeps a minimum)
__global__ void k_dense_count(long n, const BoxI* __restrict__ boxes, const int* __restrict__ pinst,
                              const unsigned char* __restrict__ active, const GridP* __restrict__ gp,
                              const uint32_t* __restrict__ cbase, uint32_t* __restrict__ ccount) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int inst = pinst[i];
    if (!active[inst]) return;
    const BoxI b = boxes[i];
    const GridP g = gp[inst];
    const uint32_t c0 = cbase[inst];
    // boxes are built inside [0, n]; the clamp only guards the table bounds
    const int zl = max(b.lo[2], 0), zh = min(b.hi[2], g.n[2]), yl = max(b.lo[1], 0), yh = min(b.hi[1], g.n[1]);
    const int xl = max(b.lo[0], 0), xh = min(b.hi[0], g.n[0]);
    for (int z = zl; z <= zh; ++z)
        for (int y = yl; y <= yh; ++y)
            for (int x = xl; x <= xh; ++x)
                atomicAdd(ccount + c0 + (uint32_t)((long)x + (long)y * g.s1 + (long)z * g.s2), 1u);
}

__global__ void k_dense_fill(long n, const BoxI* __restrict__ boxes, const int* __restrict__ pinst,
                             const unsigned char* __restrict__ active, const GridP* __restrict__ gp,
                             const uint32_t* __restrict__ cbase, const uint32_t* __restrict__ cstart,
                             uint32_t* __restrict__ ccount, uint32_t* __restrict__ entries) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int inst = pinst[i];
    if (!active[inst]) return;
    const BoxI b = boxes[i];
    const GridP g = gp[inst];
    const uint32_t c0 = cbase[inst];
    // boxes are built inside [0, n]; the clamp only guards the table bounds
    const int zl = max(b.lo[2], 0), zh = min(b.hi[2], g.n[2]), yl = max(b.lo[1], 0), yh = min(b.hi[1], g.n[1]);
    const int xl = max(b.lo[0], 0), xh = min(b.hi[0], g.n[0]);
    for (int z = zl; z <= zh; ++z)
        for (int y = yl; y <= yh; ++y)
            for (int x = xl; x <= xh; ++x) {
                const uint32_t c = c0 + (uint32_t)((long)x + (long)y * g.s1 + (long)z * g.s2);
                entries[cstart[c] + atomicSub(ccount + c, 1u) - 1u] = (uint32_t)i;
            }
}

__global__ void k_mark_heads(long n, const uint64_t* __restrict__ keys, uint32_t* __restrict__ head) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// cell starts of the sorted entries and the key -> cell hash
__global__ void k_cell_table(long n, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ head,
                             const uint32_t* __restrict__ idx, uint32_t* __restrict__ cstart,
                             const uint32_t* __restrict__ ncell, unsigned long long* __restrict__ hkey,
                             uint32_t* __restrict__ hval, uint32_t mask) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) cstart[*ncell] = (uint32_t)n;
    if (i >= n || !head[i]) return;
    const uint32_t c = idx[i];
    cstart[c] = (uint32_t)i;
    const unsigned long long key = keys[i];
    uint32_t h = cell_hash(key, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        if (atomicCAS(hkey + h, kHashEmpty, key) == kHashEmpty) {
            hval[h] = c;
            return;
        }
        h = (h + 1) & mask;
    }
}

// ---- queries
struct Cand {
    int a, b;
};

// one lane group per surface node: triangles within the +-dHat box (IPC.h:158-196)
__global__ void k_query_pt(long nN, const int* __restrict__ nodes, const int* __restrict__ ninst,
                           const unsigned char* __restrict__ active, const double* __restrict__ X,
                           const unsigned char* __restrict__ dbc, const int* __restrict__ tris,
                           const BoxI* __restrict__ tbox, const GridP* __restrict__ gp,
                           const double* __restrict__ dHat2, const double* __restrict__ thick,
                           CellHash cells, const uint32_t* __restrict__ cstart,
                           const uint32_t* __restrict__ entries, Cand* __restrict__ out, unsigned int* counter,
                           long cap) {
    long s = ((long)blockIdx.x * blockDim.x + threadIdx.x) / kQueryLanes;
    if (s >= nN) return;  // the whole group leaves together
    int inst = ninst[s];
    if (!active[inst]) return;
    int vI = nodes[s];
    D3 p = ld3(X, vI);
    double r = sqrt(dHat2[inst]) + thick[inst];
    GridP g = gp[inst];
    double rq = r * (1.0 + 1e-12) + 1e-300;
    int lo[3], hi[3];
    vox3(g, mk3(p.x - rq, p.y - rq, p.z - rq), lo);
    vox3(g, mk3(p.x + rq, p.y + rq, p.z + rq), hi);
    BoxI qb;
    for (int d = 0; d < 3; ++d) { qb.lo[d] = lo[d]; qb.hi[d] = hi[d]; }
    const double pp[3] = {p.x, p.y, p.z};
    const bool pdbc = dbc[vI] != 0;
    group_walk_emit<kQueryLanes>(qb, inst, g, cells, cstart, entries, out, counter, cap,
                   [&](uint32_t ent, int cx, int cy, int cz, Cand& c) -> bool {
                       int f = (int)ent;
                       if (!is_first_shared(qb, tbox[f], cx, cy, cz)) return false;
                       int t0 = tris[3 * f], t1 = tris[3 * f + 1], t2 = tris[3 * f + 2];
                       if (vI == t0 || vI == t1 || vI == t2) return false;
                       if (pdbc && dbc[t0] && dbc[t1] && dbc[t2]) return false;
                       D3 a = ld3(X, t0), b = ld3(X, t1), cc = ld3(X, t2);
                       double mx[3] = {fmax(fmax(a.x, b.x), cc.x), fmax(fmax(a.y, b.y), cc.y), fmax(fmax(a.z, b.z), cc.z)};
                       double mn[3] = {fmin(fmin(a.x, b.x), cc.x), fmin(fmin(a.y, b.y), cc.y), fmin(fmin(a.z, b.z), cc.z)};
                       for (int d = 0; d < 3; ++d)
                           if (pp[d] - mx[d] > r || mn[d] - pp[d] > r) return false;
                       c = {(int)s, f};
                       return true;
                   });
}

// one lane group per surface edge: edges eJ > eI within the +-dHat box (IPC.h:371-420)
__global__ void k_query_ee(long nE, const int2* __restrict__ edges, const int* __restrict__ einst,
                           const unsigned char* __restrict__ active, const double* __restrict__ X,
                           const unsigned char* __restrict__ dbc, const BoxI* __restrict__ ebox,
                           const GridP* __restrict__ gp, const double* __restrict__ dHat2,
                           const double* __restrict__ thick, CellHash cells,
                           const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ entries,
                           Cand* __restrict__ out, unsigned int* counter, long cap) {
    long eI = ((long)blockIdx.x * blockDim.x + threadIdx.x) / kQueryLanes;
    if (eI >= nE) return;
    int inst = einst[eI];
    if (!active[inst]) return;
    int2 mi = edges[eI];
    D3 a0 = ld3(X, mi.x), a1 = ld3(X, mi.y);
    double r = sqrt(dHat2[inst]) + thick[inst];
    GridP g = gp[inst];
    double rq = r * (1.0 + 1e-12) + 1e-300;
    int lo[3], hi[3];
    vox3(g, mk3(fmin(a0.x, a1.x) - rq, fmin(a0.y, a1.y) - rq, fmin(a0.z, a1.z) - rq), lo);
    vox3(g, mk3(fmax(a0.x, a1.x) + rq, fmax(a0.y, a1.y) + rq, fmax(a0.z, a1.z) + rq), hi);
    BoxI qb;
    for (int d = 0; d < 3; ++d) { qb.lo[d] = lo[d]; qb.hi[d] = hi[d]; }
    const double amax[3] = {fmax(a0.x, a1.x), fmax(a0.y, a1.y), fmax(a0.z, a1.z)};
    const double amin[3] = {fmin(a0.x, a1.x), fmin(a0.y, a1.y), fmin(a0.z, a1.z)};
    const bool adbc = dbc[mi.x] && dbc[mi.y];
    group_walk_emit<kQueryLanes>(qb, inst, g, cells, cstart, entries, out, counter, cap,
                   [&](uint32_t ent, int cx, int cy, int cz, Cand& c) -> bool {
                       int eJ = (int)ent;
                       if (eJ <= eI || !is_first_shared(qb, ebox[eJ], cx, cy, cz)) return false;
                       int2 mj = edges[eJ];
                       if (mi.x == mj.x || mi.x == mj.y || mi.y == mj.x || mi.y == mj.y) return false;
                       if (adbc && dbc[mj.x] && dbc[mj.y]) return false;
                       D3 b0 = ld3(X, mj.x), b1 = ld3(X, mj.y);
                       double bmax[3] = {fmax(b0.x, b1.x), fmax(b0.y, b1.y), fmax(b0.z, b1.z)};
                       double bmin[3] = {fmin(b0.x, b1.x), fmin(b0.y, b1.y), fmin(b0.z, b1.z)};
                       for (int d = 0; d < 3; ++d)
                           if (amin[d] - bmax[d] > r || bmin[d] - amax[d] > r) return false;
                       c = {(int)eI, eJ};
                       return true;
                   });
}

// ---- narrow phase
struct Rec {
    int4 c;
    int inst;
};

__global__ void k_narrow_pt(long K, const Cand* __restrict__ cand, const int* __restrict__ nodes,
                            const int* __restrict__ ninst, const int* __restrict__ tris,
                            const double* __restrict__ X, const double* __restrict__ dHat2,
                            const double* __restrict__ thick, Rec* __restrict__ out, unsigned int* counter,
                            long cap) {
    long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    bool emit = false;
    Rec rec;
    rec.c = make_int4(0, 0, 0, 0);
    rec.inst = 0;
    if (k < K) {
        Cand cd = cand[k];
        int vI = nodes[cd.a], inst = ninst[cd.a];
        int t0 = tris[3 * cd.b], t1 = tris[3 * cd.b + 1], t2 = tris[3 * cd.b + 2];
        D3 p = ld3(X, vI), a = ld3(X, t0), b = ld3(X, t1), c = ld3(X, t2);
        double r = sqrt(dHat2[inst]) + thick[inst];
        double r2 = r * r;
        double d;
        int4 cc;
        switch (type_PT(p, a, b, c)) {
            case 0: d = d_PP(p, a); cc = make_int4(-vI - 1, t0, -1, -1); break;
            case 1: d = d_PP(p, b); cc = make_int4(-vI - 1, t1, -1, -1); break;
            case 2: d = d_PP(p, c); cc = make_int4(-vI - 1, t2, -1, -1); break;
            case 3: d = d_PE(p, a, b); cc = make_int4(-vI - 1, t0, t1, -1); break;
            case 4: d = d_PE(p, b, c); cc = make_int4(-vI - 1, t1, t2, -1); break;
            case 5: d = d_PE(p, c, a); cc = make_int4(-vI - 1, t2, t0, -1); break;
            default: d = d_PT(p, a, b, c); cc = make_int4(-vI - 1, t0, t1, t2); break;
        }
        if (d < r2) {
            emit = true;
            rec.c = cc;
            rec.inst = inst;
        }
    }
    group_emit<32>(emit, rec, out, counter, cap);
}

__global__ void k_narrow_ee(long K, const Cand* __restrict__ cand, const int2* __restrict__ edges,
                            const int* __restrict__ einst, const double* __restrict__ X,
                            const double* __restrict__ X0, const double* __restrict__ dHat2,
                            const double* __restrict__ thick, Rec* __restrict__ out, unsigned int* counter,
                            long cap) {
    long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    bool emit = false;
    Rec rec;
    rec.c = make_int4(0, 0, 0, 0);
    rec.inst = 0;
    if (k < K) {
        Cand cd = cand[k];
        int2 mi = edges[cd.a], mj = edges[cd.b];
        int inst = einst[cd.a];
        int a0 = mi.x, a1 = mi.y, b0 = mj.x, b1 = mj.y;
        D3 ea0 = ld3(X, a0), ea1 = ld3(X, a1), eb0 = ld3(X, b0), eb1 = ld3(X, b1);
        double r = sqrt(dHat2[inst]) + thick[inst];
        double r2 = r * r;
        double cn = ee_cross_norm2(ea0, ea1, eb0, eb1);
        double eps_x = mollifier_threshold(ld3(X0, a0), ld3(X0, a1), ld3(X0, b0), ld3(X0, b1));
        bool mol = cn < eps_x;
        double d;
        int4 c;
        switch (type_EE(ea0, ea1, eb0, eb1)) {
            case 0: d = d_PP(ea0, eb0); c = mol ? make_int4(a0, b0, -a1 - 1, -b1 - 1) : make_int4(-a0 - 1, b0, -1, -1); break;
            case 1: d = d_PP(ea0, eb1); c = mol ? make_int4(a0, b1, -a1 - 1, -b0 - 1) : make_int4(-a0 - 1, b1, -1, -1); break;
            case 2: d = d_PE(ea0, eb0, eb1); c = mol ? make_int4(a0, b0, b1, -a1 - 1) : make_int4(-a0 - 1, b0, b1, -1); break;
            case 3: d = d_PP(ea1, eb0); c = mol ? make_int4(a1, b0, -a0 - 1, -b1 - 1) : make_int4(-a1 - 1, b0, -1, -1); break;
            case 4: d = d_PP(ea1, eb1); c = mol ? make_int4(a1, b1, -a0 - 1, -b0 - 1) : make_int4(-a1 - 1, b1, -1, -1); break;
            case 5: d = d_PE(ea1, eb0, eb1); c = mol ? make_int4(a1, b0, b1, -a0 - 1) : make_int4(-a1 - 1, b0, b1, -1); break;
            case 6: d = d_PE(eb0, ea0, ea1); c = mol ? make_int4(b0, a0, a1, -b1 - 1) : make_int4(-b0 - 1, a0, a1, -1); break;
            case 7: d = d_PE(eb1, ea0, ea1); c = mol ? make_int4(b1, a0, a1, -b0 - 1) : make_int4(-b1 - 1, a0, a1, -1); break;
            default: d = d_EE(ea0, ea1, eb0, eb1); c = mol ? make_int4(a0, a1, -b0 - 1, b1) : make_int4(a0, a1, b0, b1); break;
        }
        if (d < r2) {
            emit = true;
            rec.c = c;
            rec.inst = inst;
        }
    }
    group_emit<32>(emit, rec, out, counter, cap);
}

// ---- sort + merge
__global__ void k_rec_keys(long n, const Rec* __restrict__ recs, int b, int off, uint64_t* __restrict__ klo,
                           uint32_t* __restrict__ perm) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int4 c = recs[i].c;
    klo[i] = ((uint64_t)(uint32_t)(c.z + off) << b) | (uint64_t)(uint32_t)(c.w + off);
    perm[i] = (uint32_t)i;
}
__global__ void k_rec_keys_hi(long n, const Rec* __restrict__ recs, const uint32_t* __restrict__ perm_in, int b,
                              int off, uint64_t* __restrict__ khi, uint32_t* __restrict__ perm_out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t j = perm_in[i];
    Rec r = recs[j];
    khi[i] = ((uint64_t)(uint32_t)r.inst << (2 * b)) | ((uint64_t)(uint32_t)(r.c.x + off) << b) |
             (uint64_t)(uint32_t)(r.c.y + off);
    perm_out[i] = j;
}

__device__ __forceinline__ bool same_rec(const Rec& a, const Rec& b) {
    return a.inst == b.inst && a.c.x == b.c.x && a.c.y == b.c.y && a.c.z == b.c.z && a.c.w == b.c.w;
}

// head of a run: first record, or differs from predecessor, or not mergeable
__global__ void k_merge_heads(long n, const Rec* __restrict__ recs, const uint32_t* __restrict__ perm,
                              uint32_t* __restrict__ head) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rec r = recs[perm[i]];
    bool mergeable = r.c.x < 0 && r.c.w < 0;
    bool h = true;
    if (i > 0 && mergeable) h = !same_rec(r, recs[perm[i - 1]]);
    head[i] = h ? 1u : 0u;
}

__global__ void k_merge_write(long n, const Rec* __restrict__ recs, const uint32_t* __restrict__ perm,
                              const uint32_t* __restrict__ head, const uint32_t* __restrict__ pos,
                              int4* __restrict__ cons, int* __restrict__ cinst) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !head[i]) return;
    Rec r = recs[perm[i]];
    int4 c = r.c;
    if (c.x < 0 && c.w < 0) {
        long j = i + 1;
        int cnt = 1;
        while (j < n && !head[j]) { ++cnt; ++j; }
        c.w = -cnt;
    }
    cons[pos[i]] = c;
    cinst[pos[i]] = r.inst;
}

__global__ void k_inst_offsets(int nI, const uint32_t* __restrict__ count, const int* __restrict__ cinst,
                               int* __restrict__ off) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > nI) return;
    long lo = 0, hi = *count;
    while (lo < hi) {
        long mid = (lo + hi) >> 1;
        if (cinst[mid] < i) lo = mid + 1;
        else hi = mid;
    }
    off[i] = (int)lo;
}

// ---- intersection check (Check_Edge_Tri_Intersect, FEM/IPC.h:2444-2517):
// one lane group per surface triangle walks the cells of the triangle's box
// in the edge grid; each (triangle, edge) pair is tested once (lowest shared
// cell) after the reference's exclusions (shared vertex; triangle and edge
// all DBC), an AABB overlap test and the exact segment-triangle test
__global__ void k_query_tri_edges(long nT, const int* __restrict__ tris, const int* __restrict__ tinst,
                                  const unsigned char* __restrict__ active, const double* __restrict__ X,
                                  const unsigned char* __restrict__ dbc, const int2* __restrict__ edges,
                                  const BoxI* __restrict__ tbox, const BoxI* __restrict__ ebox,
                                  const GridP* __restrict__ gp, CellHash cells, const uint32_t* __restrict__ cstart,
                                  const uint32_t* __restrict__ entries, Cand* __restrict__ out, unsigned int* counter,
                                  long cap, unsigned int* __restrict__ inst_count) {
    const long f = ((long)blockIdx.x * blockDim.x + threadIdx.x) / kQueryLanes;
    if (f >= nT) return;  // the whole group leaves together
    const int inst = tinst[f];
    if (!active[inst]) return;
    const int t0 = tris[3 * f], t1 = tris[3 * f + 1], t2 = tris[3 * f + 2];
    const double ta[3] = {X[3 * t0], X[3 * t0 + 1], X[3 * t0 + 2]};
    const double tb[3] = {X[3 * t1], X[3 * t1 + 1], X[3 * t1 + 2]};
    const double tc[3] = {X[3 * t2], X[3 * t2 + 1], X[3 * t2 + 2]};
    double tmin[3], tmax[3];
    for (int d = 0; d < 3; ++d) {
        tmin[d] = fmin(fmin(ta[d], tb[d]), tc[d]);
        tmax[d] = fmax(fmax(ta[d], tb[d]), tc[d]);
    }
    const bool tdbc = dbc[t0] && dbc[t1] && dbc[t2];
    const BoxI qb = tbox[f];
    const GridP g = gp[inst];
    group_walk_emit<kQueryLanes>(qb, inst, g, cells, cstart, entries, out, counter, cap,
                   [&](uint32_t ent, int cx, int cy, int cz, Cand& c) -> bool {
                       const int eJ = (int)ent;
                       if (!is_first_shared(qb, ebox[eJ], cx, cy, cz)) return false;
                       const int2 m = edges[eJ];
                       if (m.x == t0 || m.x == t1 || m.x == t2 || m.y == t0 || m.y == t1 || m.y == t2) return false;
                       if (tdbc && dbc[m.x] && dbc[m.y]) return false;
                       const double e0[3] = {X[3 * m.x], X[3 * m.x + 1], X[3 * m.x + 2]};
                       const double e1[3] = {X[3 * m.y], X[3 * m.y + 1], X[3 * m.y + 2]};
                       for (int d = 0; d < 3; ++d)
                           if (fmax(e0[d], e1[d]) < tmin[d] || fmin(e0[d], e1[d]) > tmax[d]) return false;
                       if (!pred::seg_tri_intersect(e0, e1, ta, tb, tc)) return false;
                       atomicAdd(inst_count + inst, 1u);
                       c = {(int)f, eJ};
                       return true;
                   });
}

__global__ void k_min_dist2(long C, const int4* __restrict__ cons, const int* __restrict__ cinst,
                            const unsigned char* __restrict__ active, const double* __restrict__ X,
                            double* __restrict__ dist2, double* __restrict__ inst_min) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    int inst = cinst[i];
    Stencil st = decode(cons[i]);
    double d = stencil_dist2(st, X);
    if (dist2) dist2[i] = d;
    if (inst_min && active[inst]) atomic_min_nonneg(inst_min + inst, d);
}

}  // namespace

// ---------------------------------------------------------------- host side
int box_grid_count(Work& W, int slot, const BoxI* boxes, const int* inst, const unsigned char* active, long nprim,
                   uint32_t* h_total, cudaStream_t s) {
    DBuf& bcnt = W[(slot == 0 ? W_GRID0 : W_GRID1) + 0];
    long np = nprim > 0 ? nprim : 1;
    if (bcnt.ensure(sizeof(uint32_t) * (np + 1))) return IDP_ERR_CUDA;
    if (W[W_SCRATCH].ensure(scan_scratch_bytes(np) + 64)) return IDP_ERR_CUDA;
    uint32_t* cnt = bcnt.as<uint32_t>();
    (::idp::count_launch(), k_box_count<<<grid_for(np), kBlock, 0, s>>>(nprim, boxes, inst, active, cnt));
    if (scan_exclusive(cnt, cnt, nprim, cnt + nprim, W[W_SCRATCH].p, s) != cudaSuccess) return IDP_ERR_CUDA;
    IDP_CUDA_TRY(cudaMemcpyAsync(h_total, cnt + nprim, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    return IDP_OK;
}

int grid_cell_bases(Work& W, const GridP* gp, int nI, unsigned long long* h_cells, cudaStream_t s) {
    if (W[W_CBASE].ensure(sizeof(uint32_t) * (nI + 1) + 64)) return IDP_ERR_CUDA;
    uint32_t* cbase = W[W_CBASE].as<uint32_t>();
    unsigned long long* total = reinterpret_cast<unsigned long long*>(W[W_CBASE].as<char>() +
                                                                      ((sizeof(uint32_t) * (nI + 1) + 15) & ~size_t(15)));
    (::idp::count_launch(), k_cell_bases<<<1, 1, 0, s>>>(nI, gp, cbase, total, ~0ull, nullptr));
    IDP_CUDA_TRY(cudaMemcpyAsync(h_cells, total, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    return IDP_OK;
}

int box_grid_finish(Work& W, int slot, const BoxI* boxes, const int* inst, const unsigned char* active, long nprim,
                    const GridP* gp, int nI, long ne, unsigned long long ncells, BoxGrid& out, cudaStream_t s) {
    int base = slot == 0 ? W_GRID0 : W_GRID1;
    DBuf& bcnt = W[base + 0];
    DBuf& bkeys = W[base + 1];
    DBuf& bvals = W[base + 2];
    DBuf& bkeys2 = W[base + 3];
    DBuf& bvals2 = W[base + 4];
    DBuf& bcell = W[base + 5];
    long np = nprim > 0 ? nprim : 1;
    long nalloc = ne > 0 ? ne : 1;
    if (ncells > 0 && ncells <= kDenseMaxCells) {
        // dense table: cstart (ncells + 1) | per-cell counts (ncells + 1)
        const long nc = (long)ncells;
        if (bvals.ensure(4 * nalloc) || bcell.ensure(sizeof(uint32_t) * 2 * (nc + 1) + 64) ||
            W[W_SCRATCH].ensure(scan_scratch_bytes(nc) + 64))
            return IDP_ERR_CUDA;
        uint32_t* cstart = bcell.as<uint32_t>();
        uint32_t* ccount = cstart + nc + 1;
        const uint32_t* cbase = W[W_CBASE].as<uint32_t>();
        IDP_CUDA_TRY(cudaMemsetAsync(ccount, 0, sizeof(uint32_t) * (nc + 1), s));
        if (nprim > 0)
            (::idp::count_launch(), k_dense_count<<<grid_for(np), kBlock, 0, s>>>(nprim, boxes, inst, active, gp, cbase,
                                                                                  ccount));
        if (scan_exclusive(ccount, cstart, nc, cstart + nc, W[W_SCRATCH].p, s) != cudaSuccess) return IDP_ERR_CUDA;
        if (nprim > 0)
            (::idp::count_launch(), k_dense_fill<<<grid_for(np), kBlock, 0, s>>>(nprim, boxes, inst, active, gp, cbase,
                                                                                 cstart, ccount, bvals.as<uint32_t>()));
        out.cell_start = cstart;
        out.entries = bvals.as<uint32_t>();
        out.cells = CellHash();
        out.cells.dense = 1;
        out.cells.cbase = cbase;
        out.cells.cap = (uint32_t)nc;
        out.nent = ne;
        return IDP_OK;
    }
    // the sort's spare buffers later hold the cell hash (2x entries, power of two)
    uint32_t hcap = 16;
    while ((long)hcap < 2 * nalloc) hcap <<= 1;
    if (bkeys.ensure(8 * nalloc) || bvals.ensure(4 * nalloc) || bkeys2.ensure(8 * (long)hcap) ||
        bvals2.ensure(4 * (long)hcap))
        return IDP_ERR_CUDA;
    if (bcell.ensure((8 + 4) * (nalloc + 1) + 4 * (nalloc + 1) * 2 + 64)) return IDP_ERR_CUDA;
    uint32_t* cnt = bcnt.as<uint32_t>();
    (::idp::count_launch(), k_box_emit<<<grid_for(np), kBlock, 0, s>>>(nprim, boxes, inst, active, gp, cnt,
                                                                       bkeys.as<uint64_t>(), bvals.as<uint32_t>()));
    int bits = 32 + bits_for((uint64_t)(nI > 0 ? nI : 1));
    if (W[W_SCRATCH].ensure(radix_sort_scratch_bytes(nalloc) + scan_scratch_bytes(nalloc) + 64)) return IDP_ERR_CUDA;
    if (radix_sort_pairs(bkeys.as<uint64_t>(), bvals.as<uint32_t>(), bkeys2.as<uint64_t>(), bvals2.as<uint32_t>(), ne,
                         bits, W[W_SCRATCH].p, s) != cudaSuccess)
        return IDP_ERR_CUDA;
    // cell table: cstart (4B x (ne+1)) | head | idx (+ cell count at idx[ne]);
    // the hash (twice the entries, rounded up to a power of two) reuses the
    // sort's spare buffers
    uint32_t* cstart = bcell.as<uint32_t>();
    uint32_t* head = cstart + nalloc + 1;
    uint32_t* idx = head + nalloc + 1;
    unsigned long long* hkey = bkeys2.as<unsigned long long>();
    uint32_t* hval = bvals2.as<uint32_t>();
    IDP_CUDA_TRY(cudaMemsetAsync(hkey, 0xff, sizeof(unsigned long long) * hcap, s));
    if (ne > 0) {
        (::idp::count_launch(), k_mark_heads<<<grid_for(ne), kBlock, 0, s>>>(ne, bkeys.as<uint64_t>(), head));
        if (scan_exclusive(head, idx, ne, idx + ne, W[W_SCRATCH].p, s) != cudaSuccess) return IDP_ERR_CUDA;
        (::idp::count_launch(), k_cell_table<<<grid_for(ne), kBlock, 0, s>>>(ne, bkeys.as<uint64_t>(), head, idx, cstart,
                                                                              idx + ne, hkey, hval, hcap - 1));
    } else {
        IDP_CUDA_TRY(cudaMemsetAsync(cstart, 0, sizeof(uint32_t), s));
    }
    out.cell_start = cstart;
    out.entries = bvals.as<uint32_t>();
    out.cells = CellHash();
    out.cells.key = hkey;
    out.cells.val = hval;
    out.cells.mask = hcap - 1;
    out.nent = ne;
    return IDP_OK;
}

bool grids_overflowed(Work& W, int set, unsigned int flag) {
    if (!flag) return false;
    W.dense_ready[set] = false;  // the next build counts with a round trip and resizes
    return true;
}

int grids_build(Work& W, int set, const BoxI* tbox, long nt, const int* tinst, const BoxI* ebox, long ne,
                const int* einst, const unsigned char* active, const GridP* gp, int nI, unsigned int* d_flag,
                BoxGrid& gt, BoxGrid& ge, cudaStream_t s) {
    if (W[W_CBASE].ensure(sizeof(uint32_t) * (nI + 1) + 64)) return IDP_ERR_CUDA;
    uint32_t* cbase = W[W_CBASE].as<uint32_t>();
    unsigned long long* d_total = reinterpret_cast<unsigned long long*>(W[W_CBASE].as<char>() +
                                                                        ((sizeof(uint32_t) * (nI + 1) + 15) & ~size_t(15)));
    if (W.dense_ready[set]) {
        // dense tables at the capacities of earlier builds, no round trip
        const unsigned long long cap = W.dense_cells_cap[set];
        const long ent_cap = W.dense_ent_cap[set];
        const size_t slots = 2 * (size_t)(cap + 1);
        DBuf& tab = W[set ? W_DENSE1 : W_DENSE0];
        DBuf& ent = W[W_GRID0 + 2];
        if (tab.ensure(sizeof(uint32_t) * (2 * slots + 2)) || ent.ensure(sizeof(uint32_t) * (ent_cap + 1)) ||
            W[W_SCRATCH].ensure(scan_scratch_bytes((long)slots) + 64))
            return IDP_ERR_CUDA;
        uint32_t* ccount = tab.as<uint32_t>();
        uint32_t* cstart = ccount + slots + 1;
        (::idp::count_launch(), k_cell_bases<<<1, 1, 0, s>>>(nI, gp, cbase, d_total, cap, d_flag));
        IDP_CUDA_TRY(cudaMemsetAsync(ccount, 0, sizeof(uint32_t) * slots, s));
        const long n = nt + ne;
        if (n > 0)
            (::idp::count_launch(), k_dense_count2<<<grid_for(n), kBlock, 0, s>>>(nt, ne, tbox, tinst, ebox, einst, active,
                                                                                  gp, cbase, (uint32_t)cap, ccount));
        if (scan_exclusive(ccount, cstart, (long)slots, cstart + slots, W[W_SCRATCH].p, s) != cudaSuccess)
            return IDP_ERR_CUDA;
        if (n > 0)
            (::idp::count_launch(), k_dense_fill2<<<grid_for(n), kBlock, 0, s>>>(
                                        nt, ne, tbox, tinst, ebox, einst, active, gp, cbase, (uint32_t)cap, cstart,
                                        ccount, ent.as<uint32_t>(), ent_cap, d_flag));
        for (int g = 0; g < 2; ++g) {
            BoxGrid& o = g ? ge : gt;
            o.cell_start = cstart + (size_t)g * (cap + 1);
            o.entries = ent.as<uint32_t>();
            o.cells = CellHash();
            o.cells.dense = 1;
            o.cells.cbase = cbase;
            o.cells.cap = (uint32_t)cap;
            o.cells.ent_cap = (uint32_t)ent_cap;
            o.nent = -1;
        }
        return IDP_OK;
    }
    // counted build with one round trip; records capacities for the next ones
    uint32_t* hp = W.pinned();
    if (!hp) return IDP_ERR_CUDA;
    unsigned long long* hcells = reinterpret_cast<unsigned long long*>(hp + 8);
    int rc = box_grid_count(W, 0, tbox, tinst, active, nt, hp, s);
    if (!rc) rc = box_grid_count(W, 1, ebox, einst, active, ne, hp + 1, s);
    if (!rc) rc = grid_cell_bases(W, gp, nI, hcells, s);
    if (rc) return rc;
    IDP_CUDA_TRY(cudaStreamSynchronize(s));
    const long nt_ent = hp[0], ne_ent = hp[1];
    const unsigned long long ncells = *hcells;
    if ((rc = box_grid_finish(W, 0, tbox, tinst, active, nt, gp, nI, nt_ent, ncells, gt, s))) return rc;
    if ((rc = box_grid_finish(W, 1, ebox, einst, active, ne, gp, nI, ne_ent, ncells, ge, s))) return rc;
    if (ncells > 0 && ncells * 5 / 4 + 1024 <= kDenseMaxCells) {
        W.dense_ready[set] = true;
        W.dense_cells_cap[set] = std::max(W.dense_cells_cap[set], ncells * 5 / 4 + 1024);
        W.dense_ent_cap[set] = std::max(W.dense_ent_cap[set], (nt_ent + ne_ent) * 5 / 4 + 1024);
    }
    return IDP_OK;
}

// per-instance grid over the surface at X and the integer boxes of every
// surface triangle and edge in it
static int surface_boxes(Arena& A, Work& W, const double* X, GridP*& gp, BoxI*& tbox, BoxI*& ebox, cudaStream_t s) {
    const int nI = A.nI;
    if (W[W_BBOX].ensure(sizeof(unsigned long long) * 6 * nI) || W[W_GRIDP].ensure(sizeof(GridP) * nI))
        return IDP_ERR_CUDA;
    unsigned long long* bb = W[W_BBOX].as<unsigned long long>();
    gp = W[W_GRIDP].as<GridP>();
    (::idp::count_launch(), k_bbox_init<<<grid_for(6 * nI), kBlock, 0, s>>>(nI, bb));
    if (A.Sn) (::idp::count_launch(), k_bbox<<<grid_for(A.Sn), kBlock, 0, s>>>(A.Sn, A.snode, A.sn_inst, A.active, X, bb));
    (::idp::count_launch(), k_grid_params<<<grid_for(nI), kBlock, 0, s>>>(nI, bb, A.cell, A.dHat2, A.thickness, A.active, gp));
    long St = A.St > 0 ? A.St : 1, Se = A.Se > 0 ? A.Se : 1;
    if (W[W_BOX_A].ensure(sizeof(BoxI) * St) || W[W_BOX_B].ensure(sizeof(BoxI) * Se)) return IDP_ERR_CUDA;
    tbox = W[W_BOX_A].as<BoxI>();
    ebox = W[W_BOX_B].as<BoxI>();
    if (A.St) (::idp::count_launch(), k_prim_boxes<3><<<grid_for(A.St), kBlock, 0, s>>>(A.St, A.stri, A.st_inst, A.active, X, gp, tbox));
    if (A.Se)
        (::idp::count_launch(), k_prim_boxes<2><<<grid_for(A.Se), kBlock, 0, s>>>(A.Se, reinterpret_cast<const int*>(A.sedge), A.se_inst,
                                                           A.active, X, gp, ebox));
    return IDP_OK;
}

int build_constraint_set(Arena& A, Work& W, const double* X, ContactSet& cs, cudaStream_t s) {
    const int nI = A.nI;
    // 1-2. per-instance grid parameters, triangle and edge boxes
    GridP* gp = nullptr;
    BoxI *tbox = nullptr, *ebox = nullptr;
    if (int r = surface_boxes(A, W, X, gp, tbox, ebox, s)) return r;
    // 3. grids and candidates: PT in [0, cap_pt), EE in [cap_pt, cap_pt +
    // cap_ee); one host round trip reads both counts and the grids' overflow
    // flag (ccount[2])
    uint32_t* hp = W.pinned();
    if (!hp) return IDP_ERR_CUDA;
    if (W[W_CAND_CNT].ensure(64)) return IDP_ERR_CUDA;
    unsigned int* ccount = W[W_CAND_CNT].as<unsigned int>();
    long cap_pt = std::max<long>(W.cand_cap_pt, 2 * A.Sn + 512);
    long cap_ee = std::max<long>(W.cand_cap_ee, 2 * A.Se + 512);
    int rc = IDP_OK;
    for (int attempt = 0; attempt < 6; ++attempt) {
        BoxGrid gt, ge;
        IDP_CUDA_TRY(cudaMemsetAsync(ccount, 0, 3 * sizeof(unsigned int), s));
        if ((rc = grids_build(W, 0, tbox, A.St, A.st_inst, ebox, A.Se, A.se_inst, A.active, gp, nI, ccount + 2, gt, ge,
                              s)))
            return rc;
        if (W[W_CAND].ensure(sizeof(Cand) * (cap_pt + cap_ee))) return IDP_ERR_CUDA;
        Cand* cand = W[W_CAND].as<Cand>();
        if (A.Sn)
            (::idp::count_launch(), k_query_pt<<<grid_for(kQueryLanes * A.Sn), kBlock, 0, s>>>(A.Sn, A.snode, A.sn_inst, A.active, X, A.dbc_excl, A.stri, tbox, gp,
                                                         A.dHat2, A.thickness, gt.cells, gt.cell_start,
                                                         gt.entries, cand, ccount, cap_pt));
        if (A.Se)
            (::idp::count_launch(), k_query_ee<<<grid_for(kQueryLanes * A.Se), kBlock, 0, s>>>(A.Se, A.sedge, A.se_inst, A.active, X, A.dbc_excl, ebox, gp, A.dHat2,
                                                         A.thickness, ge.cells, ge.cell_start, ge.entries,
                                                         cand + cap_pt, ccount + 1, cap_ee));
        IDP_CUDA_TRY(cudaMemcpyAsync(hp + 2, ccount, 3 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        const long npt = hp[2], nee = hp[3];
        if (grids_overflowed(W, 0, hp[4])) continue;
        if (npt > cap_pt || nee > cap_ee) {
            if (npt > cap_pt) cap_pt = npt + npt / 2 + 1024;
            if (nee > cap_ee) cap_ee = nee + nee / 2 + 1024;
            W.cand_cap_pt = cap_pt;
            W.cand_cap_ee = cap_ee;
            continue;
        }
        if (npt + nee == 0) {
            cs.C = 0;
            cs.off.assign(nI + 1, 0);
            if (W[W_CONS_OFF].ensure(sizeof(int) * (nI + 1)) || W[W_CONS].ensure(sizeof(int4)) ||
                W[W_CONS_INST].ensure(sizeof(int)))
                return IDP_ERR_CUDA;
            IDP_CUDA_TRY(cudaMemsetAsync(W[W_CONS_OFF].p, 0, sizeof(int) * (nI + 1), s));
            cs.d_off = W[W_CONS_OFF].as<int>();
            return IDP_OK;
        }
        {
            // 4. narrow phase
            long rcap = (long)(W[W_CONS_TMP].bytes / sizeof(Rec));
            if (rcap < npt + nee + 1) {
                rcap = npt + nee + 1;
                if (W[W_CONS_TMP].ensure(sizeof(Rec) * rcap)) return IDP_ERR_CUDA;
            }
            Rec* recs = W[W_CONS_TMP].as<Rec>();
            IDP_CUDA_TRY(cudaMemsetAsync(ccount, 0, sizeof(unsigned int), s));
            if (npt)
                (::idp::count_launch(), k_narrow_pt<<<grid_for(npt), kBlock, 0, s>>>(npt, cand, A.snode, A.sn_inst, A.stri, X, A.dHat2, A.thickness,
                                                             recs, ccount, rcap));
            if (nee)
                (::idp::count_launch(), k_narrow_ee<<<grid_for(nee), kBlock, 0, s>>>(nee, cand + cap_pt, A.sedge, A.se_inst, X, A.X0, A.dHat2,
                                                             A.thickness, recs, ccount, rcap));
            unsigned int nrec = 0;
            IDP_CUDA_TRY(cudaMemcpyAsync(&nrec, ccount, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
            IDP_CUDA_TRY(cudaStreamSynchronize(s));
            long n = nrec;
            // 5. sort by (inst, c0, c1, c2, c3) and merge PP/PE duplicates
            long na = n > 0 ? n : 1;
            if (W[W_CONS_KEY_LO].ensure(8 * na) || W[W_CONS_KEY_HI].ensure(8 * na) || W[W_CONS_PERM].ensure(4 * na) ||
                W[W_CONS_PERM2].ensure(4 * na) || W[W_CONS_HEAD].ensure(8 * (na + 1)) ||
                W[W_CONS].ensure(sizeof(int4) * na) || W[W_CONS_INST].ensure(sizeof(int) * na) ||
                W[W_CONS_OFF].ensure(sizeof(int) * (nI + 1)) || W[W_SCRATCH2].ensure(8 * na + 64) ||
                W[W_MISC2].ensure(4 * na + 64))
                return IDP_ERR_CUDA;
            if (W[W_SCRATCH].ensure(radix_sort_scratch_bytes(na) + scan_scratch_bytes(na) + 64)) return IDP_ERR_CUDA;
            int b = bits_for((uint64_t)(2 * A.V + 4));
            int offv = (int)(A.V + 2);
            uint64_t* klo = W[W_CONS_KEY_LO].as<uint64_t>();
            uint64_t* khi = W[W_CONS_KEY_HI].as<uint64_t>();
            uint32_t* p1 = W[W_CONS_PERM].as<uint32_t>();
            uint32_t* p2 = W[W_CONS_PERM2].as<uint32_t>();
            uint64_t* kalt = W[W_SCRATCH2].as<uint64_t>();
            uint32_t* valt = W[W_MISC2].as<uint32_t>();
            int4* cons = W[W_CONS].as<int4>();
            int* cinst = W[W_CONS_INST].as<int>();
            uint32_t total = 0;
            if (n > 0) {
                (::idp::count_launch(), k_rec_keys<<<grid_for(n), kBlock, 0, s>>>(n, recs, b, offv, klo, p1));
                if (radix_sort_pairs(klo, p1, kalt, valt, n, 2 * b, W[W_SCRATCH].p, s) != cudaSuccess) return IDP_ERR_CUDA;
                (::idp::count_launch(), k_rec_keys_hi<<<grid_for(n), kBlock, 0, s>>>(n, recs, p1, b, offv, khi, p2));
                if (radix_sort_pairs(khi, p2, kalt, valt, n, 2 * b + bits_for((uint64_t)nI), W[W_SCRATCH].p, s) !=
                    cudaSuccess)
                    return IDP_ERR_CUDA;
                uint32_t* head = W[W_CONS_HEAD].as<uint32_t>();
                uint32_t* pos = head + na + 1;
                (::idp::count_launch(), k_merge_heads<<<grid_for(n), kBlock, 0, s>>>(n, recs, p2, head));
                if (scan_exclusive(head, pos, n, pos + n, W[W_SCRATCH].p, s) != cudaSuccess) return IDP_ERR_CUDA;
                (::idp::count_launch(), k_merge_write<<<grid_for(n), kBlock, 0, s>>>(n, recs, p2, head, pos, cons, cinst));
                // per-instance offsets from the device-side count, then one
                // round trip for the count and the offsets
                (::idp::count_launch(), k_inst_offsets<<<grid_for(nI + 1), kBlock, 0, s>>>(nI, pos + n, cinst,
                                                                                            W[W_CONS_OFF].as<int>()));
                cs.off.resize(nI + 1);
                IDP_CUDA_TRY(cudaMemcpyAsync(&total, pos + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                IDP_CUDA_TRY(cudaMemcpyAsync(cs.off.data(), W[W_CONS_OFF].as<int>(), sizeof(int) * (nI + 1),
                                             cudaMemcpyDeviceToHost, s));
                IDP_CUDA_TRY(cudaStreamSynchronize(s));
            } else {
                cs.off.assign(nI + 1, 0);
                IDP_CUDA_TRY(cudaMemsetAsync(W[W_CONS_OFF].p, 0, sizeof(int) * (nI + 1), s));
            }
            cs.C = total;
            cs.d_off = W[W_CONS_OFF].as<int>();
            return IDP_OK;
        }
    }
    return IDP_ERR_CAPACITY;
}

int edge_tri_intersections(Arena& A, Work& W, const double* X, unsigned int* inst_count, const int2** pairs,
                           long* npairs, cudaStream_t s) {
    const int nI = A.nI;
    GridP* gp = nullptr;
    BoxI *tbox = nullptr, *ebox = nullptr;
    if (int r = surface_boxes(A, W, X, gp, tbox, ebox, s)) return r;
    uint32_t* hp = W.pinned();
    if (!hp || W[W_CAND_CNT].ensure(64)) return IDP_ERR_CUDA;
    unsigned int* ccount = W[W_CAND_CNT].as<unsigned int>();
    long cap = std::max<long>(W.isect_cap, 1024);
    for (int attempt = 0; attempt < 6; ++attempt) {
        BoxGrid gt, ge;
        IDP_CUDA_TRY(cudaMemsetAsync(ccount, 0, 3 * sizeof(unsigned int), s));
        IDP_CUDA_TRY(cudaMemsetAsync(inst_count, 0, sizeof(unsigned int) * nI, s));
        if (int r = grids_build(W, 0, tbox, A.St, A.st_inst, ebox, A.Se, A.se_inst, A.active, gp, nI, ccount + 2, gt,
                                ge, s))
            return r;
        if (W[W_CAND].ensure(sizeof(Cand) * cap)) return IDP_ERR_CUDA;
        Cand* out = W[W_CAND].as<Cand>();
        if (A.St)
            (::idp::count_launch(),
             k_query_tri_edges<<<grid_for(kQueryLanes * A.St), kBlock, 0, s>>>(
                 A.St, A.stri, A.st_inst, A.active, X, A.dbc_excl, A.sedge, tbox, ebox, gp, ge.cells, ge.cell_start,
                 ge.entries, out, ccount, cap, inst_count));
        IDP_CUDA_TRY(cudaMemcpyAsync(hp + 2, ccount, 3 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        if (grids_overflowed(W, 0, hp[4])) continue;
        const long n = hp[2];
        if (n > cap) {
            cap = n + n / 2 + 1024;
            W.isect_cap = cap;
            continue;
        }
        *pairs = reinterpret_cast<const int2*>(out);
        *npairs = n;
        return IDP_OK;
    }
    return IDP_ERR_CAPACITY;
}

int constraint_min_dist2(Arena& A, Work& W, const double* X, const int4* cons, const int* cinst, long C,
                         double* dist2, double* inst_min, cudaStream_t s) {
    (void)W;
    if (C <= 0) return IDP_OK;
    (::idp::count_launch(), k_min_dist2<<<grid_for(C), kBlock, 0, s>>>(C, cons, cinst, A.active, X, dist2, inst_min));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

}  // namespace idp
