// Intersection-free step size (compiled with --fmad=false): GPU restatement
// of Compute_Intersection_Free_StepSize, 3D tet-surface branch
// (FEM/IPC.h:1879-2244), with the CCD spatial hash of Grid/SPATIAL_HASH.h:432-622
// and additive CCD of Math/Distance/CCD.h:279-395.
//
// The reference's hash changes the result (its span cap lowers the starting
// step, and pairs whose voxel boxes do not overlap are never tested), so the
// voxel grid is replicated exactly: voxel size = mean surface-edge length,
// span cap = alpha * mean|dir| / voxel size, grid corner = min over x and
// x + alpha*dir minus thickness/2, floor((p - corner) / voxel) per axis. The
// two means are summed in the reference's own order: the edge lengths as
// Eigen's vectorised mean() adds them, |dir| by the reference's serial loop
// (SPATIAL_HASH.h:455-475). A pair is tested iff the integer boxes overlap.
//
// Every pair's ACCD result is independent of the order pairs are visited (a
// pair either finishes below the bound with its own toc, or is discarded), so
// alpha = min(capped alpha, min over pairs) is exact. ACCD loops carry an
// iteration cap; a capped pair reports its accumulated (still safe) toc.
#include <cstdlib>
#include <algorithm>
#include "engine.hpp"
#include "grid.cuh"
#include "geom.cuh"
#include "prims.cuh"

namespace idp {

using namespace geo;

namespace {

constexpr int ACCD_MAX_ITERS = 200000;
// diagnostics (read back when IDP_PROFILE is set): longest ACCD loop,
// pairs above 1000 iterations, total iterations, pairs
__device__ unsigned long long g_accd_stats[4];

__global__ void k_edge_len(long nE, const int2* __restrict__ e, const double* __restrict__ X, double* __restrict__ len) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nE) return;
    int2 v = e[i];
    len[i] = sqrt(sqn(ld3(X, v.x) - ld3(X, v.y)));
}

__global__ void k_abs_dir(long nN, const int* __restrict__ nodes, const double* __restrict__ dir, double* __restrict__ out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nN) return;
    int v = nodes[i];
    out[3 * i] = fabs(dir[3 * v]);
    out[3 * i + 1] = fabs(dir[3 * v + 1]);
    out[3 * i + 2] = fabs(dir[3 * v + 2]);
}

// first level of the fixed-order estimate of sum |dir| (a span cap can only
// apply when this estimate comes near 1), one CTA per 2048-item tile of every
// instance's |dir| segment
__global__ void k_span_tiles(const SpanTile* __restrict__ tiles, const unsigned char* __restrict__ active,
                             const double* __restrict__ absdir, double* __restrict__ out) {
    __shared__ double a[256];
    const SpanTile t = tiles[blockIdx.x];
    if (!active[t.inst]) return;
    const double* in = absdir + t.start;
    double s = 0.0;
    for (int r = 0; r < 8; ++r) {
        long i = (long)t.k * 2048 + r * 256 + threadIdx.x;
        if (i < t.m) s += in[i];
    }
    a[threadIdx.x] = s;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) a[threadIdx.x] += a[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = a[0];
}

constexpr int kStageTile = 1024;  // items staged in shared memory per step (multiple of 8)

// Sum of x[0..n) in the order of Eigen's vectorised redux of a dense double
// vector on the reference's AVX build (`eLen.mean()`, SPATIAL_HASH.h:455-464;
// Eigen/src/Core/Redux.h, LinearVectorizedTraversal over 4-lane packets):
// lane l of accumulator 0 sums items l, l+8, ..., lane l of accumulator 1
// items 4+l, 12+l, ... over the first 8*floor(n/8) items; the accumulators
// are added lane by lane, one more 4-item packet is added when n mod 8 >= 4,
// the lanes reduce as (l0 + l2) + (l1 + l3) and the last n mod 4 items follow
// one at a time; fewer than 4 items are summed left to right. The whole CTA
// stages the items through shared memory (double-buffered tiles); threads
// 0-7 carry the eight accumulator lanes. Every thread must call it; thread 0
// receives the result.
__device__ double cta_eigen_sum(const double* __restrict__ x, long n, double (*buf)[kStageTile]) {
    const int tid = threadIdx.x;
    const long aligned = n & ~3L, aligned2 = n & ~7L;
    double acc = 0.0;
    if (aligned > 4) {
        for (long base = 0, k = 0; base < aligned2; base += kStageTile, ++k) {
            double* t = buf[k & 1];
            const long m = min((long)kStageTile, aligned2 - base);
            for (long i = tid; i < m; i += blockDim.x) t[i] = x[base + i];
            __syncthreads();
            if (tid < 8) {
#pragma unroll 8
                for (long i = tid; i < m; i += 8) acc += t[i];
            }
        }
        __syncthreads();
    } else if (aligned == 4 && tid < 4) {
        acc = x[tid];
    }
    __shared__ double lanes[8];
    if (tid < 8) lanes[tid] = acc;
    __syncthreads();
    double res = 0.0;
    if (tid == 0) {
        if (aligned == 0) {
            if (n > 0) {
                res = x[0];
                for (long i = 1; i < n; ++i) res += x[i];
            }
        } else {
            double p[4] = {lanes[0], lanes[1], lanes[2], lanes[3]};
            if (aligned > 4) {
                for (int l = 0; l < 4; ++l) p[l] = p[l] + lanes[4 + l];
                if (aligned > aligned2)
                    for (int l = 0; l < 4; ++l) p[l] = p[l] + x[aligned2 + l];
            }
            res = (p[0] + p[2]) + (p[1] + p[3]);
            for (long i = aligned; i < n; ++i) res += x[i];
        }
    }
    __syncthreads();
    return res;
}

// x[0] + x[1] + ... + x[n-1] added left to right into one accumulator (the
// reference's serial loop), the items staged through shared memory by the
// whole CTA while thread 0 adds the previous tile. Every thread must call
// it; thread 0 receives the result.
__device__ double cta_serial_sum(const double* __restrict__ x, long n, double (*buf)[kStageTile]) {
    const int tid = threadIdx.x;
    double acc = 0.0;
    for (long base = 0, k = 0; base < n; base += kStageTile, ++k) {
        double* t = buf[k & 1];
        const long m = min((long)kStageTile, n - base);
        for (long i = tid; i < m; i += blockDim.x) t[i] = x[base + i];
        __syncthreads();
        if (tid == 0) {
#pragma unroll 8
            for (long i = 0; i < m; ++i) acc += t[i];
        }
    }
    __syncthreads();
    return acc;
}

// fixed-order sum of the tile sums (used for the span-cap estimate only)
__device__ double cta_tree_sum(const double* x, long n, double* scratch) {
    __shared__ double a[256];
    if (n <= 0) return 0.0;
    const double* in = x;
    long m = n;
    double* out = scratch;
    while (true) {
        long tiles = (m + 2047) / 2048;
        for (long k = 0; k < tiles; ++k) {
            double s = 0.0;
            for (int r = 0; r < 8; ++r) {
                long i = k * 2048 + r * 256 + threadIdx.x;
                if (i < m) s += in[i];
            }
            a[threadIdx.x] = s;
            __syncthreads();
            for (int st = 128; st > 0; st >>= 1) {
                if (threadIdx.x < st) a[threadIdx.x] += a[threadIdx.x + st];
                __syncthreads();
            }
            if (threadIdx.x == 0) out[k] = a[0];
            __syncthreads();
        }
        if (tiles == 1) {
            double r = out[0];
            __syncthreads();
            return r;
        }
        in = out;
        out = out + tiles;
        m = tiles;
    }
}

// per instance: voxel size and span cap (SPATIAL_HASH.h:455-482). The voxel
// size is the Eigen-order mean edge length. pSize is the reference's serial
// sum; it only matters when the span exceeds 1, so it is computed (by one
// thread, 3 Sn dependent additions) only when a fixed-order estimate of the
// span is within the two sums' rounding-error bound ((n + 32) u) of 1 or
// above it.
// voxel size per instance: the mean surface edge length at X, summed in the
// reference's order (SPATIAL_HASH.h:455-465, Eigen's mean())
__global__ void k_mean_edge(int nI, const int* __restrict__ se_off, const double* __restrict__ len,
                            double* __restrict__ voxel_size) {
    __shared__ double buf[2][kStageTile];
    const int i = blockIdx.x;
    const long e0 = se_off[i], ne = se_off[i + 1] - se_off[i];
    const double es = cta_eigen_sum(len + e0, ne, buf);
    if (threadIdx.x == 0) voxel_size[i] = ne ? 1.0 * (es / (double)ne) : 1.0;
}

__global__ void k_span_cap(int nI, const unsigned char* __restrict__ active, const int* __restrict__ se_off,
                           const int* __restrict__ sn_off, const int* __restrict__ tile_off,
                           const double* __restrict__ tsum, const double* __restrict__ len,
                           const double* __restrict__ absdir, double* __restrict__ scratch,
                           double* __restrict__ alpha, double* __restrict__ voxel_size,
                           const double* __restrict__ voxel_pre) {
    __shared__ double buf[2][kStageTile];
    __shared__ double s_vsz, s_est;
    int i = blockIdx.x;
    if (!active[i]) return;
    const long e0 = se_off[i], ne = se_off[i + 1] - se_off[i];
    const long n0 = sn_off[i], nn = sn_off[i + 1] - sn_off[i];
    const int tn0 = tile_off[2 * i + 1], tn1 = tile_off[2 * i + 2];
    const int ntn = tn1 - tn0;
    double* sc = scratch + 2 * (long)tile_off[2 * i] + 8 * (long)i;
    const double es = voxel_pre ? 0.0 : cta_eigen_sum(len + e0, ne, buf);
    const double ps = ntn == 0 ? 0.0 : (ntn == 1 ? tsum[tn0] : cta_tree_sum(tsum + tn0, ntn, sc));
    const double cnt = (double)(nn * 3);
    if (threadIdx.x == 0) {
        s_vsz = voxel_pre ? voxel_pre[i] : (ne ? 1.0 * (es / (double)ne) : 1.0);
        s_est = alpha[i] * (ps / cnt) / s_vsz;
    }
    __syncthreads();
    const double vsz = s_vsz;
    double a = alpha[i];
    const double bound = 1.0 - ((double)(3 * nn) + 32.0) * 2.3e-16;
    if (!(s_est < bound)) {
        double pSize = cta_serial_sum(absdir + 3 * n0, 3 * nn, buf);
        if (threadIdx.x == 0) {
            pSize /= cnt;
            const double spanSize = a * pSize / vsz;
            if (spanSize > 1) a /= spanSize;
        }
    }
    if (threadIdx.x == 0) {
        alpha[i] = a;
        voxel_size[i] = vsz;
    }
}

__global__ void k_ccd_bbox(long nN, const int* __restrict__ nodes, const int* __restrict__ ninst,
                           const unsigned char* __restrict__ active, const double* __restrict__ X,
                           const double* __restrict__ dir, const double* __restrict__ alpha,
                           unsigned long long* __restrict__ bb) {
    long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int inst = s < nN ? ninst[s] : 0;
    const int inst_first = ninst[(long)blockIdx.x * blockDim.x];
    const bool valid = s < nN && active[inst];
    unsigned long long lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (valid) {
        int v = nodes[s];
        double a = alpha[inst];
        double p[3] = {X[3 * v], X[3 * v + 1], X[3 * v + 2]};
        double q[3] = {X[3 * v] + a * dir[3 * v], X[3 * v + 1] + a * dir[3 * v + 1], X[3 * v + 2] + a * dir[3 * v + 2]};
        for (int d = 0; d < 3; ++d) {
            lo[d] = ord_enc(fmin(p[d], q[d]));
            hi[d] = ord_enc(fmax(p[d], q[d]));
        }
    }
    bbox_block_update(valid, inst, inst_first, lo, hi, bb);
}

__global__ void k_bb_init(int nI, unsigned long long* bb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 6 * nI) return;
    bb[i] = (i % 6) < 3 ? 0xffffffffffffffffull : 0ull;
}

// SPATIAL_HASH.h:502-519
__global__ void k_ccd_grid(int nI, const unsigned char* __restrict__ active, const unsigned long long* __restrict__ bb,
                           const double* __restrict__ thick, const double* __restrict__ voxel_size,
                           GridP* __restrict__ gp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nI) return;
    GridP g;
    if (!active[i]) {
        for (int d = 0; d < 3; ++d) { g.lo[d] = 0; g.n[d] = 1; }
        g.inv = 1;
        g.s1 = 2;
        g.s2 = 4;
        gp[i] = g;
        return;
    }
    double ht = thick[i] / 2;
    double lo[3], range[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = ord_dec(bb[6 * i + d]) - ht;
        double hi = ord_dec(bb[6 * i + 3 + d]) + ht;
        range[d] = hi - lo[d];
    }
    double vs = voxel_size[i];
    double inv = 1.0 / vs;
    long vcl[3];
    for (int d = 0; d < 3; ++d) {
        long c = (long)ceil(range[d] * inv);
        vcl[d] = c > 1 ? c : 1;
    }
    long amt = vcl[0] * vcl[1] * vcl[2];
    if (amt > 1e9) {
        vs *= pow((double)amt / 1.0e9, 1.0 / 3);
        inv = 1.0 / vs;
    }
    int vc[3];
    for (int d = 0; d < 3; ++d) {
        int c = (int)ceil(range[d] * inv);
        vc[d] = c > 1 ? c : 1;
    }
    if (vc[0] <= 0 || vc[1] <= 0 || vc[2] <= 0) {
        double rmax = fmax(range[0], fmax(range[1], range[2]));
        inv = 1.0 / (rmax * 1.01);
        vc[0] = vc[1] = vc[2] = 1;
    }
    for (int d = 0; d < 3; ++d) { g.lo[d] = lo[d]; g.n[d] = vc[d]; }
    g.inv = inv;
    g.s1 = (long)vc[0] + 1;
    g.s2 = g.s1 * ((long)vc[1] + 1);
    gp[i] = g;
}

// swept voxel box of every surface node (SPATIAL_HASH.h:525-533)
__global__ void k_node_box(long nN, const int* __restrict__ nodes, const int* __restrict__ ninst,
                           const unsigned char* __restrict__ active, const double* __restrict__ X,
                           const double* __restrict__ dir, const double* __restrict__ alpha,
                           const double* __restrict__ thick, const GridP* __restrict__ gp, BoxI* __restrict__ nbox) {
    long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nN) return;
    int inst = ninst[s];
    BoxI b;
    if (!active[inst]) {
        for (int d = 0; d < 3; ++d) { b.lo[d] = 1; b.hi[d] = 0; }
        nbox[s] = b;
        return;
    }
    GridP g = gp[inst];
    int v = nodes[s];
    double a = alpha[inst], ht = thick[inst] / 2;
    for (int d = 0; d < 3; ++d) {
        double p = X[3 * v + d], q = X[3 * v + d] + a * dir[3 * v + d];
        double mn = fmin(p, q) - ht, mx = fmax(p, q) + ht;
        b.lo[d] = (int)floor((mn - g.lo[d]) * g.inv);
        b.hi[d] = (int)floor((mx - g.lo[d]) * g.inv);
    }
    nbox[s] = b;
}

template <int K>
__global__ void k_prim_box_from_nodes(long n, const int* __restrict__ verts, const int* __restrict__ v2s,
                                      const BoxI* __restrict__ nbox, BoxI* __restrict__ out) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BoxI b = nbox[v2s[verts[K * i]]];
    for (int k = 1; k < K; ++k) {
        BoxI c = nbox[v2s[verts[K * i + k]]];
        for (int d = 0; d < 3; ++d) {
            b.lo[d] = min(b.lo[d], c.lo[d]);
            b.hi[d] = max(b.hi[d], c.hi[d]);
        }
    }
    out[i] = b;
}

struct CCand {
    int a, b;
};

// candidate search runs on a grid of cells `coarse` reference voxels wide
// (per instance: the smallest power of two that keeps the instance's grid
// within kCcdCellBudget cells); the reference's test (integer voxel boxes
// overlap) is applied to every pair it returns
constexpr double kCcdCellBudget = 4194304.0;

// coarse boxes of the triangles, edges and nodes (stored in that order),
// clamped to the coarse grid [0, n]: the clamp is monotone, so every pair of
// overlapping boxes still overlaps, and all query and table cells exist
__global__ void k_coarse_boxes(long pt, long pe, long pn, long nt, long ne, long nn, const int* __restrict__ tinst,
                               const int* __restrict__ einst, const int* __restrict__ ninst,
                               const GridP* __restrict__ gc, const BoxI* __restrict__ in, BoxI* __restrict__ out) {
    // segments are padded to pt, pe, pn boxes (at least one each); padding
    // boxes are left empty
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pt + pe + pn) return;
    int inst = -1;
    if (i < pt) { if (i < nt) inst = tinst[i]; }
    else if (i < pt + pe) { if (i - pt < ne) inst = einst[i - pt]; }
    else if (i - pt - pe < nn) inst = ninst[i - pt - pe];
    BoxI b = in[i], c;
    if (inst < 0) {
        for (int d = 0; d < 3; ++d) { c.lo[d] = 1; c.hi[d] = 0; }
        out[i] = c;
        return;
    }
    const GridP g = gc[inst];
    for (int d = 0; d < 3; ++d) {
        if (b.lo[d] > b.hi[d]) {  // empty box (inactive instance) stays empty
            c.lo[d] = 1;
            c.hi[d] = 0;
            continue;
        }
        const int lo = b.lo[d] >= 0 ? b.lo[d] / g.coarse : -1;
        const int hi = b.hi[d] >= 0 ? b.hi[d] / g.coarse : -1;
        c.lo[d] = clampi(lo, 0, g.n[d]);
        c.hi[d] = clampi(hi, 0, g.n[d]);
    }
    out[i] = c;
}

__global__ void k_coarse_grid(int nI, const GridP* __restrict__ gp, GridP* __restrict__ gc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nI) return;
    GridP g = gp[i];
    int c = 1;
    while (c < (1 << 20) && ((double)(g.n[0] / c + 2) * (double)(g.n[1] / c + 2) * (double)(g.n[2] / c + 2)) >
                                kCcdCellBudget)
        c *= 2;
    g.coarse = c;
    for (int d = 0; d < 3; ++d) g.n[d] = g.n[d] / c + 1;
    g.s1 = (long)g.n[0] + 1;
    g.s2 = g.s1 * ((long)g.n[1] + 1);
    gc[i] = g;
}

__device__ __forceinline__ bool boxes_overlap(const BoxI& a, const BoxI& b) {
    for (int d = 0; d < 3; ++d)
        if (a.lo[d] > b.hi[d] || b.lo[d] > a.hi[d]) return false;
    return true;
}

__device__ __forceinline__ bool swept_far(const double* lo_a, const double* hi_a, const double* lo_b,
                                          const double* hi_b, double dist) {
    for (int d = 0; d < 3; ++d)
        if (lo_a[d] - hi_b[d] > dist || lo_b[d] - hi_a[d] > dist) return true;
    return false;
}

// one lane group per surface node: triangles whose voxel boxes overlap the node's
// swept voxel box (Query_Point_For_Primitives, SPATIAL_HASH.h:624-647), then
// the exclusions and swept-AABB test of IPC.h:1980-2006
__global__ void k_ccd_query_pt(long nN, const int* __restrict__ nodes, const int* __restrict__ ninst,
                               const unsigned char* __restrict__ active, const double* __restrict__ X,
                               const double* __restrict__ dir, const unsigned char* __restrict__ dbc,
                               const int* __restrict__ tris, const BoxI* __restrict__ nbox,
                               const BoxI* __restrict__ tbox, const BoxI* __restrict__ nboxc,
                               const BoxI* __restrict__ tboxc, const GridP* __restrict__ gp,
                               const double* __restrict__ thick, CellHash cells,
                               const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ entries,
                               CCand* __restrict__ out, unsigned int* counter, long cap) {
    long s = ((long)blockIdx.x * blockDim.x + threadIdx.x) / kCcdQueryLanes;
    if (s >= nN) return;
    int inst = ninst[s];
    if (!active[inst]) return;
    int vI = nodes[s];
    GridP g = gp[inst];
    double th = thick[inst];
    double plo[3], phi[3];
    for (int d = 0; d < 3; ++d) {
        double p = X[3 * vI + d], pe = p + dir[3 * vI + d];
        plo[d] = fmin(p, pe);
        phi[d] = fmax(p, pe);
    }
    const BoxI qc = nboxc[s], qx = nbox[s];
    const bool pdbc = dbc[vI] != 0;
    group_walk_emit<kCcdQueryLanes>(qc, inst, g, cells, cstart, entries, out, counter, cap,
                   [&](uint32_t ent, int cx, int cy, int cz, CCand& c) -> bool {
                       int f = (int)ent;
                       if (!is_first_shared(qc, tboxc[f], cx, cy, cz) || !boxes_overlap(qx, tbox[f])) return false;
                       int t0 = tris[3 * f], t1 = tris[3 * f + 1], t2 = tris[3 * f + 2];
                       if (vI == t0 || vI == t1 || vI == t2) return false;
                       if (pdbc && dbc[t0] && dbc[t1] && dbc[t2]) return false;
                       double tlo[3], thi[3];
                       const int tv[3] = {t0, t1, t2};
                       for (int d = 0; d < 3; ++d) {
                           double mn = X[3 * t0 + d], mx = mn;
                           for (int k = 0; k < 3; ++k) {
                               double a = X[3 * tv[k] + d], b = a + dir[3 * tv[k] + d];
                               mn = fmin(mn, fmin(a, b));
                               mx = fmax(mx, fmax(a, b));
                           }
                           tlo[d] = mn;
                           thi[d] = mx;
                       }
                       if (swept_far(plo, phi, tlo, thi, th)) return false;
                       c = {(int)s, f};
                       return true;
                   });
}

// one lane group per surface edge: edges eJ > eI with overlapping voxel boxes
// (SPATIAL_HASH.h:650-662), exclusions and swept-AABB test of IPC.h:2193-2230
__global__ void k_ccd_query_ee(long nE, const int2* __restrict__ edges, const int* __restrict__ einst,
                               const unsigned char* __restrict__ active, const double* __restrict__ X,
                               const double* __restrict__ dir, const unsigned char* __restrict__ dbc,
                               const BoxI* __restrict__ ebox, const BoxI* __restrict__ eboxc,
                               const GridP* __restrict__ gp, const double* __restrict__ thick,
                               CellHash cells, const uint32_t* __restrict__ cstart,
                               const uint32_t* __restrict__ entries, CCand* __restrict__ out, unsigned int* counter,
                               long cap) {
    long eI = ((long)blockIdx.x * blockDim.x + threadIdx.x) / kCcdQueryLanes;
    if (eI >= nE) return;
    int inst = einst[eI];
    if (!active[inst]) return;
    int2 mi = edges[eI];
    GridP g = gp[inst];
    double th = thick[inst];
    double alo[3], ahi[3];
    const int av[2] = {mi.x, mi.y};
    for (int d = 0; d < 3; ++d) {
        double mn = X[3 * mi.x + d], mx = mn;
        for (int k = 0; k < 2; ++k) {
            double a = X[3 * av[k] + d], b = a + dir[3 * av[k] + d];
            mn = fmin(mn, fmin(a, b));
            mx = fmax(mx, fmax(a, b));
        }
        alo[d] = mn;
        ahi[d] = mx;
    }
    const BoxI qc = eboxc[eI], qx = ebox[eI];
    const bool adbc = dbc[mi.x] && dbc[mi.y];
    group_walk_emit<kCcdQueryLanes>(qc, inst, g, cells, cstart, entries, out, counter, cap,
                   [&](uint32_t ent, int cx, int cy, int cz, CCand& c) -> bool {
                       int eJ = (int)ent;
                       if (eJ <= eI || !is_first_shared(qc, eboxc[eJ], cx, cy, cz) || !boxes_overlap(qx, ebox[eJ]))
                           return false;
                       int2 mj = edges[eJ];
                       if (mi.x == mj.x || mi.x == mj.y || mi.y == mj.x || mi.y == mj.y) return false;
                       if (adbc && dbc[mj.x] && dbc[mj.y]) return false;
                       double blo[3], bhi[3];
                       const int bv[2] = {mj.x, mj.y};
                       for (int d = 0; d < 3; ++d) {
                           double mn = X[3 * mj.x + d], mx = mn;
                           for (int k = 0; k < 2; ++k) {
                               double a = X[3 * bv[k] + d], b = a + dir[3 * bv[k] + d];
                               mn = fmin(mn, fmin(a, b));
                               mx = fmax(mx, fmax(a, b));
                           }
                           blo[d] = mn;
                           bhi[d] = mx;
                       }
                       if (swept_far(alo, ahi, blo, bhi, th)) return false;
                       c = {(int)eI, eJ};
                       return true;
                   });
}

// ---- ACCD (CCD.h:279-328, 330-395)
// Every 64 iterations a running pair compares its accumulated time of impact
// with the instance's best result so far (atomic minimum of the finished
// pairs): once above it, the pair can no longer lower the minimum (its own
// result only grows), so it stops and contributes nothing. The per-instance
// minimum, the step size, is unchanged by this.
constexpr int ACCD_POLL = 64;

__device__ __forceinline__ bool accd_beaten(double toc, const double* best) {
    return toc > *(volatile const double*)best;
}

__device__ int accd_pt(D3 p, D3 t0, D3 t1, D3 t2, D3 dp, D3 dt0, D3 dt1, D3 dt2, double eta, double thickness,
                       double& toc, int& its, const double* best) {
    D3 mov = 0.25 * (((dt0 + dt1) + dt2) + dp);
    dt0 = dt0 - mov; dt1 = dt1 - mov; dt2 = dt2 - mov; dp = dp - mov;
    double m2 = fmax(sqn(dt0), fmax(sqn(dt1), sqn(dt2)));
    double maxDispMag = sqrt(sqn(dp)) + sqrt(m2);
    if (maxDispMag == 0) return 0;
    double th2 = thickness * thickness;
    double dist2_cur = d_PT_unclassified(p, t0, t1, t2);
    double dist_cur = sqrt(dist2_cur);
    double gap = eta * (dist2_cur - th2) / (dist_cur + thickness);
    double toc_prev = toc;
    toc = 0;
    for (its = 0; its < ACCD_MAX_ITERS; ++its) {
        double tocLB = (1 - eta) * (dist2_cur - th2) / ((dist_cur + thickness) * maxDispMag);
        p = p + tocLB * dp; t0 = t0 + tocLB * dt0; t1 = t1 + tocLB * dt1; t2 = t2 + tocLB * dt2;
        // short chains share the FP64 pipe with many others: evaluate only the
        // branch taken; a chain past ACCD_POLL iterations is one of the few
        // long ones that decide the launch time: evaluate for latency
        dist2_cur = its < ACCD_POLL ? d_PT_unclassified(p, t0, t1, t2) : d_PT_unclassified_ilp(p, t0, t1, t2);
        dist_cur = sqrt(dist2_cur);
        if (toc != 0 && ((dist2_cur - th2) / (dist_cur + thickness) < gap)) return 1;
        toc += tocLB;
        if (toc > toc_prev) return 0;
        if ((its & (ACCD_POLL - 1)) == ACCD_POLL - 1 && accd_beaten(toc, best)) return 0;
    }
    return 2;
}

__device__ __forceinline__ void ee_eval(D3 ea0, D3 ea1, D3 eb0, D3 eb1, double th2, double& d2, double& dF) {
    d2 = d_EE_unclassified(ea0, ea1, eb0, eb1);
    dF = d2 - th2;
    if (dF <= 0) {
        d2 = fmin(fmin(sqn(ea0 - eb0), sqn(ea0 - eb1)), fmin(sqn(ea1 - eb0), sqn(ea1 - eb1)));
        dF = d2 - th2;
    }
}

__device__ int accd_ee(D3 ea0, D3 ea1, D3 eb0, D3 eb1, D3 dea0, D3 dea1, D3 deb0, D3 deb1, double eta,
                       double thickness, double& toc, int& its, const double* best) {
    D3 mov = 0.25 * (((dea0 + dea1) + deb0) + deb1);
    dea0 = dea0 - mov; dea1 = dea1 - mov; deb0 = deb0 - mov; deb1 = deb1 - mov;
    double maxDispMag = sqrt(fmax(sqn(dea0), sqn(dea1))) + sqrt(fmax(sqn(deb0), sqn(deb1)));
    if (maxDispMag == 0) return 0;
    double th2 = thickness * thickness;
    double dist2_cur, dFunc;
    ee_eval(ea0, ea1, eb0, eb1, th2, dist2_cur, dFunc);
    double dist_cur = sqrt(dist2_cur);
    double gap = eta * dFunc / (dist_cur + thickness);
    double toc_prev = toc;
    toc = 0;
    for (its = 0; its < ACCD_MAX_ITERS; ++its) {
        double tocLB = (1 - eta) * dFunc / ((dist_cur + thickness) * maxDispMag);
        ea0 = ea0 + tocLB * dea0; ea1 = ea1 + tocLB * dea1; eb0 = eb0 + tocLB * deb0; eb1 = eb1 + tocLB * deb1;
        ee_eval(ea0, ea1, eb0, eb1, th2, dist2_cur, dFunc);
        dist_cur = sqrt(dist2_cur);
        if (toc != 0 && (dFunc / (dist_cur + thickness) < gap)) return 1;
        toc += tocLB;
        if (toc > toc_prev) return 0;
        if ((its & (ACCD_POLL - 1)) == ACCD_POLL - 1 && accd_beaten(toc, best)) return 0;
    }
    return 2;
}

// flags per instance: bit 0 = an ACCD hit its cap, bit 1 = zero step
__device__ __forceinline__ void accd_one(long k, long npt, const CCand* __restrict__ cand_pt,
                                         const CCand* __restrict__ cand_ee, const int* __restrict__ nodes,
                                         const int* __restrict__ ninst, const int* __restrict__ tris,
                                         const int2* __restrict__ edges, const int* __restrict__ einst,
                                         const double* __restrict__ X, const double* __restrict__ dir,
                                         const double* __restrict__ thick, const double* __restrict__ alpha_cap,
                                         double* __restrict__ alpha_min, int* __restrict__ flags) {
    CCand c = k < npt ? cand_pt[k] : cand_ee[k - npt];
    int inst;
    double toc;
    int r, its = 0;
    if (k < npt) {
        int v = nodes[c.a];
        inst = ninst[c.a];
        int t0 = tris[3 * c.b], t1 = tris[3 * c.b + 1], t2 = tris[3 * c.b + 2];
        toc = alpha_cap[inst];
        r = accd_pt(ld3(X, v), ld3(X, t0), ld3(X, t1), ld3(X, t2), ld3(dir, v), ld3(dir, t0), ld3(dir, t1),
                    ld3(dir, t2), 0.1, thick[inst], toc, its, alpha_min + inst);
        if (toc == 0) atomicOr(flags + inst, 2);
    } else {
        int2 mi = edges[c.a], mj = edges[c.b];
        inst = einst[c.a];
        toc = alpha_cap[inst];
        r = accd_ee(ld3(X, mi.x), ld3(X, mi.y), ld3(X, mj.x), ld3(X, mj.y), ld3(dir, mi.x), ld3(dir, mi.y),
                    ld3(dir, mj.x), ld3(dir, mj.y), 0.1, thick[inst], toc, its, alpha_min + inst);
    }
    if (r == 2) atomicOr(flags + inst, 1);
    if (r != 0) atomic_min_nonneg(alpha_min + inst, toc);
    const unsigned int am = __activemask();
    const unsigned int mx = __reduce_max_sync(am, (unsigned int)its);
    const unsigned int nl = __reduce_add_sync(am, its > 1000 ? 1u : 0u);
    const unsigned int tot = __reduce_add_sync(am, (unsigned int)its);
    if ((threadIdx.x & 31) == __ffs(am) - 1) {
        atomicMax(&g_accd_stats[0], (unsigned long long)mx);
        atomicAdd(&g_accd_stats[1], (unsigned long long)nl);
        atomicAdd(&g_accd_stats[2], (unsigned long long)tot);
        atomicAdd(&g_accd_stats[3], (unsigned long long)__popc(am));
    }
}

constexpr int kAccdBlocks = 4 * 152;

// grid-stride over the candidates; the counts come from the device (clamped
// to the list capacities: an overflowing build is redone by the caller)
__global__ void k_accd(const unsigned int* __restrict__ counts, long cap_pt, long cap_ee,
                       const CCand* __restrict__ cand_pt, const CCand* __restrict__ cand_ee,
                       const int* __restrict__ nodes,
                       const int* __restrict__ ninst, const int* __restrict__ tris, const int2* __restrict__ edges,
                       const int* __restrict__ einst, const double* __restrict__ X, const double* __restrict__ dir,
                       const double* __restrict__ thick, const double* __restrict__ alpha_cap,
                       double* __restrict__ alpha_min, int* __restrict__ flags) {
    const long npt = min((long)counts[0], cap_pt), nee = min((long)counts[1], cap_ee);
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < npt + nee; k += (long)gridDim.x * blockDim.x)
        accd_one(k, npt, cand_pt, cand_ee, nodes, ninst, tris, edges, einst, X, dir, thick, alpha_cap, alpha_min, flags);
}

__global__ void k_alpha_final(int nI, const unsigned char* __restrict__ active, const double* __restrict__ amin,
                              double* __restrict__ alpha) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nI || !active[i]) return;
    alpha[i] = fmin(alpha[i], amin[i]);
}

__global__ void k_fill(int n, double v, double* a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

}  // namespace

int ccd_voxel_size(Arena& A, Work& W, const double* X, cudaStream_t s) {
    const int nI = A.nI;
    const long Se = A.Se > 0 ? A.Se : 1;
    if (W[W_CCD_VOX].ensure(sizeof(double) * (Se + nI + 8))) return IDP_ERR_CUDA;
    double* len = W[W_CCD_VOX].as<double>() + nI;
    if (A.Se) (::idp::count_launch(), k_edge_len<<<grid_for(A.Se), kBlock, 0, s>>>(A.Se, A.sedge, X, len));
    (::idp::count_launch(), k_mean_edge<<<nI, 256, 0, s>>>(nI, A.d_se_off, len, W[W_CCD_VOX].as<double>()));
    return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
}

const double* ccd_voxel_sizes(Arena& A, Work& W) {
    (void)A;
    return W[W_CCD_VOX].as<double>();
}

int ccd_stepsize(Arena& A, Work& W, const double* X, const double* dir, double* alpha, int* flags, cudaStream_t s,
                 const double* voxel_pre) {
    const int nI = A.nI;
    long Se = A.Se > 0 ? A.Se : 1, Sn = A.Sn > 0 ? A.Sn : 1;
    // scratch layout (doubles): len[Se] | absdir[3Sn] | sum scratch | voxel[nI] | amin[nI]
    long nsum = 2 * (A.Se + 3 * A.Sn) / 1024 + 16 * (long)nI + 64;
    if (W[W_CCD_TMP].ensure(sizeof(double) * (Se + 3 * Sn + nsum + 2 * nI + 8))) return IDP_ERR_CUDA;
    double* len = W[W_CCD_TMP].as<double>();
    double* absdir = len + Se;
    double* sumsc = absdir + 3 * Sn;
    double* vsz = sumsc + nsum;
    double* amin = vsz + nI;
    const int* d_se_off = A.d_se_off;
    const int* d_sn_off = A.d_sn_off;
    if (A.Se && !voxel_pre) (::idp::count_launch(), k_edge_len<<<grid_for(A.Se), kBlock, 0, s>>>(A.Se, A.sedge, X, len));
    if (A.Sn) (::idp::count_launch(), k_abs_dir<<<grid_for(A.Sn), kBlock, 0, s>>>(A.Sn, A.snode, dir, absdir));
    if (W[W_SPAN].ensure(sizeof(double) * (A.n_span_tiles + 1))) return IDP_ERR_CUDA;
    double* tsum = W[W_SPAN].as<double>();
    if (A.n_span_tiles > 0)
        (::idp::count_launch(), k_span_tiles<<<A.n_span_tiles, 256, 0, s>>>(A.span_tiles, A.active, absdir, tsum));
    (::idp::count_launch(), k_span_cap<<<nI, 256, 0, s>>>(nI, A.active, d_se_off, d_sn_off, A.span_tile_off, tsum,
                                                          len, absdir, sumsc, alpha, vsz, voxel_pre));
    // grid
    if (W[W_BBOX].ensure(sizeof(unsigned long long) * 6 * nI) || W[W_GRIDP].ensure(sizeof(GridP) * nI))
        return IDP_ERR_CUDA;
    unsigned long long* bb = W[W_BBOX].as<unsigned long long>();
    GridP* gp = W[W_GRIDP].as<GridP>();
    (::idp::count_launch(), k_bb_init<<<grid_for(6 * nI), kBlock, 0, s>>>(nI, bb));
    if (A.Sn) (::idp::count_launch(), k_ccd_bbox<<<grid_for(A.Sn), kBlock, 0, s>>>(A.Sn, A.snode, A.sn_inst, A.active, X, dir, alpha, bb));
    (::idp::count_launch(), k_ccd_grid<<<grid_for(nI), kBlock, 0, s>>>(nI, A.active, bb, A.thickness, vsz, gp));
    long St = A.St > 0 ? A.St : 1;
    if (W[W_BOX_A].ensure(sizeof(BoxI) * 2 * (St + Se + Sn)) || W[W_BOX_B].ensure(sizeof(GridP) * (nI + 1)))
        return IDP_ERR_CUDA;
    BoxI* tbox = W[W_BOX_A].as<BoxI>();
    BoxI* ebox = tbox + St;
    BoxI* nbox = ebox + Se;
    BoxI* tboxc = nbox + Sn;
    BoxI* eboxc = tboxc + St;
    BoxI* nboxc = eboxc + Se;
    GridP* gc = W[W_BOX_B].as<GridP>();
    if (A.Sn)
        (::idp::count_launch(), k_node_box<<<grid_for(A.Sn), kBlock, 0, s>>>(A.Sn, A.snode, A.sn_inst, A.active, X, dir, alpha, A.thickness, gp,
                                                     nbox));
    // triangle / edge boxes from node boxes (v2s: vertex -> surface node)
    if (A.St)
        (::idp::count_launch(), k_prim_box_from_nodes<3><<<grid_for(A.St), kBlock, 0, s>>>(A.St, A.stri, A.v2s, nbox, tbox));
    if (A.Se)
        (::idp::count_launch(), k_prim_box_from_nodes<2><<<grid_for(A.Se), kBlock, 0, s>>>(A.Se, reinterpret_cast<const int*>(A.sedge), A.v2s,
                                                                   nbox, ebox));
    (::idp::count_launch(), k_coarse_grid<<<grid_for(nI), kBlock, 0, s>>>(nI, gp, gc));
    (::idp::count_launch(), k_coarse_boxes<<<grid_for(St + Se + Sn), kBlock, 0, s>>>(
                                St, Se, Sn, A.St, A.Se, A.Sn, A.st_inst, A.se_inst, A.sn_inst, gc, tbox, tboxc));
    // grids, candidates (PT in [0, cap_pt), EE in [cap_pt, cap_pt + cap_ee))
    // and ACCD without a host round trip; one synchronisation at the end reads
    // the candidate counts and the grids' overflow flag (ccount[2]), and only
    // a build that fitted publishes its step sizes
    uint32_t* hp = W.pinned();
    if (!hp) return IDP_ERR_CUDA;
    if (W[W_CAND_CNT].ensure(64)) return IDP_ERR_CUDA;
    unsigned int* ccount = W[W_CAND_CNT].as<unsigned int>();
    long cap_pt = std::max<long>(W.ccd_cap_pt, 4 * A.Sn + 1024);
    long cap_ee = std::max<long>(W.ccd_cap_ee, 4 * A.Se + 1024);
    for (int attempt = 0; attempt < 8; ++attempt) {
        BoxGrid gt, ge;
        IDP_CUDA_TRY(cudaMemsetAsync(ccount, 0, 3 * sizeof(unsigned int), s));
        int rc = grids_build(W, 1, tboxc, A.St, A.st_inst, eboxc, A.Se, A.se_inst, A.active, gc, nI, ccount + 2, gt, ge,
                             s);
        if (rc) return rc;
        if (W[W_CAND].ensure(sizeof(CCand) * (cap_pt + cap_ee))) return IDP_ERR_CUDA;
        CCand* cand = W[W_CAND].as<CCand>();
        if (A.Sn)
            (::idp::count_launch(), k_ccd_query_pt<<<grid_for(kCcdQueryLanes * A.Sn), kBlock, 0, s>>>(A.Sn, A.snode, A.sn_inst, A.active, X, dir, A.dbc_excl, A.stri,
                                                             nbox, tbox, nboxc, tboxc, gc, A.thickness, gt.cells, gt.cell_start,
                                                             gt.entries, cand, ccount, cap_pt));
        if (A.Se)
            (::idp::count_launch(), k_ccd_query_ee<<<grid_for(kCcdQueryLanes * A.Se), kBlock, 0, s>>>(A.Se, A.sedge, A.se_inst, A.active, X, dir, A.dbc_excl, ebox, eboxc, gc,
                                                             A.thickness, ge.cells, ge.cell_start,
                                                             ge.entries, cand + cap_pt, ccount + 1, cap_ee));
        (::idp::count_launch(), k_fill<<<grid_for(nI), kBlock, 0, s>>>(nI, 1e300, amin));
        IDP_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * nI, s));
        (::idp::count_launch(), k_accd<<<kAccdBlocks, 128, 0, s>>>(ccount, cap_pt, cap_ee, cand, cand + cap_pt, A.snode,
                                                                    A.sn_inst, A.stri, A.sedge, A.se_inst, X, dir,
                                                                    A.thickness, alpha, amin, flags));
        IDP_CUDA_TRY(cudaMemcpyAsync(hp + 2, ccount, 3 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        const long npt = hp[2], nee = hp[3];
        if (grids_overflowed(W, 1, hp[4])) continue;
        if (npt > cap_pt || nee > cap_ee) {
            if (npt > cap_pt) cap_pt = npt + npt / 2 + 1024;
            if (nee > cap_ee) cap_ee = nee + nee / 2 + 1024;
            W.ccd_cap_pt = cap_pt;
            W.ccd_cap_ee = cap_ee;
            continue;
        }
        (::idp::count_launch(), k_alpha_final<<<grid_for(nI), kBlock, 0, s>>>(nI, A.active, amin, alpha));
        if (std::getenv("IDP_PROFILE")) {
            unsigned long long st[4] = {0, 0, 0, 0};
            void* sym = nullptr;
            IDP_CUDA_TRY(cudaGetSymbolAddress(&sym, g_accd_stats));
            IDP_CUDA_TRY(cudaMemcpyAsync(st, sym, sizeof(st), cudaMemcpyDeviceToHost, s));
            IDP_CUDA_TRY(cudaMemsetAsync(sym, 0, sizeof(st), s));
            IDP_CUDA_TRY(cudaStreamSynchronize(s));
            W.accd_maxit = std::max<long long>(W.accd_maxit, (long long)st[0]);
            W.accd_long += (long long)st[1];
            W.accd_total += (long long)st[2];
            W.accd_pairs += (long long)st[3];
        }
        return cudaGetLastError() == cudaSuccess ? IDP_OK : IDP_ERR_CUDA;
    }
        return IDP_ERR_CAPACITY;
}

}  // namespace idp
