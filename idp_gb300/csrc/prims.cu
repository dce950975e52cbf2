// Radix sort, scan and fixed-order sum kernels (see prims.cuh).
#include "prims.cuh"

namespace idp {

namespace {
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void rs_histogram(const uint64_t* __restrict__ keys, long n, int shift, uint32_t* __restrict__ counts,
                             int ntiles) {
    __shared__ uint32_t h[256];
    int t = threadIdx.x;
    h[t] = 0;
    __syncthreads();
    long base = (long)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; ++r) {
        long i = base + r * RS_THREADS + t;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[(long)t * ntiles + blockIdx.x] = h[t];
}

__global__ void rs_scatter(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, long n, int shift,
                           const uint32_t* __restrict__ offsets, int ntiles, uint64_t* __restrict__ okeys,
                           uint32_t* __restrict__ ovals) {
    __shared__ uint32_t wc[RS_WARPS][256];
    __shared__ uint32_t running[256];
    __shared__ uint32_t gbase[256];
    int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    running[t] = 0;
    gbase[t] = offsets[(long)t * ntiles + blockIdx.x];
    for (int w = 0; w < RS_WARPS; ++w) wc[w][t] = 0;
    __syncthreads();
    long base = (long)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; ++r) {
        long i = base + r * RS_THREADS + t;
        bool valid = i < n;
        uint64_t k = valid ? keys[i] : 0;
        uint32_t v = valid ? vals[i] : 0;
        uint32_t d = valid ? (uint32_t)((k >> shift) & 255u) : (256u + lane);
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t lt = (1u << lane) - 1u;
        uint32_t rank_w = __popc(peers & lt);
        if (valid && (peers & lt) == 0) wc[warp][d] = __popc(peers);
        __syncthreads();
        // exclusive prefix over warps for digit t, in place
        {
            uint32_t run = 0;
            for (int w = 0; w < RS_WARPS; ++w) {
                uint32_t c = wc[w][t];
                wc[w][t] = run;
                run += c;
            }
            // this pass's total stays in a register (the prefix overwrote the slots)
            __syncthreads();
            if (valid) {
                uint32_t pos = gbase[d] + running[d] + wc[warp][d] + rank_w;
                okeys[pos] = k;
                ovals[pos] = v;
            }
            __syncthreads();
            running[t] += run;
            for (int w = 0; w < RS_WARPS; ++w) wc[w][t] = 0;
            __syncthreads();
        }
    }
}

// ---- scan
constexpr int SC_THREADS = 256;
constexpr int SC_ITEMS = 8;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t ws[SC_THREADS / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < SC_THREADS / 32) ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SC_THREADS / 32) ws[lane] = w;
    }
    __syncthreads();
    uint32_t prefix = (warp > 0 ? ws[warp - 1] : 0) + x - v;
    if (total) *total = ws[SC_THREADS / 32 - 1];
    __syncthreads();
    return prefix;
}

__global__ void scan_tile_sums(const uint32_t* __restrict__ in, long n, uint32_t* __restrict__ sums) {
    long base = (long)blockIdx.x * SC_TILE + (long)threadIdx.x * SC_ITEMS;
    uint32_t s = 0;
    for (int k = 0; k < SC_ITEMS; ++k)
        if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan_tiles(const uint32_t* in, uint32_t* out, long n, const uint32_t* __restrict__ tile_off,
                           uint32_t* total) {
    long base = (long)blockIdx.x * SC_TILE + (long)threadIdx.x * SC_ITEMS;
    uint32_t loc[SC_ITEMS];
    uint32_t s = 0;
    for (int k = 0; k < SC_ITEMS; ++k) {
        loc[k] = (base + k < n) ? in[base + k] : 0;
        s += loc[k];
    }
    uint32_t tot;
    uint32_t pre = block_excl_scan(s, &tot);
    uint32_t off = (tile_off ? tile_off[blockIdx.x] : 0) + pre;
    for (int k = 0; k < SC_ITEMS; ++k) {
        if (base + k < n) out[base + k] = off;
        off += loc[k];
    }
    if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == SC_THREADS - 1) *total = off;
}

// ---- fixed-order double sum
constexpr int DS_THREADS = 256;
constexpr int DS_ITEMS = 8;
constexpr int DS_TILE = DS_THREADS * DS_ITEMS;

__global__ void det_sum_tiles(const double* __restrict__ x, long n, double* __restrict__ out) {
    __shared__ double a[DS_THREADS];
    long base = (long)blockIdx.x * DS_TILE;
    double s = 0.0;
    for (int k = 0; k < DS_ITEMS; ++k) {
        long i = base + k * DS_THREADS + threadIdx.x;
        if (i < n) s += x[i];
    }
    a[threadIdx.x] = s;
    __syncthreads();
    for (int st = DS_THREADS / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) a[threadIdx.x] += a[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = a[0];
}
}  // namespace

int bits_for(uint64_t m) {
    int b = 0;
    while (b < 64 && (m >> b) != 0) ++b;
    return b < 1 ? 1 : b;
}

size_t radix_sort_scratch_bytes(long n) {
    long tiles = (n + RS_TILE - 1) / RS_TILE;
    if (tiles < 1) tiles = 1;
    return 256 * tiles * sizeof(uint32_t) + scan_scratch_bytes(256 * tiles) + 256;
}

size_t scan_scratch_bytes(long n) {
    // level sizes: n/2048, n/2048^2, ... each level needs sums + offsets
    size_t bytes = 0;
    long m = n;
    while (m > SC_TILE) {
        long t = (m + SC_TILE - 1) / SC_TILE;
        bytes += 2 * ((t + 63) / 64 * 64) * sizeof(uint32_t);
        m = t;
    }
    return bytes + 256;
}

cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, long n, uint32_t* total, void* scratch,
                           cudaStream_t s) {
    if (n <= 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
        return cudaSuccess;
    }
    long tiles = (n + SC_TILE - 1) / SC_TILE;
    if (tiles == 1) {
        (::idp::count_launch(), scan_tiles<<<1, SC_THREADS, 0, s>>>(in, out, n, nullptr, total));
        return cudaGetLastError();
    }
    uint32_t* sums = reinterpret_cast<uint32_t*>(scratch);
    long padded = (tiles + 63) / 64 * 64;
    uint32_t* offs = sums + padded;
    void* rest = offs + padded;
    (::idp::count_launch(), scan_tile_sums<<<(int)tiles, SC_THREADS, 0, s>>>(in, n, sums));
    cudaError_t e = scan_exclusive(sums, offs, tiles, nullptr, rest, s);
    if (e != cudaSuccess) return e;
    (::idp::count_launch(), scan_tiles<<<(int)tiles, SC_THREADS, 0, s>>>(in, out, n, offs, total));
    return cudaGetLastError();
}

cudaError_t radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, long n,
                             int bits, void* scratch, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    long tiles = (n + RS_TILE - 1) / RS_TILE;
    uint32_t* counts = reinterpret_cast<uint32_t*>(scratch);
    void* scan_scratch = counts + 256 * tiles;
    uint64_t* kin = keys;
    uint32_t* vin = vals;
    uint64_t* kout = keys_alt;
    uint32_t* vout = vals_alt;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        (::idp::count_launch(), rs_histogram<<<(int)tiles, RS_THREADS, 0, s>>>(kin, n, shift, counts, (int)tiles));
        cudaError_t e = scan_exclusive(counts, counts, 256 * tiles, nullptr, scan_scratch, s);
        if (e != cudaSuccess) return e;
        (::idp::count_launch(), rs_scatter<<<(int)tiles, RS_THREADS, 0, s>>>(kin, vin, n, shift, counts, (int)tiles, kout, vout));
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    if (kin != keys) {
        cudaMemcpyAsync(keys, kin, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    }
    return cudaGetLastError();
}

cudaError_t det_sum(const double* x, long n, double* result, double* scratch, cudaStream_t s) {
    if (n <= 0) return cudaMemsetAsync(result, 0, sizeof(double), s);
    const double* in = x;
    long m = n;
    double* buf[2] = {scratch, scratch + (n / DS_TILE + 2)};
    int which = 0;
    while (true) {
        long tiles = (m + DS_TILE - 1) / DS_TILE;
        double* out = (tiles == 1) ? result : buf[which];
        (::idp::count_launch(), det_sum_tiles<<<(int)tiles, DS_THREADS, 0, s>>>(in, m, out));
        if (tiles == 1) break;
        in = out;
        m = tiles;
        which ^= 1;
    }
    return cudaGetLastError();
}

}  // namespace idp
