// Device primitives written for this engine: LSD radix sort of (u64 key,
// u32 value) pairs, exclusive scan of u32 counts, and a fixed-order double
// sum. All three are deterministic: their results do not depend on thread
// scheduling.
#pragma once
#include "common.cuh"

namespace idp {

// Scratch bytes needed by radix_sort_pairs / scan_exclusive for n items.
size_t radix_sort_scratch_bytes(long n);
size_t scan_scratch_bytes(long n);

// Stable LSD sort of keys[0..n) (only the low `bits` bits are significant)
// with values carried along. keys/vals are sorted in place; keys_alt/vals_alt
// are ping-pong buffers of the same size. scratch must hold
// radix_sort_scratch_bytes(n).
cudaError_t radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, long n,
                             int bits, void* scratch, cudaStream_t s);

// out[i] = sum_{j<i} in[j]; if total != nullptr, *total (device) = sum of all.
// in and out may alias.
cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, long n, uint32_t* total, void* scratch,
                           cudaStream_t s);

// Fixed-order sum of x[0..n) into *result (device): 2048-item tiles, thread t
// sums items t, t+256, ... of its tile in order, then a shared-memory tree
// (stride 128, 64, ..., 1); tile sums are reduced the same way until one
// value remains. scratch needs 16 * (n / 2048 + 2) bytes.
cudaError_t det_sum(const double* x, long n, double* result, double* scratch, cudaStream_t s);

int bits_for(uint64_t maxval);

}  // namespace idp
