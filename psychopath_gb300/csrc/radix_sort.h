// Stable LSD radix sort of (uint32 key, uint32 value) pairs on the device
// (radix_sort.cu): the ray order of trace calls and the Morton order of the
// GPU BVH build.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

// Scratch words the sort needs for n pairs (digit histograms per tile plus
// the digit totals), besides the second key / value buffers.
size_t radix_sort_scratch_words(uint32_t n);

// Sorts the low `bits` bits of keys[0..n) (values move with their keys;
// equal keys keep their order).  8-bit digits, ceil(bits / 8) passes that
// alternate between (keys, vals) and (keys2, vals2); *out_keys / *out_vals
// receive the buffers that hold the result.  scratch: radix_sort_scratch_words(n).
cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2, uint32_t *scratch,
                             uint32_t n, int bits, uint32_t **out_keys, uint32_t **out_vals, cudaStream_t st);

// The same with the pair count read from device memory (*d_n <= max_n) by
// the kernels, so the launch sequence does not depend on it (CUDA graphs,
// no host synchronisation).  Passes = ceil(bits / 8); the result is in
// (keys, vals) after an even number of passes, else in (keys2, vals2).
cudaError_t radix_sort_pairs_dev(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2, uint32_t *scratch,
                                 const uint32_t *d_n, uint32_t max_n, int bits, cudaStream_t st);
