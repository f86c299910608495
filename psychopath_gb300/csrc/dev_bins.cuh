// Counting-sort helpers shared by the ray binning of trace calls
// (trace_kernels.cu) and of the render wavefront's queues (kernels.cu).
#pragma once

#include <cstdint>

// Warp-aggregated increment of counters[key]: one atomic per distinct key
// in the warp.  Returns this lane's slot (old value + rank among equal keys).
__device__ __forceinline__ uint32_t warp_add_key(uint32_t *counters, uint32_t key, uint32_t active) {
    uint32_t same = __match_any_sync(active, key);
    uint32_t lane = threadIdx.x & 31u;
    uint32_t leader = __ffs(same) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counters + key, (uint32_t)__popc(same));
    base = __shfl_sync(same, base, leader);
    return base + __popc(same & ((1u << lane) - 1u));
}
// Exclusive prefix sum of nbins (a power of two, <= 2^20) bin counts in
// place (one block of 1024 threads).
static __global__ void __launch_bounds__(1024) k_scan_bins(uint32_t *hist, uint32_t nbins) {
    __shared__ uint32_t part[1024];
    uint32_t per = (nbins + 1023) / 1024, t = threadIdx.x;
    uint32_t sum = 0;
    for (uint32_t k = 0; k < per; k++)
        if (t * per + k < nbins) sum += hist[t * per + k];
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {
        uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
    for (uint32_t k = 0; k < per; k++) {
        if (t * per + k >= nbins) break;
        uint32_t c = hist[t * per + k];
        hist[t * per + k] = run;
        run += c;
    }
}
