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

// Two-point sort key of a ray: 6-D Morton code of the ray's origin and of
// the point at distance len along its unit direction, p bits per coordinate
// over the box (lo, 1 / extent) (bit b of coordinate k at bit 6b + k).
__device__ __forceinline__ uint32_t tp_cell(float v, float lo, float inv, float cells) {
    float c = (v - lo) * inv * cells;
    c = fminf(fmaxf(c, 0.0f), cells - 1.0f);  // NaN -> 0
    return (uint32_t)c;
}
__device__ __forceinline__ uint32_t two_point_key(float ox, float oy, float oz, float dx, float dy, float dz, float4 lo,
                                                  float4 inv, float len, int p) {
    const float cells = (float)(1u << p);
    float l2 = dx * dx + dy * dy + dz * dz;
    float s = l2 > 0.0f ? len / sqrtf(l2) : 0.0f;
    uint32_t c[6] = {tp_cell(ox, lo.x, inv.x, cells), tp_cell(oy, lo.y, inv.y, cells), tp_cell(oz, lo.z, inv.z, cells),
                     tp_cell(ox + dx * s, lo.x, inv.x, cells), tp_cell(oy + dy * s, lo.y, inv.y, cells),
                     tp_cell(oz + dz * s, lo.z, inv.z, cells)};
    uint32_t key = 0;
    for (int b = 0; b < p; b++)
#pragma unroll
        for (int k = 0; k < 6; k++) key |= ((c[k] >> b) & 1u) << (6 * b + k);
    return key;
}
