// Stable LSD radix sort of (key, value) pairs, 8-bit digits.  One pass:
//   count   per tile of 4096 keys, the count of each digit (shared-memory
//           histogram) -> counts[digit][tile];
//   rows    one block per digit: exclusive prefix over the tiles of its row
//           that hold keys (those below the count), the row total ->
//           tot[digit];
//   scatter per tile: the digit's base (prefix of tot) + the tile's row
//           prefix + the key's rank among the tile's equal digits.  Each
//           warp ranks a contiguous run of the tile's keys (rounds of 32, a
//           match_any per round, running per-warp digit counts), then the
//           warps' counts are prefixed per digit; ranks follow key order, so
//           equal digits keep their order.  The tile is staged in shared
//           memory in digit order and each digit's run written contiguously.
#include "radix_sort.h"

#include <algorithm>

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr uint32_t kTile = kThreads * kItems;
constexpr int kWarps = kThreads / 32;

__host__ __device__ inline uint32_t tiles(uint32_t n) { return (n + kTile - 1) / kTile; }

__global__ void __launch_bounds__(kThreads) k_rs_count(const uint32_t *__restrict__ keys, uint32_t n_host,
                                                       const uint32_t *__restrict__ n_dev, int shift,
                                                       uint32_t *__restrict__ counts, uint32_t ntiles) {
    const uint32_t n = n_dev ? *n_dev : n_host;
    if (blockIdx.x * kTile >= n) return;  // a tile past the count: no row scan or scatter reads it
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kTile;
#pragma unroll 4
    for (int k = 0; k < kItems; k++) {
        uint32_t i = base + k * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Block-wide inclusive scan of one value per thread (blockDim.x = 32 * w).
template <int THREADS>
__device__ __forceinline__ uint32_t block_scan_incl(uint32_t v, uint32_t *warp_sums) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= (uint32_t)off) v += u;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < (uint32_t)(THREADS / 32) ? warp_sums[lane] : 0u;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, s, off);
            if (lane >= (uint32_t)off) s += u;
        }
        if (lane < (uint32_t)(THREADS / 32)) warp_sums[lane] = s;
    }
    __syncthreads();
    return warp ? v + warp_sums[warp - 1] : v;
}

// One block per digit: the exclusive prefix of the digit's row over the
// tiles in use (those below the count), in chunks of 1024 consecutive
// entries (coalesced), carrying each chunk's total into the next.
__global__ void __launch_bounds__(1024) k_rs_rows(uint32_t *__restrict__ counts, uint32_t ntiles, uint32_t n_host,
                                                  const uint32_t *__restrict__ n_dev, uint32_t *__restrict__ tot) {
    __shared__ uint32_t ws[32];
    const uint32_t n = n_dev ? *n_dev : n_host;
    const uint32_t used = min(ntiles, tiles(n));
    uint32_t *row = counts + (size_t)blockIdx.x * ntiles;
    uint32_t carry = 0;
    for (uint32_t c0 = 0; c0 < used; c0 += 1024) {
        const uint32_t i = c0 + threadIdx.x;
        const uint32_t v = i < used ? row[i] : 0u;
        const uint32_t incl = block_scan_incl<1024>(v, ws);
        if (i < used) row[i] = carry + incl - v;
        carry += ws[31];  // the scanned warp totals: the last is the chunk's total
        __syncthreads();  // ws is rewritten by the next chunk's scan
    }
    if (threadIdx.x == 0) tot[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kThreads) k_rs_scatter(const uint32_t *__restrict__ keys,
                                                         const uint32_t *__restrict__ vals, uint32_t n_host,
                                                         const uint32_t *__restrict__ n_dev, int shift,
                                                         const uint32_t *__restrict__ counts, uint32_t ntiles,
                                                         const uint32_t *__restrict__ tot, uint32_t *__restrict__ okeys,
                                                         uint32_t *__restrict__ ovals) {
    const uint32_t n = n_dev ? *n_dev : n_host;
    if (blockIdx.x * kTile >= n) return;  // a tile past the device-side count (whole block)
    __shared__ uint32_t cnt[kWarps][256];  // per warp: digit counts, then the warp's offsets in the tile
    __shared__ uint32_t goff[256];         // global position of the tile's first key of each digit
    __shared__ uint32_t tstart[256];       // tile position of the first key of each digit
    __shared__ uint32_t ws[32];
    __shared__ uint32_t skey[kTile], sval[kTile];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (int w = 0; w < kWarps; w++) cnt[w][threadIdx.x] = 0;
    {
        uint32_t t = tot[threadIdx.x];
        uint32_t incl = block_scan_incl<kThreads>(t, ws);  // (its barriers also publish the zeroed counts)
        goff[threadIdx.x] = incl - t + counts[threadIdx.x * ntiles + blockIdx.x];
    }
    // each warp ranks its own contiguous 32 * kItems keys, in order
    const uint32_t tile0 = blockIdx.x * kTile;
    const uint32_t wbase = warp * (32u * kItems);
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t key[kItems], val[kItems], pos[kItems];
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        const uint32_t i = tile0 + wbase + r * 32u + lane;
        const bool valid = i < n;
        key[r] = valid ? keys[i] : 0u;
        val[r] = valid ? vals[i] : 0u;
        pos[r] = 0;
        const uint32_t active = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            const uint32_t d = (key[r] >> shift) & 255u;
            const uint32_t peers = __match_any_sync(active, d);
            const uint32_t before = cnt[warp][d];
            pos[r] = before + __popc(peers & lt);
            __syncwarp(active);
            if ((peers & lt) == 0) cnt[warp][d] = before + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    uint32_t run = 0;
    {  // per digit: exclusive offsets over the warps; run = the tile's count
        const uint32_t dg = threadIdx.x;
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
            uint32_t c = cnt[w][dg];
            cnt[w][dg] = run;
            run += c;
        }
    }
    {
        uint32_t incl = block_scan_incl<kThreads>(run, ws);
        tstart[threadIdx.x] = incl - run;
    }
    __syncthreads();
    // stage the tile in digit order, then write each digit's run contiguously
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        if (tile0 + wbase + r * 32u + lane < n) {
            const uint32_t d = (key[r] >> shift) & 255u;
            const uint32_t lp = tstart[d] + cnt[warp][d] + pos[r];
            skey[lp] = key[r];
            sval[lp] = val[r];
        }
    }
    __syncthreads();
    const uint32_t len = min(kTile, n - tile0);
    for (uint32_t j = threadIdx.x; j < len; j += kThreads) {
        const uint32_t k = skey[j], d = (k >> shift) & 255u;
        const uint32_t dst = goff[d] + (j - tstart[d]);
        okeys[dst] = k;
        ovals[dst] = sval[j];
    }
}

}  // namespace

size_t radix_sort_scratch_words(uint32_t n) { return 256 * (size_t)std::max(1u, tiles(n)) + 256; }

cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2, uint32_t *scratch,
                             uint32_t n, int bits, uint32_t **out_keys, uint32_t **out_vals, cudaStream_t st) {
    uint32_t *ka = keys, *va = vals, *kb = keys2, *vb = vals2;
    if (n > 1) {
        const uint32_t nt = tiles(n);
        uint32_t *counts = scratch, *tot = scratch + 256 * (size_t)nt;
        for (int shift = 0; shift < bits; shift += 8) {
            k_rs_count<<<nt, kThreads, 0, st>>>(ka, n, nullptr, shift, counts, nt);
            k_rs_rows<<<256, 1024, 0, st>>>(counts, nt, n, nullptr, tot);
            k_rs_scatter<<<nt, kThreads, 0, st>>>(ka, va, n, nullptr, shift, counts, nt, tot, kb, vb);
            std::swap(ka, kb);
            std::swap(va, vb);
        }
    }
    *out_keys = ka;
    *out_vals = va;
    return cudaGetLastError();
}

cudaError_t radix_sort_pairs_dev(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2, uint32_t *scratch,
                                 const uint32_t *d_n, uint32_t max_n, int bits, cudaStream_t st) {
    if (max_n == 0) return cudaSuccess;
    uint32_t *ka = keys, *va = vals, *kb = keys2, *vb = vals2;
    const uint32_t nt = tiles(max_n);
    uint32_t *counts = scratch, *tot = scratch + 256 * (size_t)nt;
    for (int shift = 0; shift < bits; shift += 8) {
        k_rs_count<<<nt, kThreads, 0, st>>>(ka, 0, d_n, shift, counts, nt);
        k_rs_rows<<<256, 1024, 0, st>>>(counts, nt, 0, d_n, tot);
        k_rs_scatter<<<nt, kThreads, 0, st>>>(ka, va, 0, d_n, shift, counts, nt, tot, kb, vb);
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    return cudaGetLastError();
}
