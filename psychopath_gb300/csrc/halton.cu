// Halton sample generation on the GPU: halton::sample(index, dimension) of
// sub_crates/halton (Gruenschloss' Halton points with Faure permutations,
// generated by sub_crates/halton/build.rs), bit-exact.
//
// Host side, once per device: the first 128 primes, the Faure permutations
// of 0..b-1 (build.rs get_faure_permutation, :237-273), and per dimension
// i >= 1 with base b = primes[i] a table of b^d 16-bit entries -- the
// Faure-permuted radical inverse of d base-b digits (invert, :275-284) for
// the most digits d with b^d <= 500 (:133-139) -- plus the number K of
// digit groups, (b^d)^K being the largest power of b^d below 2^32
// (:140-146), and the f32 scale 0.999999940395355224609375 / (b^d)^K.
// Device side: dimension 0 is the base-2 radical inverse by bit reversal
// times 2^-32 (:108-123); dimension i sums table[(index / (b^d)^k) % b^d] *
// (b^d)^(K-1-k) over k < K in u32 and scales the f32 of the sum (:176-216).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/psy_gpu.h"

int psy_fail(int code, const std::string &msg);  // capi.cu: sets psy_last_error

namespace {

constexpr int kHaltonDims = 128;

struct HaltonDim {
    uint32_t pow_base, groups, max_power, perm_offset;
    float scale;
    uint32_t pad[3];
};

__device__ HaltonDim g_halton_dims[kHaltonDims];
__device__ uint16_t *g_halton_perm;  // concatenated permutation tables

__global__ void k_halton(uint32_t dimension, const uint32_t *__restrict__ idx, uint32_t n, float *__restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t x = idx[i];
    if (dimension == 0) {
        x = __brev(x);  // the reference's five swap steps reverse all 32 bits
        out[i] = __uint2float_rn(x) * (1.0f / 4294967296.0f);
        return;
    }
    const HaltonDim d = g_halton_dims[dimension];
    const uint16_t *perm = g_halton_perm + d.perm_offset;
    uint32_t sum = 0, w = d.max_power / d.pow_base;
    for (uint32_t k = 0; k < d.groups; k++) {
        sum += (uint32_t)perm[x % d.pow_base] * w;
        x /= d.pow_base;
        w /= d.pow_base;
    }
    out[i] = __fmul_rn(__uint2float_rn(sum), d.scale);
}

struct HostTables {
    std::vector<HaltonDim> dims;
    std::vector<uint16_t> perm;
    HostTables() {
        std::vector<uint32_t> primes;
        for (uint32_t c = 2; (int)primes.size() < kHaltonDims; c++) {
            bool prime = true;
            for (uint32_t q = 2; q * q <= c; q++)
                if (c % q == 0) { prime = false; break; }
            if (prime) primes.push_back(c);
        }
        // Faure permutations: odd b inserts the middle digit into b-1's
        // permutation, even b interleaves two copies of b/2's
        std::vector<std::vector<uint32_t>> faure(primes.back() + 1);
        for (uint32_t b = 0; b <= primes.back(); b++) {
            std::vector<uint32_t> &p = faure[b];
            if (b < 2) { p = {0}; continue; }
            if (b == 2) { p = {0, 1}; continue; }
            p.resize(b);
            if (b % 2 == 1) {
                uint32_t c = (b - 1) / 2;
                for (uint32_t i = 0; i < b; i++) {
                    if (i == c) { p[i] = c; continue; }
                    uint32_t f = faure[b - 1][i > c ? i - 1 : i];
                    p[i] = f >= c ? f + 1 : f;
                }
            } else {
                uint32_t c = b / 2;
                for (uint32_t i = 0; i < b; i++) p[i] = i < c ? 2 * faure[c][i] : 2 * faure[c][i - c] + 1;
            }
        }
        dims.assign(kHaltonDims, HaltonDim{});
        for (int i = 1; i < kHaltonDims; i++) {
            const uint64_t b = primes[i];
            uint64_t pb = b;
            uint32_t digits = 1;
            for (; pb * b <= 500; digits++) pb *= b;
            uint64_t mp = pb;
            uint32_t groups = 1;
            for (; mp * pb < (1ull << 32); groups++) mp *= pb;
            HaltonDim &d = dims[i];
            d.pow_base = (uint32_t)pb;
            d.groups = groups;
            d.max_power = (uint32_t)mp;
            d.perm_offset = (uint32_t)perm.size();
            d.scale = 0.999999940395355224609375f / (float)(uint32_t)mp;
            for (uint64_t j = 0; j < pb; j++) {
                uint64_t rest = j, r = 0;
                for (uint32_t k = 0; k < digits; k++) {
                    r = r * b + faure[b][rest % b];
                    rest /= b;
                }
                perm.push_back((uint16_t)r);
            }
        }
    }
};

std::mutex g_halton_mu;
void *g_halton_dev_perm[64] = {nullptr};  // per device: the uploaded tables

int ensure_tables(cudaStream_t st) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return psy_fail(PSY_E_CUDA, "no CUDA device");
    std::lock_guard<std::mutex> lk(g_halton_mu);
    if (g_halton_dev_perm[dev]) return PSY_OK;
    static const HostTables t;
    void *p = nullptr;
    size_t bytes = t.perm.size() * sizeof(uint16_t);
    if (cudaMalloc(&p, bytes) != cudaSuccess) return psy_fail(PSY_E_NOMEM, "halton tables: cudaMalloc failed");
    uint16_t *pp = static_cast<uint16_t *>(p);
    if (cudaMemcpyAsync(p, t.perm.data(), bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyToSymbolAsync(g_halton_perm, &pp, sizeof(pp), 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyToSymbolAsync(g_halton_dims, t.dims.data(), sizeof(HaltonDim) * kHaltonDims, 0,
                                cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaFree(p);
        return psy_fail(PSY_E_CUDA, "halton tables: upload failed");
    }
    g_halton_dev_perm[dev] = p;
    return PSY_OK;
}

}  // namespace

// psy_halton_samples (include/psy_gpu.h).
extern "C" int psy_halton_samples(uint32_t dimension, const uint32_t *d_indices, uint32_t n, float *d_out,
                                  void *stream) {
    if (dimension >= (uint32_t)kHaltonDims) return psy_fail(PSY_E_INVALID, "halton: dimension must be below 128");
    if (n == 0) return PSY_OK;
    if (!d_indices || !d_out) return psy_fail(PSY_E_INVALID, "halton: null buffer");
    cudaStream_t st = (cudaStream_t)stream;
    int r = ensure_tables(st);
    if (r != PSY_OK) return r;
    k_halton<<<(n + 255) / 256, 256, 0, st>>>(dimension, d_indices, n, d_out);
    if (cudaGetLastError() != cudaSuccess) return psy_fail(PSY_E_CUDA, "halton: launch failed");
    return PSY_OK;
}
