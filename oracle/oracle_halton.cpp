// Oracle (test infrastructure only): halton::sample restated from the
// generator of sub_crates/halton/build.rs (Gruenschloss' Halton points with
// Faure permutations).  Used by tests/ as the checker of the GPU library's
// psy_halton_samples; the product never links it.
//
// build.rs (:35-47) takes the first 128 primes; dimension 0 is the base-2
// radical inverse by bit reversal (:108-123); dimension i >= 1 uses base
// b = primes[i] with a permutation table of b^d entries (d = the most digits
// with b^d <= 500, :133-139) holding the Faure-permuted radical inverse of d
// digits (:148-151, invert :275-284, get_faure_permutation :237-273), applied
// to the index's base-b^d digit groups with weights (b^d)^(K-1) ... 1, where
// (b^d)^K is the largest power below 2^32 (:140-146, :176-216); the sum is
// converted to f32 and scaled by 0.999999940395355224609375 / (b^d)^K, both
// in f32 (:205-208).
#include <stdint.h>

#include <vector>

namespace {

struct HaltonTables {
    struct Dim {
        uint32_t pow_base, groups, max_power;
        float scale;
        std::vector<uint16_t> perm;
    };
    std::vector<Dim> dims;  // index 0 unused (bit reversal)

    HaltonTables() {
        const int kDims = 128;
        std::vector<uint32_t> primes;
        for (uint32_t c = 2; (int)primes.size() < kDims; c++) {
            bool p = true;
            for (uint32_t i = 2; i < c; i++)
                if (c % i == 0) { p = false; break; }
            if (p) primes.push_back(c);
        }
        // Faure permutations of 0..b-1 for b = 0 .. largest prime
        std::vector<std::vector<uint32_t>> faure;
        for (uint32_t b = 0; b <= primes.back(); b++) {
            std::vector<uint32_t> perm;
            if (b < 2) {
                perm = {0};
            } else if (b == 2) {
                perm = {0, 1};
            } else if (b & 1u) {
                uint32_t c = (b - 1) / 2;
                for (uint32_t i = 0; i < b; i++) {
                    if (i == c) { perm.push_back(c); continue; }
                    uint32_t f = faure[b - 1][i - (i > c ? 1u : 0u)];
                    perm.push_back(f + (f >= c ? 1u : 0u));
                }
            } else {
                uint32_t c = b / 2;
                for (uint32_t i = 0; i < b; i++)
                    perm.push_back(i < c ? 2 * faure[c][i] : 2 * faure[c][i - c] + 1);
            }
            faure.push_back(perm);
        }
        dims.resize(kDims);
        for (int i = 1; i < kDims; i++) {
            uint64_t base = primes[i], pow_base = base;
            uint32_t digits = 1;
            while (pow_base * base <= 500) { pow_base *= base; digits++; }
            uint64_t max_power = pow_base;
            uint32_t groups = 1;
            while (max_power * pow_base < (1ull << 32)) { max_power *= pow_base; groups++; }
            Dim &d = dims[i];
            d.pow_base = (uint32_t)pow_base;
            d.groups = groups;
            d.max_power = (uint32_t)max_power;
            d.scale = 0.999999940395355224609375f / (float)(uint32_t)max_power;
            for (uint64_t j = 0; j < pow_base; j++) {
                uint64_t idx = j, r = 0;
                for (uint32_t k = 0; k < digits; k++) {
                    uint64_t rem = idx % base;
                    idx /= base;
                    r = r * base + faure[base][rem];
                }
                d.perm.push_back((uint16_t)r);
            }
        }
    }
};

const HaltonTables &tables() {
    static HaltonTables t;
    return t;
}

}  // namespace

extern "C" int psyo_halton_sample(uint32_t index, uint32_t dimension, float *out) {
    if (dimension >= 128) return -1;
    if (dimension == 0) {
        uint32_t x = index;
        x = (x << 16) | (x >> 16);
        x = ((x & 0x00ff00ffu) << 8) | ((x & 0xff00ff00u) >> 8);
        x = ((x & 0x0f0f0f0fu) << 4) | ((x & 0xf0f0f0f0u) >> 4);
        x = ((x & 0x33333333u) << 2) | ((x & 0xccccccccu) >> 2);
        x = ((x & 0x55555555u) << 1) | ((x & 0xaaaaaaaau) >> 1);
        *out = (float)x * (1.0f / 4294967296.0f);
        return 0;
    }
    const HaltonTables::Dim &d = tables().dims[dimension];
    // digit groups of the index, lowest first, weighted (b^d)^(K-1) .. 1
    uint32_t sum = 0, w = d.max_power / d.pow_base, rest = index;
    for (uint32_t k = 0; k < d.groups; k++) {
        sum += (uint32_t)d.perm[rest % d.pow_base] * w;
        rest /= d.pow_base;
        w /= d.pow_base;
    }
    *out = (float)sum * d.scale;
    return 0;
}
