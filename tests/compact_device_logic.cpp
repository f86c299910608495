// Host build of the GPU codecs' device functions (psychopath_gb300/csrc/
// dev_compact.cuh) against the oracle: the fast paths' decision rules --
// fluv32's chroma from an approximate reciprocal, encode_precise's f32
// sin^2 ranking with f64 cosines on near ties, the 40/48-bit codes built
// in 32-bit halves -- are checked on the CPU without a GPU.  __fdividef is
// replaced by the correctly rounded quotient moved by a random 0-2 ulps
// either way (its documented error bound), so the margins are exercised
// adversarially.  Exit status 0 iff every code equals the oracle's.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#define __device__
#define __forceinline__ inline
#define __noinline__
struct float2 {
    float x, y;
};
struct float3 {
    float x, y, z;
};
static inline float2 make_float2(float a, float b) { return {a, b}; }
static inline float3 make_float3(float a, float b, float c) { return {a, b, c}; }
static inline float __uint_as_float(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static inline uint32_t __float_as_uint(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static std::mt19937_64 g_rng(20240605);
static inline float __fdividef(float a, float b) {
    float q = (float)((double)a / (double)b);
    for (int k = (int)(g_rng() % 5) - 2; k != 0; k += (k > 0 ? -1 : 1)) q = std::nextafter(q, k > 0 ? INFINITY : -INFINITY);
    return q;
}
using std::isinf;
using std::isnan;
using std::max;
using std::min;
#include "../include/psy_gpu.h"
#include "../psychopath_gb300/csrc/dev_compact.cuh"

extern "C" int psyo_compact_encode(uint32_t format, const float *xyz, uint32_t n, uint8_t *out, uint32_t *invalid);
extern "C" int psyo_compact_decode(uint32_t format, const uint8_t *in, uint32_t n, float *xyz);

static const float kSpecial[] = {0.0f, -0.0f, INFINITY, -INFINITY, NAN, 1e-45f, -1e-45f, 1.1754942e-38f,
                                 3.4028235e38f, -3.4028235e38f, 2.0e38f, 1e28f, 65504.0f, 0.5f};

static std::vector<float> triples(uint32_t n, bool positive) {
    std::uniform_real_distribution<double> e70(-70, 70), wide(-150, 127), u(-1, 1), u01(0, 1);
    std::vector<float> v(3 * (size_t)n);
    for (uint32_t i = 0; i < n; i++) {
        const int mode = i % 4;
        const double scale = std::exp2(wide(g_rng));
        for (int c = 0; c < 3; c++) {
            double m = mode == 0 ? std::exp2(e70(g_rng)) * (u(g_rng) < 0 ? -1 : 1)
                       : mode == 1 ? u(g_rng) * scale
                       : mode == 2 ? std::floor(u01(g_rng) * 64) * scale
                                   : u(g_rng);
            if (g_rng() % 32 == 0) m = kSpecial[g_rng() % (sizeof(kSpecial) / sizeof(float))];
            v[3 * (size_t)i + c] = positive ? std::fabs((float)m) : (float)m;
        }
    }
    return v;
}

// directions half-way between neighbouring oct32 grid points, at grid points
// and at cell centres, at three magnitudes: candidates within rounding
static std::vector<float> near_ties(uint32_t n) {
    std::vector<uint32_t> codes(4 * (size_t)n);
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t c = (uint32_t)g_rng();
        codes[4 * i] = c;
        codes[4 * i + 1] = (c & 0xffff0000u) | ((c + 1) & 0xffffu);
        codes[4 * i + 2] = c + 0x10000u;
        codes[4 * i + 3] = c + 0x10001u;
    }
    std::vector<float> d(12 * (size_t)n);
    psyo_compact_decode(PSY_COMPACT_OCT32, reinterpret_cast<const uint8_t *>(codes.data()), 4 * n, d.data());
    std::vector<float> v;
    v.reserve(3 * (size_t)n);
    const float scale[3] = {1.0f, 1e-20f, 3e25f};
    for (uint32_t i = 0; i < n; i++) {
        const float *a = &d[12 * (size_t)i];
        const int m = i % 5;
        for (int c = 0; c < 3; c++) {
            float o = m == 0   ? a[c]
                      : m < 4  ? (a[c] + a[3 * m + c]) * 0.5f
                               : (a[c] + a[3 + c] + a[6 + c] + a[9 + c]) * 0.25f;
            v.push_back(o * scale[i % 3]);
        }
    }
    return v;
}

template <class Fn>
static uint64_t check(const char *name, uint32_t format, int size, const std::vector<float> &v, Fn device) {
    const uint32_t n = (uint32_t)(v.size() / 3);
    std::vector<uint8_t> want((size_t)n * size);
    psyo_compact_encode(format, v.data(), n, want.data(), nullptr);
    uint64_t bad = 0;
    for (uint32_t i = 0; i < n; i++) {
        const uint64_t got = device(v[3 * (size_t)i], v[3 * (size_t)i + 1], v[3 * (size_t)i + 2]);
        uint64_t w = 0;
        for (int k = 0; k < size; k++) w |= (uint64_t)want[(size_t)i * size + k] << (8 * k);
        if (got != w) {
            if (bad < 5)
                printf("%s mismatch at %u: (%g, %g, %g) device %llx oracle %llx\n", name, i, v[3 * (size_t)i],
                       v[3 * (size_t)i + 1], v[3 * (size_t)i + 2], (unsigned long long)got, (unsigned long long)w);
            bad++;
        }
    }
    printf("%s: %u checked, %llu mismatches\n", name, n, (unsigned long long)bad);
    return bad;
}

// decoders on random codes: equal bits, any NaN matching any NaN
template <class Fn>
static uint64_t check_decode(const char *name, uint32_t format, int size, uint32_t n, Fn device) {
    std::vector<uint8_t> codes((size_t)n * size);
    for (auto &b : codes) b = (uint8_t)g_rng();
    std::vector<float> want(3 * (size_t)n);
    psyo_compact_decode(format, codes.data(), n, want.data());
    uint64_t bad = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint64_t c = 0;
        for (int k = 0; k < size; k++) c |= (uint64_t)codes[(size_t)i * size + k] << (8 * k);
        const float3 g = device(c);
        const float got[3] = {g.x, g.y, g.z};
        for (int k = 0; k < 3; k++) {
            const float w = want[3 * (size_t)i + k];
            if (!(std::isnan(got[k]) && std::isnan(w)) && __float_as_uint(got[k]) != __float_as_uint(w)) {
                if (bad < 5) printf("%s mismatch at %u: code %llx\n", name, i, (unsigned long long)c);
                bad++;
                break;
            }
        }
    }
    printf("%s: %u checked, %llu mismatches\n", name, n, (unsigned long long)bad);
    return bad;
}

int main(int argc, char **argv) {
    const uint32_t n = argc > 1 ? (uint32_t)atoi(argv[1]) : 1000000;
    uint64_t bad = 0;
    const std::vector<float> pos = triples(n, true), sgn = triples(n, false), ties = near_ties(n / 2);
    bad += check("fluv32", PSY_COMPACT_FLUV32, 4, pos,
                 [](float x, float y, float z) { return (uint64_t)psyc::fluv32_encode(x, y, z); });
    bad += check("fluv32 signed", PSY_COMPACT_FLUV32, 4, sgn,
                 [](float x, float y, float z) { return (uint64_t)psyc::fluv32_encode(x, y, z); });
    bad += check("oct32", PSY_COMPACT_OCT32, 4, sgn,
                 [](float x, float y, float z) { return (uint64_t)psyc::oct32_encode(x, y, z); });
    for (const std::vector<float> *v : {&sgn, &ties})
        bad += check("oct32 encode_precise", PSY_COMPACT_OCT32_PRECISE, 4, *v,
                     [](float x, float y, float z) { return (uint64_t)psyc::oct32_encode_precise(x, y, z); });
    bad += check("unsigned32", PSY_COMPACT_UNSIGNED32, 4, sgn,
                 [](float x, float y, float z) { return (uint64_t)psyc::unsigned32_encode(x, y, z); });
    bad += check("unsigned40", PSY_COMPACT_UNSIGNED40, 5, sgn,
                 [](float x, float y, float z) { return psyc::unsigned40_encode(x, y, z); });
    bad += check("signed48", PSY_COMPACT_SIGNED48, 6, sgn,
                 [](float x, float y, float z) { return psyc::signed48_encode(x, y, z); });
    bad += check_decode("fluv32 decode", PSY_COMPACT_FLUV32, 4, n,
                        [](uint64_t c) { return psyc::fluv32_decode((uint32_t)c); });
    bad += check_decode("oct32 decode", PSY_COMPACT_OCT32, 4, n, [](uint64_t c) { return psyc::oct32_decode((uint32_t)c); });
    bad += check_decode("unsigned32 decode", PSY_COMPACT_UNSIGNED32, 4, n,
                        [](uint64_t c) { return psyc::unsigned32_decode((uint32_t)c); });
    bad += check_decode("unsigned40 decode", PSY_COMPACT_UNSIGNED40, 5, n,
                        [](uint64_t c) { return psyc::unsigned40_decode(c); });
    bad += check_decode("signed48 decode", PSY_COMPACT_SIGNED48, 6, n,
                        [](uint64_t c) { return psyc::signed48_decode(c); });
    return bad != 0;
}
