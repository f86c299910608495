// Oracle (test infrastructure only): Sobol direction numbers and the
// Burley hash-based Owen scrambling used by get_sample_4d.
#include "oracle_math.h"

namespace psyo {

// Joe & Kuo (2008) primitive polynomials and initial direction numbers for
// Sobol dimensions 2..8 (dimension 1 is the van der Corput sequence).
struct JoeKuoEntry {
    uint32_t s, a;
    uint32_t m[5];
};
static const JoeKuoEntry kJoeKuo[7] = {
    {1, 0, {1, 0, 0, 0, 0}},   {2, 1, {1, 3, 0, 0, 0}},   {3, 1, {1, 3, 1, 0, 0}},
    {3, 2, {1, 1, 1, 0, 0}},   {4, 1, {1, 1, 3, 3, 0}},   {4, 4, {1, 3, 5, 13, 0}},
    {5, 2, {1, 1, 5, 5, 17}},
};

void sobol_directions(uint32_t dirs[8][32]) {
    for (int k = 0; k < 32; k++) dirs[0][k] = 1u << (31 - k);
    for (int d = 1; d < 8; d++) {
        const JoeKuoEntry &e = kJoeKuo[d - 1];
        uint32_t *v = dirs[d];
        for (uint32_t k = 0; k < 32; k++) {
            if (k < e.s) {
                v[k] = e.m[k] << (31 - k);
            } else {
                uint32_t x = v[k - e.s] ^ (v[k - e.s] >> e.s);
                for (uint32_t j = 1; j < e.s; j++)
                    if ((e.a >> (e.s - 1 - j)) & 1u) x ^= v[k - j];
                v[k] = x;
            }
        }
    }
}

static struct SobolTable {
    uint32_t d[8][32];
    SobolTable() { sobol_directions(d); }
} g_sobol;

void sobol_burley_4d(uint32_t index, uint32_t set, uint32_t seed, float out[4]) {
    uint32_t idx = nested_uniform_scramble(index, seed);
    for (uint32_t k = 0; k < 4; k++) {
        uint32_t dim = set * 4 + k;
        uint32_t x = 0;
        for (uint32_t b = 0; b < 32; b++)
            if ((idx >> b) & 1u) x ^= g_sobol.d[dim][b];
        x = nested_uniform_scramble(x, hash_combine(seed, dim));
        out[k] = (float)(x >> 8) * (1.0f / 16777216.0f);
    }
}

}  // namespace psyo
