// Oracle (test infrastructure only): the `compact` crate's encodings
// (sub_crates/compact) restated for the CPU, with the colour and closure
// byte formats built on them (src/color.rs:144-249,
// src/shading/surface_closure.rs:157-253).  Used by tests/ as the checker
// of the GPU library's psy_compact_* / psy_color_* / psy_closure_* calls and
// by bench.py's CPU baseline; the product never links it.
//
// Pinned by the known answers of the crate's own unit tests (fluv32.rs,
// oct32.rs, shared_exp/*.rs `mod tests`) and its oct32 property tests
// (tests/proptest_tests.rs).  Compiled with -ffp-contract=off; f32 maths
// stays f32 (the PSYO_F64 build does not change this file), encode_precise's
// cosine is f64 as in the crate (oct32.rs:26-30).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "psy_oracle.h"

namespace {

uint32_t fbits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
float bitsf(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}
// Rust's f32::max / f32::min: the non-NaN operand wins (IEEE maxNum/minNum)
float rmax(float a, float b) { return fmaxf(a, b); }
float rmin(float a, float b) { return fminf(a, b); }
// Rust's saturating float -> unsigned cast (NaN -> 0)
uint64_t cast_unsigned(float f, double hi) {
    if (!(f > 0.0f)) return 0;
    if ((double)f >= hi) return (uint64_t)hi;
    return (uint64_t)f;
}
int16_t cast_i16(float f) {
    if (f != f) return 0;
    if (f <= -32768.0f) return -32768;
    if (f >= 32767.0f) return 32767;
    return (int16_t)f;
}

// shared_exp/mod.rs:14-31
float fiddle_exp2(int e) { return bitsf((uint32_t)(e + 127) << 23); }
int fiddle_log2(float n) { return (int)((fbits(n) >> 23) & 0xff) - 127; }

// ------------------------------------------------------------ fluv32.rs
const float U_SCALE = 817.0f / 2.0f;   // :60
const float V_SCALE = 1235.0f / 3.0f;  // :63
const uint32_t BIAS_OFFSET = 127 - 63; // :56-57

uint32_t encode_uv(float x, float y, float z) {  // :94-105
    float s = (x + (15.0f * y)) + (3.0f * z);
    float u = rmin(rmax((((4.0f * U_SCALE) * x) / s) + 0.5f, 0.0f), 255.0f);
    float v = rmin(rmax((((9.0f * V_SCALE) * y) / s) + 0.5f, 1.0f), 255.0f);
    return ((uint32_t)cast_unsigned(u, 4294967295.0) << 8) | (uint32_t)cast_unsigned(v, 4294967295.0);
}

uint32_t fluv32_encode(float x, float y, float z) {  // :76-127
    uint32_t y_bits = fbits(y) & 0x7fffffffu;
    if (y_bits < ((BIAS_OFFSET + 1) << 23)) return encode_uv(1.0f, 1.0f, 1.0f);
    if (y_bits >= ((BIAS_OFFSET + 128) << 23)) {
        if (isinf(y)) return 0xffff0000u | encode_uv(1.0f, 1.0f, 1.0f);
        return 0xffff0000u | encode_uv(x, y, z);
    }
    return (((y_bits - (BIAS_OFFSET << 23)) << 2) & 0xffff0000u) | encode_uv(x, y, z);
}

void fluv32_decode_yuv(uint32_t c, float *y, uint8_t *u, uint8_t *v) {  // :160-170
    float yy = bitsf(((c & 0xffff0000u) >> 2) + (BIAS_OFFSET << 23));
    *u = (uint8_t)(c >> 8);
    *v = (uint8_t)c;
    *y = c <= 0xffffu ? 0.0f : yy;
}

void fluv32_decode(uint32_t c, float *out) {  // :131-150
    float y;
    uint8_t ub, vb;
    fluv32_decode_yuv(c, &y, &ub, &vb);
    const float u = (float)ub, v = (float)vb;
    const float VU_RATIO = V_SCALE / U_SCALE;
    const float tmp = y / v;
    const float x = tmp * ((2.25f * VU_RATIO) * u);
    const float z = tmp * (((3.0f * V_SCALE) - ((0.75f * VU_RATIO) * u)) - (5.0f * v));
    out[0] = x;
    out[1] = y;
    out[2] = rmax(z, 0.0f);
}

// ------------------------------------------------------------- oct32.rs
const float STEPS = 32767.0f;          // :8
const float STEP_SIZE = 1.0f / STEPS;  // :7

float sign(float n) { return n < 0.0f ? -1.0f : 1.0f; }  // :111-117

void vec3_to_oct(const float *v, float *o) {  // :73-83
    float l1 = (fabsf(v[0]) + fabsf(v[1])) + fabsf(v[2]);
    float u = v[0] / l1, w = v[1] / l1;
    if (v[2] > 0.0f) {
        o[0] = u;
        o[1] = w;
    } else {
        o[0] = (1.0f - fabsf(w)) * sign(v[0]);
        o[1] = (1.0f - fabsf(u)) * sign(v[1]);
    }
}

void oct_to_vec3(const float *o, float *v) {  // :86-98
    float v2 = 1.0f - (fabsf(o[0]) + fabsf(o[1]));
    if (v2 < 0.0f) {
        v[0] = (1.0f - fabsf(o[1])) * sign(o[0]);
        v[1] = (1.0f - fabsf(o[0])) * sign(o[1]);
    } else {
        v[0] = o[0];
        v[1] = o[1];
    }
    v[2] = v2;
}

uint16_t to_snorm_16(float n) { return (uint16_t)cast_i16(roundf(n * STEPS)); }   // :101-103
float from_snorm_16(uint16_t n) { return (float)(int16_t)n * STEP_SIZE; }         // :106-108

uint32_t oct32_encode(const float *v) {  // :15-18
    float o[2];
    vec3_to_oct(v, o);
    return ((uint32_t)to_snorm_16(o[0]) << 16) | to_snorm_16(o[1]);
}

uint32_t oct32_encode_precise(const float *v) {  // :24-61
    float s[2];
    vec3_to_oct(v, s);
    s[0] = floorf(rmin(rmax(s[0], -1.0f), 1.0f) * STEPS) * STEP_SIZE;
    s[1] = floorf(rmin(rmax(s[1], -1.0f), 1.0f) * STEPS) * STEP_SIZE;
    float best[2] = {s[0], s[1]};
    double max_dot = 0.0;
    const float cand[4][2] = {{0.0f, 0.0f}, {0.0f, STEP_SIZE}, {STEP_SIZE, 0.0f}, {STEP_SIZE, STEP_SIZE}};
    for (int k = 0; k < 4; k++) {
        float c[2] = {s[0] + cand[k][0], s[1] + cand[k][1]};
        float a[3];
        oct_to_vec3(c, a);
        double l = sqrt(((double)a[0] * (double)a[0] + (double)a[1] * (double)a[1]) + (double)a[2] * (double)a[2]);
        double dot = (((double)a[0] * (double)v[0] + (double)a[1] * (double)v[1]) + (double)a[2] * (double)v[2]) / l;
        if (dot > max_dot) {
            best[0] = c[0];
            best[1] = c[1];
            max_dot = dot;
        }
    }
    return ((uint32_t)to_snorm_16(best[0]) << 16) | to_snorm_16(best[1]);
}

void oct32_decode(uint32_t n, float *v) {  // :68-70
    float o[2] = {from_snorm_16((uint16_t)(n >> 16)), from_snorm_16((uint16_t)n)};
    oct_to_vec3(o, v);
}

// ------------------------------------------------------------ shared_exp
// One unsigned format: mantissa bits, exponent bits, bias.
struct UFormat {
    int mbits, ebits, bias;
};
const UFormat U32F = {9, 5, 11};   // unsigned32.rs:3-25
const UFormat U40F = {11, 7, 32};  // unsigned40.rs:3-25

uint64_t unsigned_encode(const UFormat &f, const float *fs) {  // unsigned32.rs:36-65, unsigned40.rs:50-79
    const float min_value = 1.0f / (float)(1ull << (f.bias + f.mbits - 1));
    const float mmax = (float)((1u << f.mbits) - 1);
    const int emax = (1 << f.ebits) - 1 - f.bias;
    float largest = rmax(fs[0], rmax(fs[1], fs[2]));
    if (largest < min_value) return 0;
    int e = fiddle_log2(largest);
    if (e < -f.bias) e = -f.bias;
    if (e > emax) e = emax;
    float inv = fiddle_exp2(-e + (f.mbits - 1));
    uint64_t r = (uint64_t)(e + f.bias);
    for (int i = 0; i < 3; i++) {
        uint64_t m = cast_unsigned(rmin(fs[i] * inv, mmax), 1e30);
        r |= m << (f.ebits + (2 - i) * f.mbits);
    }
    return r;
}

void unsigned_decode(const UFormat &f, uint64_t t, float *out) {  // unsigned32.rs:71-85, unsigned40.rs:83-97
    const uint64_t mmask = (1ull << f.mbits) - 1;
    int e = (int)(t & ((1ull << f.ebits) - 1));
    float mult = fiddle_exp2(e - f.bias - (f.mbits - 1));
    for (int i = 0; i < 3; i++) out[i] = (float)((t >> (f.ebits + (2 - i) * f.mbits)) & mmask) * mult;
}

uint64_t signed48_encode(const float *fs) {  // signed48.rs:62-98
    const float min_positive = 1.0f / (float)(1ull << (26 + 12));
    float a[3] = {fabsf(fs[0]), fabsf(fs[1]), fabsf(fs[2])};
    float largest = rmax(a[0], rmax(a[1], a[2]));
    if (largest < min_positive) return 0;
    int e = fiddle_log2(largest);
    if (e < -26) e = -26;
    if (e > 63 - 26) e = 63 - 26;
    float inv = fiddle_exp2(-e + 12);
    uint64_t r = (uint64_t)(e + 26);
    for (int i = 0; i < 3; i++) {
        uint64_t s = fbits(fs[i]) >> 31;
        uint64_t m = cast_unsigned(rmin(a[i] * inv, 8191.0f), 1e30);
        r |= (s << (47 - 14 * i)) | (m << (34 - 14 * i));
    }
    return r;
}

void signed48_decode(uint64_t t, float *out) {  // signed48.rs:102-121
    int e = (int)(t & 63);
    float mult = fiddle_exp2(e - 26 - 12);
    for (int i = 0; i < 3; i++) {
        uint64_t m = (t >> (34 - 14 * i)) & 8191;
        uint32_t s = (uint32_t)((t >> (47 - 14 * i)) & 1) << 31;
        out[i] = bitsf(fbits((float)m * mult) | s);
    }
}

// ------------------------------------------------------------ half 1.7.1
// f16::from_f32: IEEE binary16 with round to nearest, ties to even; NaN
// keeps sign and top payload bits with the quiet bit set.  Written as
// arithmetic on the exact value rather than on bit fields.
uint16_t f16_from_f32(float f) {
    uint32_t b = fbits(f);
    uint16_t sign = (uint16_t)((b >> 16) & 0x8000u);
    float a = fabsf(f);
    if (a != a) return (uint16_t)(sign | 0x7e00u | ((b & 0x7fffffu) >> 13));
    if (a >= 65520.0f) return (uint16_t)(sign | 0x7c00u);  // rounds past 65504: infinity
    // a = q * 2^k with the binary16 quantum 2^k (k >= -24)
    int ex = fiddle_log2(a);
    int k = (a == 0.0f || ex < -14) ? -24 : ex - 10;
    double q = (double)a / ldexp(1.0, k);  // exact
    double fl = floor(q), rem = q - fl;
    uint32_t m = (uint32_t)fl;
    if (rem > 0.5 || (rem == 0.5 && (m & 1u))) m++;
    // m is the value in quanta of 2^k: rebuild the binary16 bit pattern
    if (k == -24) return (uint16_t)(sign | m);  // subnormal (m may reach 1024 = the smallest normal)
    uint32_t hexp = (uint32_t)(k + 10 + 15);
    if (m == 2048) {
        m = 1024;
        hexp++;
    }
    return (uint16_t)(sign | (hexp << 10) | (m - 1024));
}

float f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1f, m = h & 0x3ff;
    if (e == 0x1f) return bitsf(sign | 0x7f800000u | (m ? (0x400000u | (m << 13)) : 0u));
    float v = e == 0 ? (float)ldexp((double)m, -24) : (float)ldexp((double)(m | 0x400u), (int)e - 25);
    return bitsf(fbits(v) | sign);
}

// ------------------------------------------------------ colour, closures
bool nonneg3(const float *v) { return v[0] >= 0.0f && v[1] >= 0.0f && v[2] >= 0.0f; }

void put_le(uint8_t *p, uint64_t v, int n) {
    for (int i = 0; i < n; i++) p[i] = (uint8_t)(v >> (8 * i));
}
uint64_t get_le(const uint8_t *p, int n) {
    uint64_t v = 0;
    for (int i = 0; i < n; i++) v |= (uint64_t)p[i] << (8 * i);
    return v;
}

uint32_t color_write(const PsyColor &c, uint8_t *o) {  // color.rs:160-194
    if (c.kind == PSY_COLOR_XYZ) {
        o[0] = 0;
        put_le(o + 1, fluv32_encode(c.v[0], c.v[1], c.v[2]), 4);
        return nonneg3(c.v) ? 0 : 1;
    }
    if (c.kind == PSY_COLOR_BLACKBODY || c.kind == PSY_COLOR_TEMPERATURE) {
        o[0] = (uint8_t)c.kind;
        put_le(o + 1, cast_unsigned(rmin(c.v[0], 65535.0f), 65535.0), 2);
        put_le(o + 3, f16_from_f32(c.v[1]), 2);
        return 0;
    }
    memset(o, 0, 5);
    return 1;
}

uint32_t color_read(const uint8_t *in, PsyColor &c) {  // color.rs:198-249
    if (in[0] == 0) {
        c.kind = PSY_COLOR_XYZ;
        fluv32_decode((uint32_t)get_le(in + 1, 4), c.v);
        return 0;
    }
    c.v[2] = 0.0f;
    if (in[0] == 1 || in[0] == 2) {
        c.kind = in[0];
        c.v[0] = (float)get_le(in + 1, 2);
        c.v[1] = f16_to_f32((uint16_t)get_le(in + 3, 2));
        return 0;
    }
    c.kind = PSY_COLOR_XYZ;
    c.v[0] = c.v[1] = 0.0f;
    return 1;
}

}  // namespace

extern "C" {

int psyo_compact_encode(uint32_t format, const float *xyz, uint32_t n, uint8_t *out, uint32_t *invalid) {
    uint32_t bad = 0;
    for (uint32_t i = 0; i < n; i++) {
        const float *v = xyz + 3 * (size_t)i;
        switch (format) {
            case PSY_COMPACT_FLUV32: put_le(out + 4 * (size_t)i, fluv32_encode(v[0], v[1], v[2]), 4);
                                     bad += !nonneg3(v); break;
            case PSY_COMPACT_OCT32: put_le(out + 4 * (size_t)i, oct32_encode(v), 4); break;
            case PSY_COMPACT_OCT32_PRECISE: put_le(out + 4 * (size_t)i, oct32_encode_precise(v), 4); break;
            case PSY_COMPACT_UNSIGNED32: put_le(out + 4 * (size_t)i, unsigned_encode(U32F, v), 4);
                                         bad += !nonneg3(v); break;
            case PSY_COMPACT_UNSIGNED40: put_le(out + 5 * (size_t)i, unsigned_encode(U40F, v), 5);
                                         bad += !nonneg3(v); break;
            case PSY_COMPACT_SIGNED48: put_le(out + 6 * (size_t)i, signed48_encode(v), 6);
                                       bad += (v[0] != v[0]) || (v[1] != v[1]) || (v[2] != v[2]); break;
            default: return -1;
        }
    }
    if (invalid) *invalid = bad;
    return 0;
}

int psyo_compact_decode(uint32_t format, const uint8_t *in, uint32_t n, float *xyz) {
    for (uint32_t i = 0; i < n; i++) {
        float *v = xyz + 3 * (size_t)i;
        switch (format) {
            case PSY_COMPACT_FLUV32: fluv32_decode((uint32_t)get_le(in + 4 * (size_t)i, 4), v); break;
            case PSY_COMPACT_OCT32:
            case PSY_COMPACT_OCT32_PRECISE: oct32_decode((uint32_t)get_le(in + 4 * (size_t)i, 4), v); break;
            case PSY_COMPACT_UNSIGNED32: unsigned_decode(U32F, get_le(in + 4 * (size_t)i, 4), v); break;
            case PSY_COMPACT_UNSIGNED40: unsigned_decode(U40F, get_le(in + 5 * (size_t)i, 5), v); break;
            case PSY_COMPACT_SIGNED48: signed48_decode(get_le(in + 6 * (size_t)i, 6), v); break;
            default: return -1;
        }
    }
    return 0;
}

// signed48's decode_64 on a whole u64 (upper 16 bits ignored)
void psyo_signed48_decode_u64(uint64_t t, float *out) { signed48_decode(t, out); }

void psyo_fluv32_decode_yuv(const uint32_t *in, uint32_t n, PsyYuv *out) {
    for (uint32_t i = 0; i < n; i++) {
        fluv32_decode_yuv(in[i], &out[i].y, &out[i].u, &out[i].v);
        out[i].pad[0] = out[i].pad[1] = 0;
    }
}

uint32_t psyo_f16_from_f32(float f) { return f16_from_f32(f); }
float psyo_f16_to_f32(uint32_t h) { return f16_to_f32((uint16_t)h); }

int psyo_color_compress(const PsyColor *c, uint32_t n, uint8_t *out, uint32_t *invalid) {
    uint32_t bad = 0;
    for (uint32_t i = 0; i < n; i++) bad += color_write(c[i], out + 5 * (size_t)i);
    if (invalid) *invalid = bad;
    return 0;
}

int psyo_color_decompress(const uint8_t *in, uint32_t n, PsyColor *c, uint32_t *invalid) {
    uint32_t bad = 0;
    for (uint32_t i = 0; i < n; i++) bad += color_read(in + 5 * (size_t)i, c[i]);
    if (invalid) *invalid = bad;
    return 0;
}

// surface_closure.rs:157-208
int psyo_closure_compress(const PsyShaderDesc *s, uint32_t n, uint32_t stride, uint8_t *out, uint32_t *invalid) {
    if (stride < 6) return -1;
    uint32_t bad = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint8_t *o = out + (size_t)i * stride;
        const PsyShaderDesc &c = s[i];
        if (c.kind == PSY_SHADER_GGX) {
            if (stride < 10) {
                bad++;
                continue;
            }
            o[0] = 1;
            put_le(o + 1, cast_unsigned(rmin(rmax(c.roughness, 0.0f), 1.0f) * 65535.0f, 65535.0), 2);
            put_le(o + 3, cast_unsigned(rmin(rmax(c.fresnel, 0.0f), 1.0f) * 65535.0f, 65535.0), 2);
            bad += color_write(c.color, o + 5);
        } else if (c.kind == PSY_SHADER_LAMBERT || c.kind == PSY_SHADER_EMIT) {
            o[0] = c.kind == PSY_SHADER_LAMBERT ? 0 : 2;
            bad += color_write(c.color, o + 1);
        } else {
            bad++;
        }
    }
    if (invalid) *invalid = bad;
    return 0;
}

// surface_closure.rs:212-253
int psyo_closure_decompress(const uint8_t *in, uint32_t n, uint32_t stride, PsyShaderDesc *s, uint32_t *invalid) {
    if (stride < 6) return -1;
    uint32_t bad = 0;
    for (uint32_t i = 0; i < n; i++) {
        const uint8_t *r = in + (size_t)i * stride;
        PsyShaderDesc &c = s[i];
        c.roughness = c.fresnel = 0.0f;
        if (r[0] == 1) {
            if (stride < 10) {
                bad++;
                c.kind = PSY_SHADER_EMIT;
                c.color.kind = PSY_COLOR_XYZ;
                c.color.v[0] = c.color.v[1] = c.color.v[2] = 0.0f;
                continue;
            }
            c.kind = PSY_SHADER_GGX;
            c.roughness = (float)get_le(r + 1, 2) * (1.0f / 65535.0f);
            c.fresnel = (float)get_le(r + 3, 2) * (1.0f / 65535.0f);
            bad += color_read(r + 5, c.color);
        } else {
            c.kind = r[0] == 0 ? PSY_SHADER_LAMBERT : PSY_SHADER_EMIT;
            bad += color_read(r + 1, c.color) | (r[0] > 2 ? 1u : 0u);
        }
    }
    if (invalid) *invalid = bad;
    return 0;
}

}  // extern "C"
