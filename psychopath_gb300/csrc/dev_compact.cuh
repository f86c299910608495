// Compact encodings of Psychopath's `compact` crate (sub_crates/compact) as
// device functions, bit-exact with the crate's f32 arithmetic: this file is
// compiled with --fmad=false, every division and square root is the IEEE
// one, and the crate's f32::max / f32::min (which return the other operand
// when one is NaN) are fmaxf / fminf.
//
//   fluv32      sub_crates/compact/src/fluv/fluv32.rs: 7-bit exponent (bias
//               63) and 9-bit mantissa of Y, then 8-bit u' and v' scaled by
//               817/2 and 1235/3 (:56-63, encode :76-127, decode :131-170).
//   oct32       sub_crates/compact/src/unit_vec/oct32.rs: octahedral unit
//               vector, two snorm16 coordinates (:7-8, :15-117).
//   unsigned32  sub_crates/compact/src/shared_exp/unsigned32.rs: three 9-bit
//               mantissas and a 5-bit shared exponent, bias 11 (:17-85).
//   unsigned40  sub_crates/compact/src/shared_exp/unsigned40.rs: 11-bit
//               mantissas, 7-bit exponent, bias 32, low five bytes of the
//               little-endian u64 (:17-120).
//   signed48    sub_crates/compact/src/shared_exp/signed48.rs: sign + 13-bit
//               mantissa each, 6-bit exponent, bias 26, low six bytes
//               (:21-144).
//
// The shared-exponent formats take 2^e and floor(log2 x) from the IEEE bit
// fields as the crate does (shared_exp/mod.rs:14-31); mantissas are
// truncated and clamped to the largest mantissa; a negative product
// converts to 0 as Rust's saturating `as u32` does.
#pragma once

#include <stdint.h>

namespace psyc {

__device__ __forceinline__ float exp2_bits(int e) { return __uint_as_float((uint32_t)(e + 127) << 23); }
__device__ __forceinline__ int log2_bits(float f) { return (int)((__float_as_uint(f) >> 23) & 0xffu) - 127; }
// Rust's `f as u32` for a value already clamped from above and not NaN
__device__ __forceinline__ uint32_t sat_u32(float f) { return f > 0.0f ? (uint32_t)f : 0u; }

// ------------------------------------------------------------------ fluv32
constexpr float kUScale = 817.0f / 2.0f;
constexpr float kVScale = 1235.0f / 3.0f;
constexpr float kVURatio = kVScale / kUScale;
constexpr uint32_t kFluvBias = 64;  // 127 - 63

// The two chroma bytes, trunc(clamp(fl(fl(a / s) + 0.5), lo, 255)) for
// a = 1634 x (lo 0) and a = 9 * 1235/3 y (lo 1) with the IEEE quotient
// (fluv32.rs:94-105), as the crate computes them.  Out of line: the fast
// form below decides all but a few inputs in ten thousand.
__device__ __noinline__ uint32_t fluv32_uv_exact(float au, float av, float s) {
    return ((uint32_t)fminf(fmaxf(au / s + 0.5f, 0.0f), 255.0f) << 8) |
           (uint32_t)fminf(fmaxf(av / s + 0.5f, 1.0f), 255.0f);
}

// A fast chroma value t = fl(q + 0.5) floors to the exact computation's
// integer when it is over 2^-11 from an integer, or at least 256 (both clamp
// to 255).
__device__ __forceinline__ bool fluv32_chroma_sure(float t, float fl) {
    return t >= 256.0f || (t > -1.0f && t - fl > 0x1p-11f && t - fl < 1.0f - 0x1p-11f);
}

// Only the integers matter, so the quotients are first taken as a * sc *
// r with r = __fdividef(1, s * sc) (within 2 ulps for 2^-126 < |s * sc| <
// 2^126) and sc = 2^-clamp(floor(log2 s), -126, 126), which puts s * sc in
// [2^-23, 4) without changing the quotient (the scalings are exact, except
// that an a below 2^-126 of s may lose bits far under the margin, and an a
// that overflows gives infinity as the exact quotient does).  For a
// quotient below 256 that is within 2^-21.7 relative, 2^-13.7 absolute, of
// the exact one, and the fast fl(q + 0.5) within 2^-13.3 of the exact
// computation's; whenever it is over 2^-11 from an integer both floor to
// the same integer.  Any other case (an s that is zero, negative, not
// finite or NaN included) takes the exact form.
__device__ __forceinline__ uint32_t fluv32_uv(float x, float y, float z) {
    const float s = x + 15.0f * y + 3.0f * z;
    const float au = (4.0f * kUScale) * x, av = (9.0f * kVScale) * y;
    const float sc = exp2_bits(-min(max(log2_bits(s), -126), 126));  // used only for a positive finite s
    const float r = __fdividef(1.0f, s * sc);
    const float tu = (au * sc) * r + 0.5f, tv = (av * sc) * r + 0.5f;
    const float fu = floorf(tu), fv = floorf(tv);
    if (s > 0.0f && s <= 3.40282347e38f && fluv32_chroma_sure(tu, fu) && fluv32_chroma_sure(tv, fv))
        return ((uint32_t)fminf(fmaxf(fu, 0.0f), 255.0f) << 8) | (uint32_t)fminf(fmaxf(fv, 1.0f), 255.0f);
    return fluv32_uv_exact(au, av, s);
}

// encode_uv((1, 1, 1)): u = 1634/19 + 0.5 = 86.5 -> 0x56, v = 3705/19 + 0.5 = 195.5 -> 0xc3
constexpr uint32_t kFluvWhiteUV = 0x56c3u;

// Black (Y below the format) and infinite Y take the chroma of (1, 1, 1);
// Y above the format saturates to the brightest Y with its own chroma
// (fluv32.rs:107-126).  Branch-free: those lanes evaluate the chroma of
// (1, 1, 1) itself (86.5 and 195.5 before truncation, far from integer
// boundaries, so the fast form returns kFluvWhiteUV), and every lane of a
// warp stays active.
__device__ __forceinline__ uint32_t fluv32_encode(float x, float y, float z) {
    const uint32_t yb = __float_as_uint(y) & 0x7fffffffu;
    const bool black = yb < ((kFluvBias + 1) << 23), bright = yb >= ((kFluvBias + 128) << 23);
    const bool white = black || (bright && isinf(y));
    const uint32_t uv = fluv32_uv(white ? 1.0f : x, white ? 1.0f : y, white ? 1.0f : z);
    const uint32_t lum = black ? 0u : bright ? 0xffff0000u : (((yb - (kFluvBias << 23)) << 2) & 0xffff0000u);
    return lum | uv;
}

__device__ __forceinline__ float fluv32_y(uint32_t c) {
    return c <= 0xffffu ? 0.0f : __uint_as_float(((c & 0xffff0000u) >> 2) + (kFluvBias << 23));
}

__device__ __forceinline__ float3 fluv32_decode(uint32_t c) {
    const float y = fluv32_y(c);
    const float u = (float)((c >> 8) & 0xffu), v = (float)(c & 0xffu);
    const float t = y / v;
    const float x = t * ((2.25f * kVURatio) * u);
    const float z = t * ((3.0f * kVScale) - ((0.75f * kVURatio) * u) - (5.0f * v));
    return make_float3(x, y, fmaxf(z, 0.0f));
}

// ------------------------------------------------------------------- oct32
constexpr float kOctSteps = 32767.0f;
constexpr float kOctStep = 1.0f / kOctSteps;

__device__ __forceinline__ float oct_sign(float n) { return n < 0.0f ? -1.0f : 1.0f; }

__device__ __forceinline__ float2 vec3_to_oct(float x, float y, float z) {
    const float l1 = fabsf(x) + fabsf(y) + fabsf(z);
    const float u = x / l1, v = y / l1;
    if (z > 0.0f) return make_float2(u, v);
    return make_float2((1.0f - fabsf(v)) * oct_sign(x), (1.0f - fabsf(u)) * oct_sign(y));
}

__device__ __forceinline__ float3 oct_to_vec3(float a, float b) {
    const float w = 1.0f - (fabsf(a) + fabsf(b));
    if (w < 0.0f) return make_float3((1.0f - fabsf(b)) * oct_sign(a), (1.0f - fabsf(a)) * oct_sign(b), w);
    return make_float3(a, b, w);
}

// round half away from zero, then Rust's saturating `as i16`
__device__ __forceinline__ uint32_t to_snorm16(float n) {
    const float r = roundf(n * kOctSteps);
    const int32_t i = isnan(r) ? 0 : (int32_t)fminf(fmaxf(r, -32768.0f), 32767.0f);
    return (uint32_t)(uint16_t)(int16_t)i;
}

__device__ __forceinline__ float from_snorm16(uint32_t b) { return (float)(int16_t)(uint16_t)b * kOctStep; }

__device__ __forceinline__ uint32_t oct32_encode(float x, float y, float z) {
    const float2 o = vec3_to_oct(x, y, z);
    return (to_snorm16(o.x) << 16) | to_snorm16(o.y);
}

// The crate's f64 cosine of candidate o with the input v (oct32.rs:26-30).
// Out of line: only the rare inputs the f32 ranking cannot decide call it.
__device__ __noinline__ double oct_dot64(float3 o, float x, float y, float z) {
    const double ox = o.x, oy = o.y, oz = o.z;
    const double l = sqrt(ox * ox + oy * oy + oz * oz);
    return (ox * (double)x + oy * (double)y + oz * (double)z) / l;
}

// a*b - c*d with Kahan's FMA algorithm: within 2 ulps of the exact value
// (Jeannerod, Louvet, Muller, "Further analysis of Kahan's algorithm for
// the accurate computation of 2x2 determinants", Math. Comp. 82, 2013).
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d) {
    const float w = c * d;
    const float e = fmaf(-c, d, w);  // w - c*d exactly
    const float f = fmaf(a, b, -w);
    return f + e;
}

// The floored grid point and its three upper neighbours; the one whose
// decoded direction has the largest f64 cosine with the input wins (ties
// keep the earlier candidate, a cosine <= 0 keeps the floored point).
//
// FP64 runs at a small fraction of the f32 rate on this GPU, and the
// candidates' cosines differ only in second order (~1e-9), so they are
// ranked by sin^2 of their angle to the input instead, a first-order
// quantity computed in f32: |o x v|^2 / (|o|^2 |v|^2) with the cross product
// by diff_of_products, v scaled by a power of two to |v|_1 in [1, 2) (exact,
// except that components below 2^-149 of |v|_1 may flush: an angle change
// far under the 2^-40 floor below).
// Every rounding there is relative to the quantity itself, so each f32
// sin^2 is within 15 * 2^-24 (relative) of the exact value.  With every
// candidate within 30 degrees of the input and in front of it (cosine > 0:
// the first candidate beats the floored point's 0), a larger cosine is a
// smaller sin^2, and the difference of two cosines is at least half the
// difference of their sin^2.  A comparison whose f32 sin^2 differ by more
// than 2^-16 of the larger one (8x the sum of both errors) and by more than
// 2^-40 (the cosines then differ by over 100x the f64 rounding of the
// crate's cosines) therefore has the outcome of the crate's f64 comparison; any
// other comparison, and any input outside this regime (a zero vector, NaN,
// infinity, |v|_1 overflowing, a candidate over 30 degrees away), is
// decided by the crate's own f64 cosines, in the crate's order, so the code
// is bit-identical.
__device__ __forceinline__ uint32_t oct32_encode_precise(float x, float y, float z) {
    float2 s = vec3_to_oct(x, y, z);
    s.x = floorf(fminf(fmaxf(s.x, -1.0f), 1.0f) * kOctSteps) * kOctStep;
    s.y = floorf(fminf(fmaxf(s.y, -1.0f), 1.0f) * kOctSteps) * kOctStep;
    float2 cand[4];
    float3 o[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        cand[k] = make_float2(s.x + ((k & 2) ? kOctStep : 0.0f), s.y + ((k & 1) ? kOctStep : 0.0f));
        o[k] = oct_to_vec3(cand[k].x, cand[k].y);
    }
    const float l1 = fabsf(x) + fabsf(y) + fabsf(z);
    bool fast = l1 > 0.0f && l1 <= 3.40282347e38f;  // finite, non-zero (false for NaN)
    float s2[4];
    if (fast) {
        const float sc = exp2_bits(-log2_bits(l1));
        const float vx = x * sc, vy = y * sc, vz = z * sc;
        const float vv = vx * vx + vy * vy + vz * vz;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float3 q = o[k];
            const float cx = diff_of_products(q.y, vz, q.z, vy);
            const float cy = diff_of_products(q.z, vx, q.x, vz);
            const float cz = diff_of_products(q.x, vy, q.y, vx);
            const float oo = q.x * q.x + q.y * q.y + q.z * q.z;
            s2[k] = (cx * cx + cy * cy + cz * cz) / (oo * vv);
            const float dt = q.x * vx + q.y * vy + q.z * vz;
            fast = fast && dt > 0.0f && s2[k] < 0.25f;
        }
    }
    if (!fast) {  // the crate's sequence on f64 cosines
        float2 bc = s;
        double best = 0.0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const double d = oct_dot64(o[k], x, y, z);
            if (d > best) {
                bc = cand[k];
                best = d;
            }
        }
        return (to_snorm16(bc.x) << 16) | to_snorm16(bc.y);
    }
    // candidate 0 beats the floored point; then each later one in turn
    float2 bc = cand[0];
    float3 bo = o[0];
    float bs2 = s2[0];
    double best_d = 0.0;
    bool best_d_known = false;  // best_d holds the f64 cosine of the winner
#pragma unroll
    for (int k = 1; k < 4; k++) {
        const float diff = s2[k] - bs2;
        bool wins;
        if (fabsf(diff) > fmaxf(fmaxf(s2[k], bs2) * 0x1p-16f, 0x1p-45f)) {
            wins = diff < 0.0f;
            if (wins) best_d_known = false;
        } else {
            if (!best_d_known) best_d = oct_dot64(bo, x, y, z);
            const double d = oct_dot64(o[k], x, y, z);
            wins = d > best_d;
            if (wins) best_d = d;
            best_d_known = true;
        }
        if (wins) {
            bc = cand[k];
            bo = o[k];
            bs2 = s2[k];
        }
    }
    return (to_snorm16(bc.x) << 16) | to_snorm16(bc.y);
}

__device__ __forceinline__ float3 oct32_decode(uint32_t c) { return oct_to_vec3(from_snorm16(c >> 16), from_snorm16(c)); }

// ------------------------------------------------------ shared exponent
__device__ __forceinline__ uint32_t unsigned32_encode(float a, float b, float c) {
    const float big = fmaxf(a, fmaxf(b, c));
    if (big < 1.0f / 524288.0f) return 0;  // 2^-19, the smallest non-zero value
    const int e = min(max(log2_bits(big), -11), 20);
    const float inv = exp2_bits(8 - e);
    const uint32_t x = sat_u32(fminf(a * inv, 511.0f));
    const uint32_t y = sat_u32(fminf(b * inv, 511.0f));
    const uint32_t z = sat_u32(fminf(c * inv, 511.0f));
    return (x << 23) | (y << 14) | (z << 5) | (uint32_t)(e + 11);
}

__device__ __forceinline__ float3 unsigned32_decode(uint32_t t) {
    const float m = exp2_bits((int)(t & 31u) - 19);
    return make_float3((float)(t >> 23) * m, (float)((t >> 14) & 511u) * m, (float)((t >> 5) & 511u) * m);
}

__device__ __forceinline__ uint64_t unsigned40_encode(float a, float b, float c) {
    const float big = fmaxf(a, fmaxf(b, c));
    if (big < 0x1p-42f) return 0;
    const int e = min(max(log2_bits(big), -32), 95);
    const float inv = exp2_bits(10 - e);
    const uint32_t x = sat_u32(fminf(a * inv, 2047.0f));
    const uint32_t y = sat_u32(fminf(b * inv, 2047.0f));
    const uint32_t z = sat_u32(fminf(c * inv, 2047.0f));
    // bits: x 29..39, y 18..28, z 7..17, exponent 0..6
    const uint32_t lo = (x << 29) | (y << 18) | (z << 7) | (uint32_t)(e + 32);
    return ((uint64_t)(x >> 3) << 32) | lo;
}

__device__ __forceinline__ float3 unsigned40_decode(uint64_t t) {
    const float m = exp2_bits((int)(t & 127u) - 42);
    return make_float3((float)(uint32_t)((t >> 29) & 2047u) * m, (float)(uint32_t)((t >> 18) & 2047u) * m,
                       (float)(uint32_t)((t >> 7) & 2047u) * m);
}

__device__ __forceinline__ uint64_t signed48_encode(float a, float b, float c) {
    const float aa = fabsf(a), ab = fabsf(b), ac = fabsf(c);
    const float big = fmaxf(aa, fmaxf(ab, ac));
    if (big < 0x1p-38f) return 0;
    const int e = min(max(log2_bits(big), -26), 37);
    const float inv = exp2_bits(12 - e);
    const uint32_t x = sat_u32(fminf(aa * inv, 8191.0f));
    const uint32_t y = sat_u32(fminf(ab * inv, 8191.0f));
    const uint32_t z = sat_u32(fminf(ac * inv, 8191.0f));
    const uint32_t sx = __float_as_uint(a) >> 31, sy = __float_as_uint(b) >> 31, sz = __float_as_uint(c) >> 31;
    // bits: sign x 47, x 34..46, sign y 33, y 20..32, sign z 19, z 6..18, exponent 0..5
    const uint32_t lo = (y << 20) | (sz << 19) | (z << 6) | (uint32_t)(e + 26);
    const uint32_t hi = (sx << 15) | (x << 2) | (sy << 1) | (y >> 12);
    return ((uint64_t)hi << 32) | lo;
}

__device__ __forceinline__ float3 signed48_decode(uint64_t t) {
    const float m = exp2_bits((int)(t & 63u) - 38);
    const float x = (float)(uint32_t)((t >> 34) & 8191u) * m, y = (float)(uint32_t)((t >> 20) & 8191u) * m,
                z = (float)(uint32_t)((t >> 6) & 8191u) * m;
    return make_float3(__uint_as_float(__float_as_uint(x) | ((uint32_t)(t >> 16) & 0x80000000u)),
                       __uint_as_float(__float_as_uint(y) | ((uint32_t)(t >> 2) & 0x80000000u)),
                       __uint_as_float(__float_as_uint(z) | ((uint32_t)(t << 12) & 0x80000000u)));
}

// ------------------------------------------------------------------- f16
// IEEE binary32 -> binary16 with round to nearest even, as the `half` crate
// (1.7.1) converts: overflow goes to infinity, a NaN keeps its sign and top
// payload bits with the quiet bit set.  binary16 -> binary32 is exact (a NaN
// gets the quiet bit).
__device__ __forceinline__ uint32_t f32_to_f16_bits(float f) {
    const uint32_t x = __float_as_uint(f);
    const uint32_t sign = (x >> 16) & 0x8000u, ex = (x >> 23) & 0xffu, man = x & 0x7fffffu;
    if (ex == 0xffu) return sign | 0x7c00u | (man ? 0x200u | (man >> 13) : 0u);
    const int e = (int)ex - 112;  // binary16 biased exponent
    if (e >= 31) return sign | 0x7c00u;
    if (e <= 0) {  // subnormal binary16 or zero
        if (e < -10) return sign;
        const uint32_t m = man | 0x800000u;
        const int shift = 14 - e;
        uint32_t h = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) h++;
        return sign | h;
    }
    uint32_t h = sign | ((uint32_t)e << 10) | (man >> 13);
    const uint32_t rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;  // a carry rounds up into the exponent
    return h;
}

__device__ __forceinline__ float f16_bits_to_f32(uint32_t h) {
    const uint32_t sign = (h & 0x8000u) << 16, e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    if (e == 0x1fu) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u | (m << 13) : 0u));
    if (e == 0) {
        const float v = (float)m * 0x1p-24f;  // exact
        return __uint_as_float(__float_as_uint(v) | sign);
    }
    return __uint_as_float(sign | ((e + 112u) << 23) | (m << 13));
}

}  // namespace psyc
