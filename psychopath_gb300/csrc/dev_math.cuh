// Device arithmetic of the tracing path: vectors, Psychopath's affine
// transforms, slab and watertight triangle tests, samplers, spectral
// upsampling, closures and light sampling.
//
// Every function evaluates the same IEEE operations, in the same order, as
// the reference's CPU code (glam on x86_64: SSE, no fused multiply-add), so
// with --fmad=false the traversal and sampling arithmetic is bit-identical
// to the CPU path.  Vector min/max use the SSE operand order ((a < b) ? a
// : b); scalar Rust f32::min/max map to fminf/fmaxf.  Transcendental
// functions (sin, cos, acos, asin, log in f32/f64) are CUDA's and may differ
// from the host libm in the last ulp.
#pragma once

#include <math_constants.h>
#include <stdint.h>

#include "psy_layout.h"

#define PSY_MENG_CONST static __device__ const
#include "spectra_tables.inc"

namespace psyd {

#define DI __device__ __forceinline__

// ------------------------------------------------------------------ scalars
DI float vmin(float a, float b) { return (a < b) ? a : b; }
DI float vmax(float a, float b) { return (a > b) ? a : b; }
DI float rmin(float a, float b) { return fminf(a, b); }
DI float rmax(float a, float b) { return fmaxf(a, b); }
DI float rclamp(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
DI float signum(float v) { return isnan(v) ? v : (signbit(v) ? -1.0f : 1.0f); }

// ------------------------------------------------------------------ float3
struct V3 {
    float x, y, z;
    DI float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
DI V3 v3(float x, float y, float z) { return V3{x, y, z}; }
DI V3 v3(float4 a) { return V3{a.x, a.y, a.z}; }
DI V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
DI V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
DI V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
DI V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
DI V3 neg(V3 a) { return a * -1.0f; }
DI float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
DI V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
DI float length2(V3 a) { return dot(a, a); }
DI float length(V3 a) { return sqrtf(dot(a, a)); }
DI V3 normalized(V3 a) { return a * (1.0f / length(a)); }
DI V3 vmin3(V3 a, V3 b) { return v3(vmin(a.x, b.x), vmin(a.y, b.y), vmin(a.z, b.z)); }
DI V3 vmax3(V3 a, V3 b) { return v3(vmax(a.x, b.x), vmax(a.y, b.y), vmax(a.z, b.z)); }
DI V3 vabs(V3 a) { return v3(a.x * signum(a.x), a.y * signum(a.y), a.z * signum(a.z)); }
DI float max_elem3(V3 a) { return vmax(vmax(a.x, a.y), a.z); }
DI V3 recip(V3 a) { return v3(1.0f / a.x, 1.0f / a.y, 1.0f / a.z); }

struct V4 {
    float e[4];
    DI float &operator[](int i) { return e[i]; }
    DI float operator[](int i) const { return e[i]; }
};
DI V4 v4(float a, float b, float c, float d) { return V4{{a, b, c, d}}; }
DI V4 v4(float4 a) { return V4{{a.x, a.y, a.z, a.w}}; }
DI float4 f4(V4 a) { return make_float4(a[0], a[1], a[2], a[3]); }
DI V4 splat4(float s) { return v4(s, s, s, s); }
DI V4 operator+(V4 a, V4 b) { return v4(a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]); }
DI V4 operator-(V4 a, V4 b) { return v4(a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]); }
DI V4 operator*(V4 a, V4 b) { return v4(a[0] * b[0], a[1] * b[1], a[2] * b[2], a[3] * b[3]); }
DI V4 operator/(V4 a, V4 b) { return v4(a[0] / b[0], a[1] / b[1], a[2] / b[2], a[3] / b[3]); }
DI V4 operator*(V4 a, float s) { return v4(a[0] * s, a[1] * s, a[2] * s, a[3] * s); }
DI float max_elem4(V4 a) { return vmax(vmax(a[0], a[2]), vmax(a[1], a[3])); }

// ------------------------------------------------------------------ affine
// 3x4 row-major affine (Transform over glam Affine3A): m[r*4 + c].
struct Xf {
    float m[12];
};
DI Xf xf_identity() {
    Xf x;
#pragma unroll
    for (int i = 0; i < 12; i++) x.m[i] = 0.0f;
    x.m[0] = 1.0f; x.m[5] = 1.0f; x.m[10] = 1.0f;
    return x;
}
DI Xf xf_load(const float4 *p) {
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    Xf x;
    x.m[0] = a.x; x.m[1] = a.y; x.m[2] = a.z; x.m[3] = a.w;
    x.m[4] = b.x; x.m[5] = b.y; x.m[6] = b.z; x.m[7] = b.w;
    x.m[8] = c.x; x.m[9] = c.y; x.m[10] = c.z; x.m[11] = c.w;
    return x;
}
DI V3 xf_point(V3 p, const Xf &t) {
    const float *m = t.m;
    return v3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
              ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}
DI V3 xf_vector(V3 v, const Xf &t) {
    const float *m = t.m;
    return v3((m[0] * v.x + m[1] * v.y) + m[2] * v.z, (m[4] * v.x + m[5] * v.y) + m[6] * v.z,
              (m[8] * v.x + m[9] * v.y) + m[10] * v.z);
}
DI void mat3_inverse(const Xf &t, float inv[9]) {
    const float *m = t.m;
    V3 c0 = v3(m[0], m[4], m[8]), c1 = v3(m[1], m[5], m[9]), c2 = v3(m[2], m[6], m[10]);
    V3 r0 = cross(c1, c2), r1 = cross(c2, c0), r2 = cross(c0, c1);
    float det = dot(c2, r2);
    float id = 1.0f / det;
    inv[0] = r0.x * id; inv[1] = r0.y * id; inv[2] = r0.z * id;
    inv[3] = r1.x * id; inv[4] = r1.y * id; inv[5] = r1.z * id;
    inv[6] = r2.x * id; inv[7] = r2.y * id; inv[8] = r2.z * id;
}
DI Xf xf_inverse(const Xf &t) {
    float inv[9];
    mat3_inverse(t, inv);
    Xf o;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        o.m[r * 4 + 0] = inv[r * 3 + 0];
        o.m[r * 4 + 1] = inv[r * 3 + 1];
        o.m[r * 4 + 2] = inv[r * 3 + 2];
        float tr = (inv[r * 3 + 0] * t.m[3] + inv[r * 3 + 1] * t.m[7]) + inv[r * 3 + 2] * t.m[11];
        o.m[r * 4 + 3] = tr * -1.0f;
    }
    return o;
}
DI V3 xf_normal(V3 n, const Xf &t) {
    float inv[9];
    mat3_inverse(t, inv);
    return v3((inv[0] * n.x + inv[3] * n.y) + inv[6] * n.z, (inv[1] * n.x + inv[4] * n.y) + inv[7] * n.z,
              (inv[2] * n.x + inv[5] * n.y) + inv[8] * n.z);
}
DI Xf xf_lerp(const Xf &a, const Xf &b, float alpha) {
    Xf o;
    float ia = 1.0f - alpha;
#pragma unroll
    for (int i = 0; i < 12; i++) o.m[i] = a.m[i] * ia + b.m[i] * alpha;
    return o;
}

// ------------------------------------------------------------------ lerp_slice
DI bool lerp_index(uint32_t n, float alpha, uint32_t *i1, float *a2) {
    if (n == 1 || alpha == 1.0f) {
        *i1 = n - 1;
        *a2 = 0.0f;
        return true;
    }
    float tmp = alpha * (float)(n - 1);
    uint32_t i = (uint32_t)tmp;
    *i1 = i;
    *a2 = tmp - (float)i;
    return false;
}
DI float lerpf(float a, float b, float alpha) { return (a * (1.0f - alpha)) + (b * alpha); }
DI V3 lerp3(V3 a, V3 b, float alpha) {
    float ia = 1.0f - alpha;
    return (a * ia) + (b * alpha);
}
DI float lerp_slice_f(const float *s, uint32_t n, float alpha) {
    uint32_t i; float a2;
    if (lerp_index(n, alpha, &i, &a2)) return __ldg(s + i);
    return lerpf(__ldg(s + i), __ldg(s + i + 1), a2);
}
DI V3 lerp_slice_v3(const float4 *s, uint32_t n, float alpha) {
    uint32_t i; float a2;
    if (lerp_index(n, alpha, &i, &a2)) return v3(__ldg(s + i));
    return lerp3(v3(__ldg(s + i)), v3(__ldg(s + i + 1)), a2);
}
DI Xf lerp_slice_xf(const float4 *keys, uint32_t n, float alpha) {
    uint32_t i; float a2;
    if (lerp_index(n, alpha, &i, &a2)) return xf_load(keys + 3 * i);
    return xf_lerp(xf_load(keys + 3 * i), xf_load(keys + 3 * (i + 1)), a2);
}

// ------------------------------------------------------------------ hashes / samplers
DI uint32_t hash_u32(uint32_t n, uint32_t seed) {
    uint32_t h = n;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        h = h * 0x736caf6fu;
        h ^= h >> 16;
        h ^= seed;
    }
    return h;
}
DI float hash_u32_to_f32(uint32_t n, uint32_t seed) {
    const float inv_max = 1.0f / 4294967296.0f;
    return __uint2float_rn(hash_u32(n, seed)) * inv_max;
}
DI float golden_ratio_sample(uint32_t i, uint32_t scramble) {
    uint32_t n = (i + hash_u32(scramble, 0)) * 2654435769u;
    return __uint2float_rn(n) * (1.0f / 4294967296.0f);
}
// Sobol generator matrices for 8 dimensions (van der Corput + Joe & Kuo
// 2..8) as nibble tables, filled by the host at library load (each
// translation unit that samples has its own copy): entry [dim][p][v] is the
// XOR of the direction numbers of the set bits of v placed at bits 4p..4p+3
// of the index.  The Sobol point is the XOR of the direction numbers of the
// index's set bits (a matrix-vector product over GF(2)), so eight lookups
// per dimension give the same value as a loop over the index's 32 bits --
// XOR is associative and commutative -- for an eighth of the instructions.
// Global memory read through the read-only path: a warp's lookups of one
// (dim, p) fall in one 64-byte row, one L1 wavefront.
static __device__ __align__(16) uint32_t g_sobol_nib[8][8][16];
DI uint32_t laine_karras(uint32_t x, uint32_t seed) {
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return x;
}
DI uint32_t nested_uniform_scramble(uint32_t x, uint32_t seed) { return __brev(laine_karras(__brev(x), seed)); }
DI uint32_t hash_combine(uint32_t seed, uint32_t v) { return seed ^ (v + (seed << 6) + (seed >> 2)); }
DI void sobol_burley_4d(uint32_t index, uint32_t set, uint32_t seed, float out[4]) {
    uint32_t idx = nested_uniform_scramble(index, seed);
#pragma unroll
    for (uint32_t k = 0; k < 4; k++) {
        uint32_t dim = set * 4 + k;
        const uint32_t *t = &g_sobol_nib[dim][0][0];
        uint32_t x = 0;
#pragma unroll
        for (uint32_t p = 0; p < 8; p++) x ^= __ldg(t + 16 * p + ((idx >> (4 * p)) & 15u));
        x = nested_uniform_scramble(x, hash_combine(seed, dim));
        out[k] = (float)(x >> 8) * (1.0f / 16777216.0f);
    }
}
#define PSY_SOBOL_SETS 2u
DI void get_sample_4d(uint32_t i, uint32_t set, uint32_t px, uint32_t py, uint32_t seed, float out[4]) {
    uint32_t s = px ^ (py << 16) ^ (seed * 0x736caf6fu);
    if (set < PSY_SOBOL_SETS) {
        sobol_burley_4d(i, set, s, out);
    } else {
#pragma unroll
        for (uint32_t k = 0; k < 4; k++) out[k] = hash_u32_to_f32((set * 4 + k) ^ (i << 16), s);
    }
}
// Acklam's probit approximation (src/math.rs:67-132); the reference
// evaluates it in f64 (R = double), the precision variant in f32.
DI double plog(double x) { return log(x); }
DI float plog(float x) { return logf(x); }
DI double psqrt(double x) { return sqrt(x); }
DI float psqrt(float x) { return sqrtf(x); }
template <class R>
DI float probit(float nf, float width) {
    R n = (R)nf;
    const R A1 = (R)-3.969683028665376e+01, A2 = (R)2.209460984245205e+02, A3 = (R)-2.759285104469687e+02,
            A4 = (R)1.383577518672690e+02, A5 = (R)-3.066479806614716e+01, A6 = (R)2.506628277459239e+00;
    const R B1 = (R)-5.447609879822406e+01, B2 = (R)1.615858368580409e+02, B3 = (R)-1.556989798598866e+02,
            B4 = (R)6.680131188771972e+01, B5 = (R)-1.328068155288572e+01;
    const R C1 = (R)-7.784894002430293e-03, C2 = (R)-3.223964580411365e-01, C3 = (R)-2.400758277161838e+00,
            C4 = (R)-2.549732539343734e+00, C5 = (R)4.374664141464968e+00, C6 = (R)2.938163982698783e+00;
    const R D1 = (R)7.784695709041462e-03, D2 = (R)3.224671290700398e-01, D3 = (R)2.445134137142996e+00,
            D4 = (R)3.754408661907416e+00;
    const R N_LOW = (R)0.02425, N_HIGH = (R)1 - N_LOW;
    R x;
    if ((R)0 < n && n < N_LOW) {
        R q = psqrt((R)-2 * plog(n));
        x = (((((C1 * q + C2) * q + C3) * q + C4) * q + C5) * q + C6) / ((((D1 * q + D2) * q + D3) * q + D4) * q + (R)1);
    } else if (n <= N_HIGH) {
        R q = n - (R)0.5;
        R r = q * q;
        x = (((((A1 * r + A2) * r + A3) * r + A4) * r + A5) * r + A6) * q /
            (((((B1 * r + B2) * r + B3) * r + B4) * r + B5) * r + (R)1);
    } else if (n < (R)1) {
        R q = psqrt((R)-2 * plog((R)1 - n));
        x = -(((((C1 * q + C2) * q + C3) * q + C4) * q + C5) * q + C6) / ((((D1 * q + D2) * q + D3) * q + D4) * q + (R)1);
    } else if (n == (R)0) {
        x = (R)-CUDART_INF;
    } else if (n == (R)1) {
        x = (R)CUDART_INF;
    } else {
        x = (R)CUDART_NAN;
    }
    return (float)x * width;
}
// Mineiro's fastapprox exp (pow2 of p*log2(e) with a rational correction).
DI float fast_pow2(float p) {
    float offset = (p < 0.0f) ? 1.0f : 0.0f;
    float clipp = (p < -126.0f) ? -126.0f : p;
    int w = (int)clipp;
    float z = clipp - (float)w + offset;
    float v = (float)(1 << 23) * (clipp + 121.2740575f + 27.7280233f / (4.84252568f - z) - 1.49012907f * z);
    return __uint_as_float((uint32_t)v);
}
DI float fast_exp(float p) { return fast_pow2(1.442695040f * p); }

DI float fp_gamma(uint32_t n) {
    const float e = 1.1920929e-07f * 0.5f;
    return (e * (float)n) / (1.0f - (e * (float)n));
}
DI float increment_ulp(float v) {
    if (isfinite(v)) {
        if (v > 0.0f) return __uint_as_float(__float_as_uint(v) + 1);
        if (v < -0.0f) return __uint_as_float(__float_as_uint(v) - 1);
        return __uint_as_float(0x00000001u);
    }
    return v;
}
DI float decrement_ulp(float v) {
    if (isfinite(v)) {
        if (v > 0.0f) return __uint_as_float(__float_as_uint(v) - 1);
        if (v < -0.0f) return __uint_as_float(__float_as_uint(v) + 1);
        return __uint_as_float(0x80000001u);
    }
    return v;
}
DI V3 robust_ray_origin(V3 pos, float pos_err, V3 nor, V3 ray_dir) {
    V3 n = (dot(nor, ray_dir) >= 0.0f) ? nor : neg(nor);
    float d = dot(vabs(n), v3(pos_err, pos_err, pos_err));
    V3 p = pos + n * d;
    float x = (n.x >= 0.0f) ? increment_ulp(p.x) : decrement_ulp(p.x);
    float y = (n.y >= 0.0f) ? increment_ulp(p.y) : decrement_ulp(p.y);
    float z = (n.z >= 0.0f) ? increment_ulp(p.z) : decrement_ulp(p.z);
    return v3(x, y, z);
}
DI float power_heuristic(float a, float b) {
    if (isinf(a)) return a;
    float a2 = a * a, b2 = b * b;
    float mis = a2 / (a2 + b2);
    return a / mis;
}

// ------------------------------------------------------------------ slab test
#define PSY_BBOX_MAXT_ADJUST 1.00000024f
// One lane of BBox4::intersect_ray (src/bbox4.rs:63-97).
DI bool slab_hit(float xlo, float xhi, float ylo, float yhi, float zlo, float zhi, V3 o, V3 di, float max_t) {
    float t1x = (xlo - o.x) * di.x, t1y = (ylo - o.y) * di.y, t1z = (zlo - o.z) * di.z;
    float t2x = (xhi - o.x) * di.x, t2y = (yhi - o.y) * di.y, t2z = (zhi - o.z) * di.z;
    float fx = vmax(t1x, t2x), fy = vmax(t1y, t2y), fz = vmax(t1z, t2z);
    float nx = vmin(t1x, t2x), ny = vmin(t1y, t2y), nz = vmin(t1z, t2z);
    float far_t = vmin(vmin(fx, vmin(fy, fz)) * PSY_BBOX_MAXT_ADJUST, max_t);
    float near_t = vmax(vmax(nx, ny), vmax(nz, 0.0f));
    return near_t < far_t;
}
// Same test when the ray's inverse direction has no infinite or NaN
// component: then no slab distance is NaN, so IEEE minNum/maxNum (one
// instruction each) give the same hit decision as the SSE select order (the
// only difference, the sign of a zero, does not change the comparisons).
DI bool slab_hit_finite(float xlo, float xhi, float ylo, float yhi, float zlo, float zhi, V3 o, V3 di, float max_t) {
    float t1x = (xlo - o.x) * di.x, t1y = (ylo - o.y) * di.y, t1z = (zlo - o.z) * di.z;
    float t2x = (xhi - o.x) * di.x, t2y = (yhi - o.y) * di.y, t2z = (zhi - o.z) * di.z;
    float fx = fmaxf(t1x, t2x), fy = fmaxf(t1y, t2y), fz = fmaxf(t1z, t2z);
    float nx = fminf(t1x, t2x), ny = fminf(t1y, t2y), nz = fminf(t1z, t2z);
    float far_t = fminf(fminf(fx, fminf(fy, fz)) * PSY_BBOX_MAXT_ADJUST, max_t);
    float near_t = fmaxf(fmaxf(nx, ny), fmaxf(nz, 0.0f));
    return near_t < far_t;
}
// Same test with each axis's near and far plane already chosen from the sign
// of the inverse direction (finite, nonzero): for lo <= hi,
// (lo - o) * di <= (hi - o) * di when di > 0 (rounding is monotonic) and the
// reverse when di < 0, so min / max of the two slab distances are known and
// need no instructions.  Decisions equal slab_hit_finite's.
// Three-input minimum / maximum (PTX min.f32 / max.f32 with three
// operands).  Exact, like two two-input steps, for inputs without NaN.
DI float fmin3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
DI float fmax3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
DI bool slab_hit_ordered(float nxp, float fxp, float nyp, float fyp, float nzp, float fzp, V3 o, V3 di, float max_t) {
    float nx = (nxp - o.x) * di.x, ny = (nyp - o.y) * di.y, nz = (nzp - o.z) * di.z;
    float fx = (fxp - o.x) * di.x, fy = (fyp - o.y) * di.y, fz = (fzp - o.z) * di.z;
    // no NaN here (finite, nonzero inverse direction; finite or infinite
    // bounds), so the three-input forms give the same values
    float far_t = fminf(fmin3f(fx, fy, fz) * PSY_BBOX_MAXT_ADJUST, max_t);
    float near_t = fmax3f(nx, ny, fmaxf(nz, 0.0f));
    return near_t < far_t;
}
// Packed two-lane f32 arithmetic (PTX sub.rn.f32x2 / mul.rn.f32x2): each
// lane rounds to nearest like the scalar instruction, so results are the
// same bits at half the instruction count.
typedef unsigned long long f32x2;
DI f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
DI void upk2(f32x2 v, float &a, float &b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
DI f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
DI f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
// (plane - o) * di for the four children of one axis, two children per
// packed operation.
DI void slab_axis4(float4 plane, f32x2 o2, f32x2 d2, float t[4]) {
    upk2(mul2(sub2(pk2(plane.x, plane.y), o2), d2), t[0], t[1]);
    upk2(mul2(sub2(pk2(plane.z, plane.w), o2), d2), t[2], t[3]);
}
DI bool finite3(V3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }
// Inverse direction finite and nonzero in every component (so the slab
// distances (bound - o) * di are never 0 * inf).
DI bool slab_safe(V3 o, V3 di, float tmax) {
    return finite3(o) && finite3(di) && di.x != 0.0f && di.y != 0.0f && di.z != 0.0f && !isnan(tmax);
}
DI uint32_t ray_code(V3 d) {
    return (uint32_t)(d.x < 0.0f) + ((uint32_t)(d.y < 0.0f) << 1) + ((uint32_t)(d.z < 0.0f) << 2);
}

// ------------------------------------------------------------------ triangle
struct TriPre {
    int ix, iy, iz;
    float sx, sy, sz;
};
DI TriPre tri_precompute(V3 d) {
    float xa = fabsf(d.x), ya = fabsf(d.y), za = fabsf(d.z);
    TriPre p;
    if (xa > ya && xa > za) { p.ix = 1; p.iy = 2; p.iz = 0; }
    else if (ya > za) { p.ix = 2; p.iy = 0; p.iz = 1; }
    else { p.ix = 0; p.iy = 1; p.iz = 2; }
    float dx = d[p.ix], dy = d[p.iy], dz = d[p.iz];
    p.sx = dx / dz; p.sy = dy / dz; p.sz = 1.0f / dz;
    return p;
}
DI float max_abs_3(float a, float b, float c) {
    a = fabsf(a); b = fabsf(b); c = fabsf(c);
    if (a > b && a > c) return a;
    if (b > c) return b;
    return c;
}
// Watertight ray/triangle test (Woop et al.) with the f64 retest of zero
// edge functions and the PBRT t error bound (src/surface/triangle.rs:58-149).
DI bool tri_intersect(V3 o, const TriPre &pre, float max_t, V3 t0, V3 t1, V3 t2, float &t_out, float &b0o, float &b1o,
                      float &b2o) {
    V3 p0 = t0 - o, p1 = t1 - o, p2 = t2 - o;
    float p0x = p0[pre.ix] - (pre.sx * p0[pre.iz]);
    float p0y = p0[pre.iy] - (pre.sy * p0[pre.iz]);
    float p1x = p1[pre.ix] - (pre.sx * p1[pre.iz]);
    float p1y = p1[pre.iy] - (pre.sy * p1[pre.iz]);
    float p2x = p2[pre.ix] - (pre.sx * p2[pre.iz]);
    float p2y = p2[pre.iy] - (pre.sy * p2[pre.iz]);
    float e0 = (p1x * p2y) - (p1y * p2x);
    float e1 = (p2x * p0y) - (p2y * p0x);
    float e2 = (p0x * p1y) - (p0y * p1x);
    if (e0 == 0.0f || e1 == 0.0f || e2 == 0.0f) {
        e0 = (float)(((double)p1x * (double)p2y) - ((double)p1y * (double)p2x));
        e1 = (float)(((double)p2x * (double)p0y) - ((double)p2y * (double)p0x));
        e2 = (float)(((double)p0x * (double)p1y) - ((double)p0y * (double)p1x));
    }
    if ((e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) && (e0 > 0.0f || e1 > 0.0f || e2 > 0.0f)) return false;
    float det = e0 + e1 + e2;
    if (det == 0.0f) return false;
    float p0z = pre.sz * p0[pre.iz];
    float p1z = pre.sz * p1[pre.iz];
    float p2z = pre.sz * p2[pre.iz];
    float t_scaled = (e0 * p0z) + (e1 * p1z) + (e2 * p2z);
    if ((det > 0.0f && (t_scaled <= 0.0f || t_scaled > (max_t * det))) ||
        (det < 0.0f && (t_scaled >= 0.0f || t_scaled < (max_t * det))))
        return false;
    float inv_det = 1.0f / det;
    float b0 = e0 * inv_det, b1 = e1 * inv_det, b2 = e2 * inv_det;
    float t = t_scaled * inv_det;
    float max_zt = max_abs_3(p0z, p1z, p2z);
    float dz = fp_gamma(3) * max_zt;
    float max_xt = max_abs_3(p0x, p1x, p2x);
    float max_yt = max_abs_3(p0y, p1y, p2y);
    float dx = fp_gamma(5) * (max_xt + max_zt);
    float dy = fp_gamma(5) * (max_yt + max_zt);
    float de = 2.0f * ((fp_gamma(2) * max_xt * max_yt) + (dy * max_xt + dx * max_yt));
    float max_e = max_abs_3(e0, e1, e2);
    float dt = 3.0f * ((fp_gamma(3) * max_e * max_zt) + (de * max_zt + dz * max_e)) * fabsf(inv_det);
    if (t <= dt) return false;
    t_out = t; b0o = b0; b1o = b1; b2o = b2;
    return true;
}
DI void surface_point(V3 t0, V3 t1, V3 t2, float b0, float b1, float b2, V3 *pos, float *err) {
    *pos = (t0 * b0) + (t1 * b1) + (t2 * b2);
    V3 e = ((vabs(t0) * b0) + (vabs(t1) * b1) + (vabs(t2) * b2)) * fp_gamma(7);
    *err = max_elem3(e);
}

}  // namespace psyd
