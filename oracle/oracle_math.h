// Oracle (test infrastructure only): CPU restatement of the arithmetic of
// Psychopath's tracing path.  Nothing in the product links this; tests,
// __graft_entry__.smoke() and bench.py's CPU baseline load it as a checker.
//
// Build rule: compiled with -ffp-contract=off and without fast-math, so every
// float operation rounds exactly as written (the reference's glam/SSE code
// has no fused multiply-add).
//
// Precision: `real` is the arithmetic type of the whole path.  The default
// build makes it float, the reference's f32 (places where the reference
// computes in f64 stay double).  Built with -DPSYO_F64 it is double: the
// FP64 oracle, the same algorithm with every f32 operation done in f64.  In
// both builds the sample values (Sobol-Burley, hashes, golden ratio), the
// fastapprox exp (a bit-level method defined on f32), the reference's f32
// constants and the f32 scene data are the same, so the two builds follow
// the same sample sequences and differ only by arithmetic rounding.  Vector min/max follow SSE minps/maxps operand
// order ((a < b) ? a : b), which is what glam 0.15's Vec3A/Vec4 use on
// x86_64; scalar f32::min/max (IEEE minNum/maxNum) map to fminf/fmaxf.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace psyo {

#ifdef PSYO_F64
typedef double real;
#else
typedef float real;
#endif

// ------------------------------------------------------------------ floats
static inline real vmin(real a, real b) { return (a < b) ? a : b; }  // _mm_min_ps lane
static inline real vmax(real a, real b) { return (a > b) ? a : b; }  // _mm_max_ps lane
static inline real rmin(real a, real b) { return std::fmin(a, b); }  // Rust f32::min
static inline real rmax(real a, real b) { return std::fmax(a, b); }  // Rust f32::max
static inline real rclamp(real x, real lo, real hi) {              // Rust f32::clamp
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
static inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline uint64_t d2u(double f) { uint64_t u; std::memcpy(&u, &f, 8); return u; }
static inline double u2d(uint64_t u) { double f; std::memcpy(&f, &u, 8); return f; }

// ------------------------------------------------------------------ vectors
// Point / Vector / Normal share one storage type (glam Vec3A).
struct V3 {
    real x, y, z;
    real operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 v3(real x, real y, real z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, real s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator/(V3 a, real s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline V3 neg(V3 a) { return a * -1.0f; }  // math3d Neg multiplies by -1
// glam dot3: (x*x' + y*y') + z*z'
static inline real dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline real length2(V3 a) { return dot(a, a); }
static inline real length(V3 a) { return std::sqrt(dot(a, a)); }
// glam normalize: self * (1 / length)
static inline V3 normalized(V3 a) { return a * (1.0f / length(a)); }
static inline V3 vmin3(V3 a, V3 b) { return v3(vmin(a.x, b.x), vmin(a.y, b.y), vmin(a.z, b.z)); }
static inline V3 vmax3(V3 a, V3 b) { return v3(vmax(a.x, b.x), vmax(a.y, b.y), vmax(a.z, b.z)); }
// Vector::abs = co * co.signum()  (signum(+0) = 1, signum(-0) = -1)
static inline real signum(real v) { return std::isnan(v) ? v : (std::signbit(v) ? -1.0f : 1.0f); }
static inline V3 vabs(V3 a) { return v3(a.x * signum(a.x), a.y * signum(a.y), a.z * signum(a.z)); }
static inline real max_elem3(V3 a) {  // Vec3A::max_element (SSE reduction order)
    return vmax(vmax(a.x, a.y), a.z);
}

struct V4 {
    real e[4];
    real &operator[](int i) { return e[i]; }
    real operator[](int i) const { return e[i]; }
};
static inline V4 v4(real a, real b, real c, real d) { return V4{{a, b, c, d}}; }
static inline V4 splat4(real s) { return v4(s, s, s, s); }
static inline V4 operator+(V4 a, V4 b) { return v4(a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]); }
static inline V4 operator-(V4 a, V4 b) { return v4(a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]); }
static inline V4 operator*(V4 a, V4 b) { return v4(a[0] * b[0], a[1] * b[1], a[2] * b[2], a[3] * b[3]); }
static inline V4 operator/(V4 a, V4 b) { return v4(a[0] / b[0], a[1] / b[1], a[2] / b[2], a[3] / b[3]); }
static inline V4 operator*(V4 a, real s) { return v4(a[0] * s, a[1] * s, a[2] * s, a[3] * s); }
static inline V4 operator/(V4 a, real s) { return v4(a[0] / s, a[1] / s, a[2] / s, a[3] / s); }
// Vec4::max_element on SSE: max(max(e0,e2), max(e1,e3))
static inline real max_elem4(V4 a) {
    real m02 = vmax(a[0], a[2]);
    real m13 = vmax(a[1], a[3]);
    return vmax(m02, m13);
}

// ------------------------------------------------------------------ transform
// Affine 3x4, row-major: m[r*4 + c], c = 3 is the translation.
// Semantics of math3d::Transform over glam::Affine3A
// (sub_crates/math3d/src/transform.rs:38-146).
struct Xf {
    real m[12];
};
static inline Xf xf_identity() {
    Xf x{};
    x.m[0] = 1.0f; x.m[5] = 1.0f; x.m[10] = 1.0f;
    return x;
}
// Point * Transform (transform_point3a): ((c0*x + c1*y) + c2*z) + t
static inline V3 xf_point(V3 p, const Xf &t) {
    const real *m = t.m;
    return v3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3],
              ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
              ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}
// Vector * Transform (transform_vector3a)
static inline V3 xf_vector(V3 v, const Xf &t) {
    const real *m = t.m;
    return v3((m[0] * v.x + m[1] * v.y) + m[2] * v.z,
              (m[4] * v.x + m[5] * v.y) + m[6] * v.z,
              (m[8] * v.x + m[9] * v.y) + m[10] * v.z);
}
// 3x3 inverse through the adjugate (rows of the inverse are cross products
// of the columns, scaled by 1/det with det = dot(col2, cross(col0, col1))).
static inline void mat3_inverse(const Xf &t, real inv[9]) {
    const real *m = t.m;
    V3 c0 = v3(m[0], m[4], m[8]);
    V3 c1 = v3(m[1], m[5], m[9]);
    V3 c2 = v3(m[2], m[6], m[10]);
    V3 r0 = cross(c1, c2);
    V3 r1 = cross(c2, c0);
    V3 r2 = cross(c0, c1);
    real det = dot(c2, r2);
    real id = 1.0f / det;
    inv[0] = r0.x * id; inv[1] = r0.y * id; inv[2] = r0.z * id;
    inv[3] = r1.x * id; inv[4] = r1.y * id; inv[5] = r1.z * id;
    inv[6] = r2.x * id; inv[7] = r2.y * id; inv[8] = r2.z * id;
}
// Transform::inverse: 3x3 inverse, translation = -(inv * t)
static inline Xf xf_inverse(const Xf &t) {
    real inv[9];
    mat3_inverse(t, inv);
    Xf o;
    for (int r = 0; r < 3; r++) {
        o.m[r * 4 + 0] = inv[r * 3 + 0];
        o.m[r * 4 + 1] = inv[r * 3 + 1];
        o.m[r * 4 + 2] = inv[r * 3 + 2];
        real tr = (inv[r * 3 + 0] * t.m[3] + inv[r * 3 + 1] * t.m[7]) + inv[r * 3 + 2] * t.m[11];
        o.m[r * 4 + 3] = tr * -1.0f;
    }
    return o;
}
// Normal * Transform: inverse-transpose of the 3x3 times n.
static inline V3 xf_normal(V3 n, const Xf &t) {
    real inv[9];
    mat3_inverse(t, inv);
    return v3((inv[0] * n.x + inv[3] * n.y) + inv[6] * n.z,
              (inv[1] * n.x + inv[4] * n.y) + inv[7] * n.z,
              (inv[2] * n.x + inv[5] * n.y) + inv[8] * n.z);
}
// a * b in Psychopath order = glam(b) * glam(a): apply a, then b.
static inline Xf xf_mul(const Xf &a, const Xf &b) {
    // L = b, R = a; result = L.matrix3 * R.matrix3, t = L.matrix3 * R.t + L.t
    const real *L = b.m, *R = a.m;
    Xf o;
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++)
            o.m[r * 4 + c] = (L[r * 4 + 0] * R[0 * 4 + c] + L[r * 4 + 1] * R[1 * 4 + c]) + L[r * 4 + 2] * R[2 * 4 + c];
        o.m[r * 4 + 3] = ((L[r * 4 + 0] * R[3] + L[r * 4 + 1] * R[7]) + L[r * 4 + 2] * R[11]) + L[r * 4 + 3];
    }
    return o;
}
// Transform lerp: (a * (1 - alpha)) + (b * alpha), element-wise.
static inline Xf xf_lerp(const Xf &a, const Xf &b, real alpha) {
    Xf o;
    real ia = 1.0f - alpha;
    for (int i = 0; i < 12; i++) o.m[i] = a.m[i] * ia + b.m[i] * alpha;
    return o;
}

// ------------------------------------------------------------------ lerp
// src/lerp.rs:20-35
static inline real lerpf(real a, real b, real alpha) { return (a * (1.0f - alpha)) + (b * alpha); }
static inline V3 lerp3(V3 a, V3 b, real alpha) {
    real ia = 1.0f - alpha;
    return (a * ia) + (b * alpha);
}
// lerp_slice index split: returns true (and the last element index) when the
// slice has one element or alpha == 1.
static inline bool lerp_slice_index(size_t n, real alpha, size_t *i1, real *alpha2) {
    if (n == 1 || alpha == 1.0f) {
        *i1 = n - 1;
        *alpha2 = 0.0f;
        return true;
    }
    real tmp = alpha * (real)(n - 1);
    size_t i = (size_t)tmp;
    *i1 = i;
    *alpha2 = tmp - (real)i;
    return false;
}
static inline real lerp_slice_f(const real *s, size_t n, real alpha) {
    size_t i; real a2;
    if (lerp_slice_index(n, alpha, &i, &a2)) return s[i];
    return lerpf(s[i], s[i + 1], a2);
}
static inline V3 lerp_slice_v3(const V3 *s, size_t n, real alpha) {
    size_t i; real a2;
    if (lerp_slice_index(n, alpha, &i, &a2)) return s[i];
    return lerp3(s[i], s[i + 1], a2);
}
static inline Xf lerp_slice_xf(const Xf *s, size_t n, real alpha) {
    size_t i; real a2;
    if (lerp_slice_index(n, alpha, &i, &a2)) return s[i];
    return xf_lerp(s[i], s[i + 1], a2);
}

// ------------------------------------------------------------------ hashes
// src/hash.rs:1-29
static inline uint32_t hash_u32(uint32_t n, uint32_t seed) {
    uint32_t h = n;
    for (int i = 0; i < 3; i++) {
        h = h * 0x736caf6fu;
        h ^= h >> 16;
        h ^= seed;
    }
    return h;
}
static inline uint64_t hash_u64(uint64_t n, uint64_t seed) {
    uint64_t h = n;
    const uint64_t k = 32416190071ull * 314604959ull;
    for (int i = 0; i < 4; i++) {
        h = h * k;
        h ^= h >> 32;
        h ^= seed;
    }
    return h;
}
static inline float hash_u32_to_f32(uint32_t n, uint32_t seed) {
    const float inv_max = 1.0f / (float)4294967295u;
    return (float)hash_u32(n, seed) * inv_max;
}

// ------------------------------------------------------------------ floats helpers
// src/fp_utils.rs:9-43
// Unit roundoff of the arithmetic type (f32::EPSILON * 0.5 in the reference).
#ifdef PSYO_F64
static const real REAL_EPS_HALF = 2.220446049250313e-16 * 0.5;
#else
static const real REAL_EPS_HALF = 1.1920929e-07f * 0.5f;
#endif
static inline real fp_gamma(uint32_t n) {
    const real e = REAL_EPS_HALF;
    return (e * (real)n) / (1.0f - (e * (real)n));
}
static inline float increment_ulp(float v) {
    if (std::isfinite(v)) {
        if (v > 0.0f) return u2f(f2u(v) + 1);
        if (v < -0.0f) return u2f(f2u(v) - 1);
        return u2f(0x00000001u);
    }
    return v;
}
static inline float decrement_ulp(float v) {
    if (std::isfinite(v)) {
        if (v > 0.0f) return u2f(f2u(v) - 1);
        if (v < -0.0f) return u2f(f2u(v) + 1);
        return u2f(0x80000001u);
    }
    return v;
}
// The same steps on f64 bits (FP64 oracle).
static inline double increment_ulp(double v) {
    if (std::isfinite(v)) {
        if (v > 0.0) return u2d(d2u(v) + 1);
        if (v < -0.0) return u2d(d2u(v) - 1);
        return u2d(0x0000000000000001ull);
    }
    return v;
}
static inline double decrement_ulp(double v) {
    if (std::isfinite(v)) {
        if (v > 0.0) return u2d(d2u(v) - 1);
        if (v < -0.0) return u2d(d2u(v) + 1);
        return u2d(0x8000000000000001ull);
    }
    return v;
}
// src/fp_utils.rs:45-82
static inline V3 robust_ray_origin(V3 pos, real pos_err, V3 nor, V3 ray_dir) {
    V3 n = (dot(nor, ray_dir) >= 0.0f) ? nor : neg(nor);
    real d = dot(vabs(n), v3(pos_err, pos_err, pos_err));
    V3 p = pos + n * d;
    real x = (n.x >= 0.0f) ? increment_ulp(p.x) : decrement_ulp(p.x);
    real y = (n.y >= 0.0f) ? increment_ulp(p.y) : decrement_ulp(p.y);
    real z = (n.z >= 0.0f) ? increment_ulp(p.z) : decrement_ulp(p.z);
    return v3(x, y, z);
}

// src/mis.rs:12-21
static inline real power_heuristic(real a, real b) {
    if (std::isinf(a)) return a;
    real a2 = a * a, b2 = b * b;
    real mis_fac = a2 / (a2 + b2);
    return a / mis_fac;
}

// src/math.rs:67-132 (Acklam's probit approximation, evaluated in f64)
static inline real probit(float nf, real width) {
    double n = (double)nf;
    const double A1 = -3.969683028665376e+01, A2 = 2.209460984245205e+02, A3 = -2.759285104469687e+02,
                 A4 = 1.383577518672690e+02, A5 = -3.066479806614716e+01, A6 = 2.506628277459239e+00;
    const double B1 = -5.447609879822406e+01, B2 = 1.615858368580409e+02, B3 = -1.556989798598866e+02,
                 B4 = 6.680131188771972e+01, B5 = -1.328068155288572e+01;
    const double C1 = -7.784894002430293e-03, C2 = -3.223964580411365e-01, C3 = -2.400758277161838e+00,
                 C4 = -2.549732539343734e+00, C5 = 4.374664141464968e+00, C6 = 2.938163982698783e+00;
    const double D1 = 7.784695709041462e-03, D2 = 3.224671290700398e-01, D3 = 2.445134137142996e+00,
                 D4 = 3.754408661907416e+00;
    const double N_LOW = 0.02425, N_HIGH = 1.0 - N_LOW;
    double x;
    if (0.0 < n && n < N_LOW) {
        double q = std::sqrt(-2.0 * std::log(n));
        x = (((((C1 * q + C2) * q + C3) * q + C4) * q + C5) * q + C6) / ((((D1 * q + D2) * q + D3) * q + D4) * q + 1.0);
    } else if (n <= N_HIGH) {
        double q = n - 0.5;
        double r = q * q;
        x = (((((A1 * r + A2) * r + A3) * r + A4) * r + A5) * r + A6) * q /
            (((((B1 * r + B2) * r + B3) * r + B4) * r + B5) * r + 1.0);
    } else if (n < 1.0) {
        double q = std::sqrt(-2.0 * std::log(1.0 - n));
        x = -(((((C1 * q + C2) * q + C3) * q + C4) * q + C5) * q + C6) / ((((D1 * q + D2) * q + D3) * q + D4) * q + 1.0);
    } else if (n == 0.0) {
        x = -INFINITY;
    } else if (n == 1.0) {
        x = INFINITY;
    } else {
        x = NAN;
    }
    return (real)x * width;
}

// fastapprox 0.3 `fast::exp` (src/math.rs:146-148).  Published method of
// Paul Mineiro's fastapprox library: exp(p) = pow2(p * log2(e)) with a
// rational correction of the fractional part, assembled into IEEE bits.
static inline float fast_pow2(float p) {
    float offset = (p < 0.0f) ? 1.0f : 0.0f;
    float clipp = (p < -126.0f) ? -126.0f : p;
    int w = (int)clipp;
    float z = clipp - (float)w + offset;
    float v = (float)(1 << 23) * (clipp + 121.2740575f + 27.7280233f / (4.84252568f - z) - 1.49012907f * z);
    return u2f((uint32_t)v);
}
static inline float fast_exp_f32(float p) { return fast_pow2(1.442695040f * p); }
// In the FP64 oracle the argument is rounded to f32 first: fastapprox's
// method is defined on f32 bits.
static inline real fast_exp(real p) { return (real)fast_exp_f32((float)p); }

// ------------------------------------------------------------------ sampling
// Golden ratio sampler (src/renderer.rs:728-737)
static inline float golden_ratio_sample(uint32_t i, uint32_t scramble) {
    uint32_t n = (i + hash_u32(scramble, 0)) * 2654435769u;
    return (float)n * (1.0f / (float)(1ull << 32));
}

// Owen-scrambled Sobol points by Burley's hash-based scrambling ("Practical
// Hash-based Owen Scrambling", JCGT 9(4), 2020): the index is shuffled by a
// nested uniform scramble, each dimension of the Sobol point is scrambled
// with a per-dimension seed, and the result is mapped to [0,1) with 24 bits.
// Direction numbers: Joe & Kuo (2008) for the first 8 dimensions, so two 4D
// dimension sets are Sobol and higher sets use the reference's hash fallback.
static const uint32_t PSY_SOBOL_SETS = 2;
void sobol_directions(uint32_t dirs[8][32]);
static inline uint32_t reverse_bits32(uint32_t x) {
    x = (x << 16) | (x >> 16);
    x = ((x & 0x00ff00ffu) << 8) | ((x & 0xff00ff00u) >> 8);
    x = ((x & 0x0f0f0f0fu) << 4) | ((x & 0xf0f0f0f0u) >> 4);
    x = ((x & 0x33333333u) << 2) | ((x & 0xccccccccu) >> 2);
    x = ((x & 0x55555555u) << 1) | ((x & 0xaaaaaaaau) >> 1);
    return x;
}
static inline uint32_t laine_karras_permutation(uint32_t x, uint32_t seed) {
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return x;
}
static inline uint32_t nested_uniform_scramble(uint32_t x, uint32_t seed) {
    return reverse_bits32(laine_karras_permutation(reverse_bits32(x), seed));
}
static inline uint32_t hash_combine(uint32_t seed, uint32_t v) {
    return seed ^ (v + (seed << 6) + (seed >> 2));
}
void sobol_burley_4d(uint32_t index, uint32_t set, uint32_t seed, float out[4]);

// get_sample_4d (src/renderer.rs:698-725)
static inline void get_sample_4d(uint32_t i, uint32_t set, uint32_t px, uint32_t py, uint32_t seed, float out[4]) {
    uint32_t s = px ^ (py << 16) ^ (seed * 0x736caf6fu);
    if (set < PSY_SOBOL_SETS) {
        sobol_burley_4d(i, set, s, out);
    } else {
        for (uint32_t k = 0; k < 4; k++) out[k] = hash_u32_to_f32((set * 4 + k) ^ (i << 16), s);
    }
}

}  // namespace psyo
