// Device shading of the tracing path: hero-wavelength spectra (Meng et al.
// upsampling, Planck, the Wyman CIE fit), sampling routines, Lambert / GGX /
// Emit closures and surface / distant light sampling, following
// src/color.rs, src/sampling/monte_carlo.rs, src/shading/surface_closure.rs
// and src/light/*.rs of the reference.
#pragma once

#include "dev_math.cuh"

namespace psyd {

#define PSY_PI_32 3.14159265358979323846f
#define PSY_PI_64 3.14159265358979323846
#define PSY_INV_PI (1.0f / PSY_PI_32)
#define PSY_H_PI (PSY_PI_32 / 2.0f)
#define PSY_QPI_32 0.785398163397448309616f

// ------------------------------------------------------------------ wavelengths
#define PSY_WL_MIN 380.0f
#define PSY_WL_MAX 700.0f
#define PSY_WL_RANGE (PSY_WL_MAX - PSY_WL_MIN)
#define PSY_WL_RANGE_Q (PSY_WL_RANGE / 4.0f)
DI float map_0_1_to_wavelength(float n) { return n * PSY_WL_RANGE + PSY_WL_MIN; }
DI float nth_wavelength(float hero, int n) {
    float wl = hero + (PSY_WL_RANGE_Q * (float)n);
    return (wl > PSY_WL_MAX) ? wl - PSY_WL_RANGE : wl;
}

// ------------------------------------------------------------------ Meng upsampling
DI V4 spectrum_xyz_to_p_4(V4 lambdas, float X, float Y, float Z) {
    float inv_norm = X + Y + Z;
    float norm = 1.0f / inv_norm;
    if (!(norm < 3.40282347e+38f)) return splat4(0.0f);
    float xx = X * norm, yy = Y * norm;
    const float *M = psy_meng_xy_to_uv;
    float u = M[0] * xx + M[1] * yy + M[2];
    float v = M[3] * xx + M[4] * yy + M[5];
    if (u < 0.0f || u >= (float)PSY_MENG_GRID_WIDTH || v < 0.0f || v >= (float)PSY_MENG_GRID_HEIGHT) return splat4(0.0f);
    int ui = (int)u, vi = (int)v;
    const int *cell = psy_meng_grid[ui + PSY_MENG_GRID_WIDTH * vi];
    int inside = cell[0], num = cell[1];
    const int *idx = cell + 2;
    if (num == 0) return splat4(0.0f);
    V4 sb;
    int sb0[4], sb1[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        sb[k] = (lambdas[k] - PSY_MENG_SAMPLE_MIN) / (PSY_MENG_SAMPLE_MAX - PSY_MENG_SAMPLE_MIN) *
                ((float)PSY_MENG_NUM_SAMPLES - 1.0f);
        sb0[k] = (int)sb[k];
        int t = sb0[k] + 1;
        sb1[k] = t < PSY_MENG_NUM_SAMPLES - 1 ? t : PSY_MENG_NUM_SAMPLES - 1;
    }
    V4 sbf = sb - v4((float)sb0[0], (float)sb0[1], (float)sb0[2], (float)sb0[3]);
    // the spectrum of cell point k at the four wavelengths (the reference
    // computes it for every point of the cell first; only the ones combined
    // below are needed, and each is the same expression)
    auto point = [&](int k) -> V4 {
        const float *spec = psy_meng_point_spectrum[idx[k]];
        V4 p0 = v4(spec[sb0[0]], spec[sb0[1]], spec[sb0[2]], spec[sb0[3]]);
        V4 p1 = v4(spec[sb1[0]], spec[sb1[1]], spec[sb1[2]], spec[sb1[3]]);
        return p0 * (splat4(1.0f) - sbf) + p1 * sbf;
    };
    V4 ip = splat4(0.0f);
    if (inside) {
        float u2 = u - (float)ui, v2 = v - (float)vi;
        ip = point(0) * ((1.0f - u2) * (1.0f - v2)) + point(2) * ((1.0f - u2) * v2) + point(3) * (u2 * v2) +
             point(1) * (u2 * (1.0f - v2));
    } else {
        // the fan triangle (0, i + 1, i + 2) -- the last one closing on
        // point 1 -- that holds (u, v); barycentrics from the uv points only
        const float *uv0 = psy_meng_point_uv[idx[0]];
        const float *uv1 = psy_meng_point_uv[idx[1]];
        float ex = u - uv0[0], ey = v - uv0[1];
        float e0x = uv1[0] - uv0[0], e0y = uv1[1] - uv0[1];
        float uu = e0x * ey - ex * e0y;
        for (int i = 0; i < num - 1; i++) {
            float e1x, e1y;
            if (i == num - 2) {
                e1x = uv1[0] - uv0[0];
                e1y = uv1[1] - uv0[1];
            } else {
                const float *uvn = psy_meng_point_uv[idx[i + 2]];
                e1x = uvn[0] - uv0[0];
                e1y = uvn[1] - uv0[1];
            }
            float vv = ex * e1y - e1x * ey;
            float area = e0x * e1y - e1x * e0y;
            float fu = uu / area, fv = vv / area;
            float fw = 1.0f - fu - fv;
            if (fu < 0.0f || fv < 0.0f || fw < 0.0f) {
                uu = -vv;
                e0x = e1x;
                e0y = e1y;
                continue;
            }
            ip = point(0) * fw + point(i + 1) * fv + point((i == num - 2) ? 1 : i + 2) * fu;
            break;
        }
    }
    return ip * inv_norm;
}

// Meng upsampling of a constant colour at sample s of the point spectra:
// the weighted point spectra of spectrum_xyz_to_p_4 at one sample instead
// of lerped at four wavelengths, times 1 / the equal-energy reflectance.
// Tabulated for every sample, it gives the colour's spectrum at any
// wavelength as one lerp between two table entries: the same value up to
// the order of the lerp and the weighted sum (rounding only).
DI float meng_table_value(float X, float Y, float Z, int s) {
    float inv_norm = X + Y + Z;
    float norm = 1.0f / inv_norm;
    if (!(norm < 3.40282347e+38f)) return 0.0f;
    float xx = X * norm, yy = Y * norm;
    const float *M = psy_meng_xy_to_uv;
    float u = M[0] * xx + M[1] * yy + M[2];
    float v = M[3] * xx + M[4] * yy + M[5];
    if (u < 0.0f || u >= (float)PSY_MENG_GRID_WIDTH || v < 0.0f || v >= (float)PSY_MENG_GRID_HEIGHT) return 0.0f;
    int ui = (int)u, vi = (int)v;
    const int *cell = psy_meng_grid[ui + PSY_MENG_GRID_WIDTH * vi];
    int inside = cell[0], num = cell[1];
    const int *idx = cell + 2;
    if (num == 0) return 0.0f;
    auto sp = [&](int k) { return psy_meng_point_spectrum[idx[k]][s]; };
    float r = 0.0f;
    if (inside) {
        float u2 = u - (float)ui, v2 = v - (float)vi;
        r = sp(0) * ((1.0f - u2) * (1.0f - v2)) + sp(2) * ((1.0f - u2) * v2) + sp(3) * (u2 * v2) +
            sp(1) * (u2 * (1.0f - v2));
    } else {
        const float *uv0 = psy_meng_point_uv[idx[0]];
        const float *uv1 = psy_meng_point_uv[idx[1]];
        float ex = u - uv0[0], ey = v - uv0[1];
        float e0x = uv1[0] - uv0[0], e0y = uv1[1] - uv0[1];
        float uu = e0x * ey - ex * e0y;
        for (int i = 0; i < num - 1; i++) {
            float e1x, e1y;
            if (i == num - 2) {
                e1x = uv1[0] - uv0[0];
                e1y = uv1[1] - uv0[1];
            } else {
                const float *uvn = psy_meng_point_uv[idx[i + 2]];
                e1x = uvn[0] - uv0[0];
                e1y = uvn[1] - uv0[1];
            }
            float vv = ex * e1y - e1x * ey;
            float area = e0x * e1y - e1x * e0y;
            float fu = uu / area, fv = vv / area;
            float fw = 1.0f - fu - fv;
            if (fu < 0.0f || fv < 0.0f || fw < 0.0f) {
                uu = -vv;
                e0x = e1x;
                e0y = e1y;
                continue;
            }
            r = sp(0) * fw + sp(i + 1) * fv + sp((i == num - 2) ? 1 : i + 2) * fu;
            break;
        }
    }
    return r * inv_norm * (1.0f / PSY_MENG_EQUAL_ENERGY_REFLECTANCE);
}

// ------------------------------------------------------------------ colour
// (a scaled or lerped colour is a new value: its spectrum-table index is dropped)
DI GColor color_mul(GColor c, float s) {
    uint32_t kind = c.kind & PSY_COLOR_KIND_MASK;
    if (kind == PSY_COLOR_XYZ_K) return GColor{kind, c.a * s, c.b * s, c.c * s};
    return GColor{kind, c.a, c.b * s, c.c};
}
DI GColor color_lerp(GColor x, GColor y, float alpha) {
    float ia = 1.0f - alpha;
    uint32_t kind = x.kind & PSY_COLOR_KIND_MASK;
    if (kind == PSY_COLOR_XYZ_K)
        return GColor{kind, (x.a * ia) + (y.a * alpha), (x.b * ia) + (y.b * alpha), (x.c * ia) + (y.c * alpha)};
    return GColor{kind, (x.a * ia) + (y.a * alpha), (x.b * ia) + (y.b * alpha), 0.0f};
}
DI GColor lerp_slice_color(const GColor *s, uint32_t n, float alpha) {
    uint32_t i; float a2;
    if (lerp_index(n, alpha, &i, &a2)) return s[i];
    return color_lerp(s[i], s[i + 1], a2);
}
DI float plancks_law(float temperature, float wavelength) {
    const float C = 299792458.0f, H = 6.62607015e-34f, KB = 1.38064852e-23f;
    if (temperature < 200.0f) return 0.0f;
    float wl = wavelength * 1.0e-9f;
    const float TMP1 = (float)(2.0 * (double)H * (double)C * (double)C);
    const float TMP2 = (float)((double)H * (double)C / (double)KB);
    float wl2 = wl * wl;
    float wl5 = wl2 * wl2 * wl;
    float tmp3 = wl5 * (fast_exp(TMP2 / (wl * temperature)) - 1.0f);
    float energy = TMP1 / tmp3;
    return rmax(energy * 1.0e-6f, 0.0f);
}
DI V4 color_to_spectral(GColor c, float hero) {
    V4 wls = v4(nth_wavelength(hero, 0), nth_wavelength(hero, 1), nth_wavelength(hero, 2), nth_wavelength(hero, 3));
    const uint32_t kind = c.kind & PSY_COLOR_KIND_MASK;
    if (kind == PSY_COLOR_XYZ_K)
        return spectrum_xyz_to_p_4(wls, c.a, c.b, c.c) * (1.0f / PSY_MENG_EQUAL_ENERGY_REFLECTANCE);
    V4 o;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float pl = plancks_law(c.a, wls[k]);
        if (kind != PSY_COLOR_BLACKBODY_K) {
            float t2 = c.a * c.a;
            pl = pl * 4.0e7f / (t2 * t2);
        }
        o[k] = pl * c.b;
    }
    return o;
}
// A colour's spectrum at the four wavelengths of `hero` from its table
// (the lerp spectrum_xyz_to_p_4 makes between two point-spectrum samples,
// applied to the combined table).
DI V4 spectrum_from_table(const float *C, float hero) {
    V4 o;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float sb = (nth_wavelength(hero, k) - PSY_MENG_SAMPLE_MIN) / (PSY_MENG_SAMPLE_MAX - PSY_MENG_SAMPLE_MIN) *
                   ((float)PSY_MENG_NUM_SAMPLES - 1.0f);
        int s0 = (int)sb;
        int s1 = s0 + 1 < PSY_MENG_NUM_SAMPLES - 1 ? s0 + 1 : PSY_MENG_NUM_SAMPLES - 1;
        float f = sb - (float)s0;
        o[k] = __ldg(C + s0) * (1.0f - f) + __ldg(C + s1) * f;
    }
    return o;
}
// The spectrum of a colour in the shading arithmetic R: the f32 form takes
// a tabulated colour's spectrum from its table; the f64 form (the
// reference's arithmetic) and colours without a table run the upsampling.
template <class R>
DI V4 color_spectrum(const GScene &S, GColor c, float hero) {
    const uint32_t t = c.kind >> 16;
    if (sizeof(R) == sizeof(float) && t != 0u) return spectrum_from_table(S.spec_tables + PSY_SPEC_TABLE * (t - 1u), hero);
    return color_to_spectral(c, hero);
}
DI float x_1931(float w) {
    float t1 = (w - 442.0f) * ((w < 442.0f) ? 0.0624f : 0.0374f);
    float t2 = (w - 599.8f) * ((w < 599.8f) ? 0.0264f : 0.0323f);
    float t3 = (w - 501.1f) * ((w < 501.1f) ? 0.0490f : 0.0382f);
    return (0.362f * fast_exp(-0.5f * t1 * t1)) + (1.056f * fast_exp(-0.5f * t2 * t2)) - (0.065f * fast_exp(-0.5f * t3 * t3));
}
DI float y_1931(float w) {
    float t1 = (w - 568.8f) * ((w < 568.8f) ? 0.0213f : 0.0247f);
    float t2 = (w - 530.9f) * ((w < 530.9f) ? 0.0613f : 0.0322f);
    return (0.821f * fast_exp(-0.5f * t1 * t1)) + (0.286f * fast_exp(-0.5f * t2 * t2));
}
DI float z_1931(float w) {
    float t1 = (w - 437.0f) * ((w < 437.0f) ? 0.0845f : 0.0278f);
    float t2 = (w - 459.0f) * ((w < 459.0f) ? 0.0385f : 0.0725f);
    return (1.217f * fast_exp(-0.5f * t1 * t1)) + (0.681f * fast_exp(-0.5f * t2 * t2));
}
DI V3 xyz_from_spectral(V4 e, float hero) {
    V3 acc = v3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float wl = nth_wavelength(hero, k);
        V3 c = v3(x_1931(wl) * e[k], y_1931(wl) * e[k], z_1931(wl) * e[k]);
        acc = (k == 0) ? c : acc + c;
    }
    return acc * 0.75f;
}

// ------------------------------------------------------------------ precision helpers
// The reference evaluates light / cone / spherical-triangle sampling and the
// pixel filter in f64.  Those routines are templated on the real type R:
// R = double is the reference's arithmetic (the plain form); R = float is
// the precision variant (no FP64 outside the watertight triangle retest),
// whose image error against the f64 oracle is measured, not assumed.
DI double msqrt(double x) { return sqrt(x); }
DI float msqrt(float x) { return sqrtf(x); }
DI double macos(double x) { return acos(x); }
DI float macos(float x) { return acosf(x); }
DI double msin(double x) { return sin(x); }
DI float msin(float x) { return sinf(x); }
DI double mcos(double x) { return cos(x); }
DI float mcos(float x) { return cosf(x); }
DI double mlog(double x) { return log(x); }
DI float mlog(float x) { return logf(x); }
DI double mfmin(double a, double b) { return fmin(a, b); }
DI float mfmin(float a, float b) { return fminf(a, b); }
DI double mfmax(double a, double b) { return fmax(a, b); }
DI float mfmax(float a, float b) { return fmaxf(a, b); }
// sin / cos of (v * 2 pi): sincospi of 2v (exact argument), equal to the
// reference's cos(v * 2.0 * PI) up to the rounding of the product.
DI void msincos_2pi(double v, double *s, double *c) { sincospi(v * 2.0, s, c); }
DI void msincos_2pi(float v, float *s, float *c) { sincospif(v * 2.0f, s, c); }
template <class R>
DI R pi_r() { return (R)PSY_PI_64; }

// ------------------------------------------------------------------ sampling
DI void square_to_circle(float x, float y, float *ox, float *oy) {
    if (x == 0.0f && y == 0.0f) { *ox = 0.0f; *oy = 0.0f; return; }
    float radius, angle;
    if (x > fabsf(y)) { radius = x; angle = PSY_QPI_32 * (y / x); }
    else if (y > fabsf(x)) { radius = y; angle = PSY_QPI_32 * (2.0f - (x / y)); }
    else if (x < -fabsf(y)) { radius = -x; angle = PSY_QPI_32 * (4.0f + (y / x)); }
    else { radius = -y; angle = PSY_QPI_32 * (6.0f - (x / y)); }
    *ox = radius * cosf(angle);
    *oy = radius * sinf(angle);
}
DI V3 cosine_sample_hemisphere(float u, float v) {
    float cu, cv;
    square_to_circle((u * 2.0f) - 1.0f, (v * 2.0f) - 1.0f, &cu, &cv);
    float z = sqrtf(rmax(1.0f - ((cu * cu) + (cv * cv)), 0.0f));
    return v3(cu, cv, z);
}
DI V3 uniform_sample_sphere(float u, float v) {
    float z = 1.0f - (2.0f * u);
    float r = sqrtf(rmax(1.0f - (z * z), 0.0f));
    float phi = 2.0f * PSY_PI_32 * v;
    return v3(r * cosf(phi), r * sinf(phi), z);
}
template <class R>
DI V3 uniform_sample_cone(float u, float v, R cos_theta_max) {
    R cos_theta = ((R)1 - (R)u) + ((R)u * cos_theta_max);
    R sin_theta = msqrt((R)1 - (cos_theta * cos_theta));
    R sp, cp;
    msincos_2pi((R)v, &sp, &cp);
    return v3((float)(cp * sin_theta), (float)(sp * sin_theta), (float)cos_theta);
}
template <class R>
DI R uniform_sample_cone_pdf(R ctm) { return (R)1 / ((R)2 * pi_r<R>() * ((R)1 - ctm)); }
// Cone pdf from sin^2 of the cone's half angle (st2) and its cosine (ctm)
// for the f32 shading variant: 1 - ctm = st2 / (1 + ctm) exactly, which
// keeps the pdf finite where 1 - st2 rounds to 1 in f32 (a small, distant
// sphere light).  The f64 form evaluates the reference's expression.
template <class R>
DI R cone_pdf_st2(R st2, R ctm) {
    if (sizeof(R) == sizeof(double)) return uniform_sample_cone_pdf<R>(ctm);
    return ((R)1 + ctm) / ((R)2 * pi_r<R>() * st2);
}
DI V3 uniform_sample_triangle(V3 va, V3 vb, V3 vc, float i, float j) {
    float isqrt = sqrtf(i);
    float a = 1.0f - isqrt;
    float b = isqrt * (1.0f - j);
    float c = j * isqrt;
    return (va * a) + (vb * b) + (vc * c);
}
DI float triangle_surface_area(V3 p0, V3 p1, V3 p2) { return 0.5f * length(cross(p1 - p0, p2 - p0)); }
template <class R>
DI R clamp1(R x) { return mfmin(mfmax(x, (R)-1), (R)1); }
template <class R>
DI float spherical_triangle_solid_angle(V3 va, V3 vb, V3 vc) {
    R cos_a = (R)rmin(rmax(dot(vb, vc), -1.0f), 1.0f);
    R cos_b = (R)rmin(rmax(dot(vc, va), -1.0f), 1.0f);
    R cos_c = (R)rmin(rmax(dot(va, vb), -1.0f), 1.0f);
    R sin_a = msqrt((R)1 - (cos_a * cos_a));
    R sin_b = msqrt((R)1 - (cos_b * cos_b));
    R sin_c = msqrt((R)1 - (cos_c * cos_c));
    if (cos_a == (R)1 || cos_b == (R)1 || cos_c == (R)1) return 0.0f;
    R cos_va = clamp1((cos_a - (cos_b * cos_c)) / (sin_b * sin_c));
    R cos_vb = clamp1((cos_b - (cos_c * cos_a)) / (sin_c * sin_a));
    R cos_vc = clamp1((cos_c - (cos_a * cos_b)) / (sin_a * sin_b));
    return (float)(macos(cos_va) + macos(cos_vb) + macos(cos_vc) - pi_r<R>());
}
template <class R>
DI V3 uniform_sample_spherical_triangle(V3 va, V3 vb, V3 vc, float i, float j) {
    R cos_a = (R)rmin(rmax(dot(vb, vc), -1.0f), 1.0f);
    R cos_b = (R)rmin(rmax(dot(vc, va), -1.0f), 1.0f);
    R cos_c = (R)rmin(rmax(dot(va, vb), -1.0f), 1.0f);
    R sin_a = msqrt((R)1 - (cos_a * cos_a));
    R sin_b = msqrt((R)1 - (cos_b * cos_b));
    R sin_c = msqrt((R)1 - (cos_c * cos_c));
    if (cos_a == (R)1 || cos_b == (R)1 || cos_c == (R)1) return va;
    R cos_va = clamp1((cos_a - (cos_b * cos_c)) / (sin_b * sin_c));
    R cos_vb = clamp1((cos_b - (cos_c * cos_a)) / (sin_c * sin_a));
    R cos_vc = clamp1((cos_c - (cos_a * cos_b)) / (sin_a * sin_b));
    R sin_va = msqrt((R)1 - (cos_va * cos_va));
    R ang_va = macos(cos_va), ang_vb = macos(cos_vb), ang_vc = macos(cos_vc);
    R area = ang_va + ang_vb + ang_vc - pi_r<R>();
    R area_2 = area * (R)i;
    R s = msin(area_2 - ang_va);
    R t = mcos(area_2 - ang_va);
    R u = t - cos_va;
    R v = s + (sin_va * cos_c);
    R q_top = (((v * t) - (u * s)) * cos_va) - v;
    R q_bottom = ((v * s) + (u * t)) * sin_va;
    R q = q_top / q_bottom;
    V3 vc_2 = (va * (float)q) + (normalized(vc - (va * dot(vc, va))) * (float)msqrt((R)1 - (q * q)));
    float z = 1.0f - (j * (1.0f - dot(vc_2, vb)));
    return (vb * z) + (normalized(vc_2 - (vb * dot(vc_2, vb))) * sqrtf(1.0f - (z * z)));
}
DI void coordinate_system_from_vector(V3 v, V3 *o1, V3 *o2, V3 *o3) {
    float sign = signum(v.z);
    float a = -1.0f / (sign + v.z);
    float b = v.x * v.y * a;
    *o1 = v;
    *o2 = v3(1.0f + sign * v.x * v.x * a, sign * b, -sign * v.x);
    *o3 = v3(b, sign + v.y * v.y * a, -v.y);
}
DI V3 zup_to_vec(V3 from, V3 toz) {
    V3 z, x, y;
    coordinate_system_from_vector(normalized(toz), &z, &x, &y);
    return (x * from.x) + (y * from.y) + (z * from.z);
}

// ------------------------------------------------------------------ closures
#define PSY_CL_LAMBERT 0u
#define PSY_CL_GGX 1u
#define PSY_CL_EMIT 2u
struct Closure {
    uint32_t kind;
    GColor color;
    float roughness, fresnel;
};
DI Closure closure_from_shader(const GShader &s) {
    Closure c;
    c.kind = s.kind == 0u ? PSY_CL_EMIT : (s.kind == 1u ? PSY_CL_LAMBERT : PSY_CL_GGX);
    c.color = s.color;
    c.roughness = s.roughness;
    c.fresnel = s.fresnel;
    return c;
}
DI void flip_normals(V3 inc, V3 nor, V3 nor_g, V3 *nn, V3 *fng) {
    if (dot(nor_g, inc) <= 0.0f) { *nn = normalized(nor); *fng = nor_g; }
    else { *nn = neg(normalized(nor)); *fng = neg(nor_g); }
}
DI float schlick_fresnel_from_fac(float f, float c) {
    float c1 = 1.0f - c;
    float c2 = c1 * c1;
    return f + ((1.0f - f) * c1 * c2 * c2);
}
DI float ggx_d(float nh, float rough) {
    if (nh <= 0.0f) return 0.0f;
    float r2 = rough * rough;
    float tmp = 1.0f + ((r2 - 1.0f) * (nh * nh));
    return r2 / (PSY_PI_32 * tmp * tmp);
}
DI float ggx_g(float vh, float vn, float rough) {
    if ((vh * vn) <= 0.0f) return 0.0f;
    return 2.0f / (1.0f + sqrtf(1.0f + rough * rough * (1.0f - vn * vn) / (vn * vn)));
}
// spec: the closure colour's spectrum at the path's wavelengths,
// color_to_spectral(cl.color, wl), computed once per shading point by the
// caller (the light sample's evaluation and the bounce sample use the same
// value, as the reference computes it in each).
DI V4 closure_evaluate(const Closure &cl, V4 spec, V3 inc, V3 out, V3 nor, V3 nor_g, float *pdf) {
    if (cl.kind == PSY_CL_EMIT) { *pdf = 1.0f; return spec; }
    V3 nn, fng;
    if (cl.kind == PSY_CL_LAMBERT) {
        flip_normals(inc, nor, nor_g, &nn, &fng);
        if (dot(fng, out) >= 0.0f) {
            float fac = rmax(dot(nn, normalized(out)), 0.0f) * PSY_INV_PI;
            *pdf = fac;
            return spec * fac;
        }
        *pdf = 0.0f;
        return splat4(0.0f);
    }
    V3 aa = neg(normalized(inc));
    V3 bb = normalized(out);
    V3 hh = normalized(aa + bb);
    flip_normals(inc, nor, nor_g, &nn, &fng);
    if (dot(nn, aa) < 0.0f || dot(nn, bb) < 0.0f || dot(fng, bb) < 0.0f) { *pdf = 0.0f; return splat4(0.0f); }
    float na = rclamp(dot(nn, aa), -1.0f, 1.0f);
    float nb = rclamp(dot(nn, bb), -1.0f, 1.0f);
    float ha = rclamp(dot(hh, aa), -1.0f, 1.0f);
    float hb = rclamp(dot(hh, bb), -1.0f, 1.0f);
    float nh = rclamp(dot(nn, hh), -1.0f, 1.0f);
    V4 ss = spec;
    float rev = 1.0f - cl.fresnel;
    V4 col_f;
#pragma unroll
    for (int k = 0; k < 4; k++) col_f[k] = lerpf(schlick_fresnel_from_fac(ss[k], hb), ss[k], rev);
    if (cl.roughness == 0.0f) { *pdf = 0.0f; return col_f; }
    float dist = ggx_d(nh, cl.roughness) / na;
    float g1 = ggx_g(ha, na, cl.roughness);
    float g2 = ggx_g(hb, nb, cl.roughness);
    *pdf = dist * PSY_INV_PI;
    return col_f * (dist * g1 * g2) * PSY_INV_PI;
}
DI V4 closure_sample(const Closure &cl, V4 spec, V3 inc, V3 nor, V3 nor_g, float u, float v, V3 *out, float *pdf) {
    if (cl.kind == PSY_CL_EMIT) { *out = v3(0.0f, 0.0f, 0.0f); *pdf = 1.0f; return spec; }
    V3 nn, fng;
    flip_normals(inc, nor, nor_g, &nn, &fng);
    if (cl.kind == PSY_CL_LAMBERT) {
        V3 dir = cosine_sample_hemisphere(u, v);
        float p = dir.z * PSY_INV_PI;
        V3 o = zup_to_vec(dir, nn);
        *out = o;
        if (dot(fng, o) >= 0.0f) { *pdf = p; return spec * p; }
        *pdf = 0.0f;
        return splat4(0.0f);
    }
    float r2 = cl.roughness * cl.roughness;
    float theta_cos = sqrtf((1.0f - u) / (1.0f + ((r2 - 1.0f) * u)));
    float theta_sin = sqrtf(1.0f - (theta_cos * theta_cos));
    float angle = v * PSY_PI_32 * 2.0f;
    V3 half_dir = v3(cosf(angle) * theta_sin, sinf(angle) * theta_sin, theta_cos);
    half_dir = normalized(zup_to_vec(half_dir, nn));
    V3 o = inc - (half_dir * 2.0f * dot(inc, half_dir));
    *out = o;
    if (dot(fng, o) >= 0.0f) return closure_evaluate(cl, spec, inc, o, nor, nor_g, pdf);
    *pdf = 0.0f;
    return splat4(0.0f);
}
// (g and h are evaluated only past the first case -- a light entirely
// above the horizon, the common one -- with the same expressions)
DI float sphere_lambert(float nlcos, float rcos) {
    float rsin2 = 1.0f - (rcos * rcos);
    float nl = acosf(nlcos);
    float r = acosf(rcos);
    if (nl < (PSY_H_PI - r)) return nlcos * rsin2;
    if (!(nl < PSY_H_PI) && !(nl < (PSY_H_PI + r))) return 0.0f;  // the last case, NaN included
    float nlsin = sqrtf(1.0f - (nlcos * nlcos));
    float rsin = sqrtf(rsin2);
    float ysin = rcos / nlsin;
    float ycos2 = 1.0f - (ysin * ysin);
    float ycos = sqrtf(ycos2);
    float g = (-2.0f * nlsin * rcos * ycos) + PSY_H_PI - asinf(ysin) + (ysin * ycos);
    float h = nlcos * ((ycos * sqrtf(rsin2 - ycos2)) + (rsin2 * asinf(ycos / rsin)));
    if (nl < PSY_H_PI) return (nlcos * rsin2) + g - h;
    return (g + h) * PSY_INV_PI;
}
DI float closure_estimate_sphere(const Closure &cl, V3 inc, V3 to_light, float r2l, V3 nor, V3 nor_g) {
    if (cl.kind == PSY_CL_LAMBERT) {
        float dist2 = length2(to_light);
        if (dist2 <= r2l) return rmin(r2l / dist2, 4.0f);
        float stm2 = rmin(r2l / dist2, 1.0f);
        float ctm = sqrtf(1.0f - stm2);
        V3 v = normalized(to_light);
        V3 nn = (dot(nor_g, inc) <= 0.0f) ? normalized(nor) : neg(normalized(nor));
        float cos_nv = rmin(rmax(dot(nn, v), -1.0f), 1.0f);
        return sphere_lambert(cos_nv, ctm);
    }
    if (cl.kind == PSY_CL_GGX) {
        float dist2 = length2(to_light);
        float stm2 = rmin(r2l / dist2, 1.0f);
        float ctm = sqrtf(1.0f - stm2);
        V3 nn = (dot(nor, inc) < 0.0f) ? normalized(nor) : neg(normalized(nor));
        V3 aa = neg(normalized(inc));
        V3 bb = normalized(to_light);
        float theta = acosf(ctm);
        V3 hh = normalized(aa + bb);
        float nh = rclamp(dot(nn, hh), -1.0f, 1.0f);
        float fac = ggx_d(nh, rmin(1.0f, sqrtf(cl.roughness) + (2.0f * theta / PSY_PI_32)));
        return fac * rmin(1.0f, 1.0f - ctm) * PSY_INV_PI;
    }
    return 0.0f;
}

}  // namespace psyd
