// Oracle (test infrastructure only): colour, spectral upsampling, sampling
// routines and surface closures of Psychopath, restated for the CPU.
#pragma once

#include "oracle_math.h"

#define PSY_MENG_CONST static const
#include "../psychopath_gb300/csrc/spectra_tables.inc"

namespace psyo {

static const real PI_32 = 3.14159265358979323846f;
static const double PI_64 = 3.14159265358979323846;
static const real INV_PI = 1.0f / PI_32;
static const real H_PI = PI_32 / 2.0f;
static const real QPI_32 = 0.785398163397448309616f;  // FRAC_PI_4

// ------------------------------------------------------------------ wavelengths
// src/color.rs:14-43
static const real WL_MIN = 380.0f, WL_MAX = 700.0f;
static const real WL_RANGE = WL_MAX - WL_MIN;
static const real WL_RANGE_Q = WL_RANGE / 4.0f;
static inline real map_0_1_to_wavelength(real n) { return n * WL_RANGE + WL_MIN; }
static inline real nth_wavelength(real hero, int n) {
    real wl = hero + (WL_RANGE_Q * (real)n);
    return (wl > WL_MAX) ? wl - WL_RANGE : wl;
}
static inline V4 wavelengths(real hero) {
    return v4(nth_wavelength(hero, 0), nth_wavelength(hero, 1), nth_wavelength(hero, 2), nth_wavelength(hero, 3));
}

// ------------------------------------------------------------------ Meng upsampling
// sub_crates/spectral_upsampling/src/meng.rs:177-328
static inline V4 spectrum_xyz_to_p_4(V4 lambdas, real X, real Y, real Z) {
    real inv_norm = X + Y + Z;
    real norm = 1.0f / inv_norm;
    if (!(norm < 3.40282347e+38f)) return splat4(0.0f);
    real xx = X * norm, yy = Y * norm;
    const float *M = psy_meng_xy_to_uv;
    real u = M[0] * xx + M[1] * yy + M[2];
    real v = M[3] * xx + M[4] * yy + M[5];
    if (u < 0.0f || u >= (real)PSY_MENG_GRID_WIDTH || v < 0.0f || v >= (real)PSY_MENG_GRID_HEIGHT)
        return splat4(0.0f);
    int ui = (int)u, vi = (int)v;
    int cell_idx = ui + PSY_MENG_GRID_WIDTH * vi;
    const int *cell = psy_meng_grid[cell_idx];
    int inside = cell[0], num = cell[1];
    const int *idx = cell + 2;
    if (num == 0) return splat4(0.0f);
    // sb = (lambda - min) / (max - min) * (N - 1)
    V4 sb = (lambdas - splat4(PSY_MENG_SAMPLE_MIN)) / splat4(PSY_MENG_SAMPLE_MAX - PSY_MENG_SAMPLE_MIN) *
            splat4((real)PSY_MENG_NUM_SAMPLES - 1.0f);
    int sb0[4], sb1[4];
    for (int k = 0; k < 4; k++) {
        sb0[k] = (int)sb[k];
        int t = sb0[k] + 1;
        sb1[k] = t < PSY_MENG_NUM_SAMPLES - 1 ? t : PSY_MENG_NUM_SAMPLES - 1;
    }
    V4 sbf = sb - v4((real)sb0[0], (real)sb0[1], (real)sb0[2], (real)sb0[3]);
    V4 p[6];
    for (int i = 0; i < num; i++) {
        const float *spec = psy_meng_point_spectrum[idx[i]];
        V4 p0 = v4(spec[sb0[0]], spec[sb0[1]], spec[sb0[2]], spec[sb0[3]]);
        V4 p1 = v4(spec[sb1[0]], spec[sb1[1]], spec[sb1[2]], spec[sb1[3]]);
        p[i] = p0 * (splat4(1.0f) - sbf) + p1 * sbf;
    }
    V4 ip = splat4(0.0f);
    if (inside) {
        real u2 = u - (real)ui, v2 = v - (real)vi;
        ip = p[0] * ((1.0f - u2) * (1.0f - v2)) + p[2] * ((1.0f - u2) * v2) + p[3] * (u2 * v2) + p[1] * (u2 * (1.0f - v2));
    } else {
        const float *uv0 = psy_meng_point_uv[idx[0]];
        const float *uv1 = psy_meng_point_uv[idx[1]];
        real ex = u - uv0[0], ey = v - uv0[1];
        real e0x = uv1[0] - uv0[0], e0y = uv1[1] - uv0[1];
        real uu = e0x * ey - ex * e0y;
        for (int i = 0; i < num - 1; i++) {
            real e1x, e1y;
            if (i == num - 2) {
                e1x = uv1[0] - uv0[0];
                e1y = uv1[1] - uv0[1];
            } else {
                const float *uvn = psy_meng_point_uv[idx[i + 2]];
                e1x = uvn[0] - uv0[0];
                e1y = uvn[1] - uv0[1];
            }
            real vv = ex * e1y - e1x * ey;
            real area = e0x * e1y - e1x * e0y;
            real fu = uu / area, fv = vv / area;
            real fw = 1.0f - fu - fv;
            if (fu < 0.0f || fv < 0.0f || fw < 0.0f) {
                uu = -vv;
                e0x = e1x;
                e0y = e1y;
                continue;
            }
            ip = p[0] * fw + p[i + 1] * fv + p[(i == num - 2) ? 1 : i + 2] * fu;
            break;
        }
    }
    return ip * inv_norm;
}

// ------------------------------------------------------------------ colour
enum { COL_XYZ = 0, COL_BLACKBODY = 1, COL_TEMPERATURE = 2 };
struct Color {
    uint32_t kind;
    real a, b, c;  // XYZ: (x,y,z); blackbody/temperature: (temperature, factor)
};
static inline Color color_mul(Color c, real s) {
    if (c.kind == COL_XYZ) return Color{c.kind, c.a * s, c.b * s, c.c * s};
    return Color{c.kind, c.a, c.b * s, c.c};
}
static inline Color color_lerp(Color x, Color y, real alpha) {
    real ia = 1.0f - alpha;
    if (x.kind == COL_XYZ)
        return Color{x.kind, (x.a * ia) + (y.a * alpha), (x.b * ia) + (y.b * alpha), (x.c * ia) + (y.c * alpha)};
    return Color{x.kind, (x.a * ia) + (y.a * alpha), (x.b * ia) + (y.b * alpha), 0.0f};
}
static inline Color lerp_slice_color(const Color *s, size_t n, real alpha) {
    size_t i; real a2;
    if (lerp_slice_index(n, alpha, &i, &a2)) return s[i];
    return color_lerp(s[i], s[i + 1], a2);
}
// src/color.rs:336-375
static inline real plancks_law(real temperature, real wavelength) {
    const real C = 299792458.0f, H = 6.62607015e-34f, KB = 1.38064852e-23f;
    if (temperature < 200.0f) return 0.0f;
    real wl = wavelength * 1.0e-9f;
    const real TMP1 = (real)(2.0 * (double)H * (double)C * (double)C);
    const real TMP2 = (real)((double)H * (double)C / (double)KB);
    real wl2 = wl * wl;
    real wl5 = wl2 * wl2 * wl;
    real tmp3 = wl5 * (fast_exp(TMP2 / (wl * temperature)) - 1.0f);
    real energy = TMP1 / tmp3;
    return rmax(energy * 1.0e-6f, 0.0f);
}
static inline real plancks_law_normalized(real temperature, real wavelength) {
    real t2 = temperature * temperature;
    return plancks_law(temperature, wavelength) * 4.0e7f / (t2 * t2);
}
// Color::to_spectral_sample (src/color.rs:84-122)
static inline V4 color_to_spectral(Color c, real hero) {
    V4 wls = wavelengths(hero);
    if (c.kind == COL_XYZ)
        return spectrum_xyz_to_p_4(wls, c.a, c.b, c.c) * splat4(1.0f / PSY_MENG_EQUAL_ENERGY_REFLECTANCE);
    V4 o;
    for (int k = 0; k < 4; k++)
        o[k] = (c.kind == COL_BLACKBODY ? plancks_law(c.a, wls[k]) : plancks_law_normalized(c.a, wls[k])) * c.b;
    return o;
}
// Color::approximate_energy (src/color.rs:127-142)
static inline real color_energy(Color c) {
    if (c.kind == COL_XYZ) return c.b;
    if (c.kind == COL_BLACKBODY) {
        real t2 = c.a * c.a;
        return t2 * t2 * c.b;
    }
    return c.b;
}
// CIE 1931 fits (src/color.rs:610-628)
static inline real x_1931(real w) {
    real t1 = (w - 442.0f) * ((w < 442.0f) ? 0.0624f : 0.0374f);
    real t2 = (w - 599.8f) * ((w < 599.8f) ? 0.0264f : 0.0323f);
    real t3 = (w - 501.1f) * ((w < 501.1f) ? 0.0490f : 0.0382f);
    return (0.362f * fast_exp(-0.5f * t1 * t1)) + (1.056f * fast_exp(-0.5f * t2 * t2)) - (0.065f * fast_exp(-0.5f * t3 * t3));
}
static inline real y_1931(real w) {
    real t1 = (w - 568.8f) * ((w < 568.8f) ? 0.0213f : 0.0247f);
    real t2 = (w - 530.9f) * ((w < 530.9f) ? 0.0613f : 0.0322f);
    return (0.821f * fast_exp(-0.5f * t1 * t1)) + (0.286f * fast_exp(-0.5f * t2 * t2));
}
static inline real z_1931(real w) {
    real t1 = (w - 437.0f) * ((w < 437.0f) ? 0.0845f : 0.0278f);
    real t2 = (w - 459.0f) * ((w < 459.0f) ? 0.0385f : 0.0725f);
    return (1.217f * fast_exp(-0.5f * t1 * t1)) + (0.681f * fast_exp(-0.5f * t2 * t2));
}
// XYZ::from_spectral_sample (src/color.rs:520-526)
static inline V3 xyz_from_spectral(V4 e, real hero) {
    V3 acc = v3(0, 0, 0);
    for (int k = 0; k < 4; k++) {
        real wl = nth_wavelength(hero, k);
        V3 c = v3(x_1931(wl) * e[k], y_1931(wl) * e[k], z_1931(wl) * e[k]);
        acc = (k == 0) ? c : acc + c;
    }
    return acc * 0.75f;
}

// ------------------------------------------------------------------ sampling
// src/sampling/monte_carlo.rs:10-38
static inline void square_to_circle(real x, real y, real *ox, real *oy) {
    if (x == 0.0f && y == 0.0f) { *ox = 0.0f; *oy = 0.0f; return; }
    real radius, angle;
    if (x > std::fabs(y)) { radius = x; angle = QPI_32 * (y / x); }
    else if (y > std::fabs(x)) { radius = y; angle = QPI_32 * (2.0f - (x / y)); }
    else if (x < -std::fabs(y)) { radius = -x; angle = QPI_32 * (4.0f + (y / x)); }
    else { radius = -y; angle = QPI_32 * (6.0f - (x / y)); }
    *ox = radius * std::cos(angle);
    *oy = radius * std::sin(angle);
}
static inline V3 cosine_sample_hemisphere(real u, real v) {
    real cu, cv;
    square_to_circle((u * 2.0f) - 1.0f, (v * 2.0f) - 1.0f, &cu, &cv);
    real z = std::sqrt(rmax(1.0f - ((cu * cu) + (cv * cv)), 0.0f));
    return v3(cu, cv, z);
}
static inline V3 uniform_sample_sphere(real u, real v) {
    real z = 1.0f - (2.0f * u);
    real r = std::sqrt(rmax(1.0f - (z * z), 0.0f));
    real phi = 2.0f * PI_32 * v;
    return v3(r * std::cos(phi), r * std::sin(phi), z);
}
static inline V3 uniform_sample_cone(real u, real v, double cos_theta_max) {
    double cos_theta = (1.0 - (double)u) + ((double)u * cos_theta_max);
    double sin_theta = std::sqrt(1.0 - (cos_theta * cos_theta));
    double phi = (double)v * 2.0 * PI_64;
    return v3((real)(std::cos(phi) * sin_theta), (real)(std::sin(phi) * sin_theta), (real)cos_theta);
}
static inline double uniform_sample_cone_pdf(double cos_theta_max) {
    return 1.0 / (2.0 * PI_64 * (1.0 - cos_theta_max));
}
static inline V3 uniform_sample_triangle(V3 va, V3 vb, V3 vc, real i, real j) {
    real isqrt = std::sqrt(i);
    real a = 1.0f - isqrt;
    real b = isqrt * (1.0f - j);
    real c = j * isqrt;
    return (va * a) + (vb * b) + (vc * c);
}
static inline real triangle_surface_area(V3 p0, V3 p1, V3 p2) { return 0.5f * length(cross(p1 - p0, p2 - p0)); }
static inline double clampd(double x) { return std::fmin(std::fmax(x, -1.0), 1.0); }
// src/sampling/monte_carlo.rs:99-132
static inline real spherical_triangle_solid_angle(V3 va, V3 vb, V3 vc) {
    double cos_a = (double)rmin(rmax(dot(vb, vc), -1.0f), 1.0f);
    double cos_b = (double)rmin(rmax(dot(vc, va), -1.0f), 1.0f);
    double cos_c = (double)rmin(rmax(dot(va, vb), -1.0f), 1.0f);
    double sin_a = std::sqrt(1.0 - (cos_a * cos_a));
    double sin_b = std::sqrt(1.0 - (cos_b * cos_b));
    double sin_c = std::sqrt(1.0 - (cos_c * cos_c));
    if (cos_a == 1.0 || cos_b == 1.0 || cos_c == 1.0) return 0.0f;
    double cos_va = clampd((cos_a - (cos_b * cos_c)) / (sin_b * sin_c));
    double cos_vb = clampd((cos_b - (cos_c * cos_a)) / (sin_c * sin_a));
    double cos_vc = clampd((cos_c - (cos_a * cos_b)) / (sin_a * sin_b));
    return (real)(std::acos(cos_va) + std::acos(cos_vb) + std::acos(cos_vc) - PI_64);
}
// src/sampling/monte_carlo.rs:136-200 (Arvo's spherical triangle sampling)
static inline V3 uniform_sample_spherical_triangle(V3 va, V3 vb, V3 vc, real i, real j) {
    double cos_a = (double)rmin(rmax(dot(vb, vc), -1.0f), 1.0f);
    double cos_b = (double)rmin(rmax(dot(vc, va), -1.0f), 1.0f);
    double cos_c = (double)rmin(rmax(dot(va, vb), -1.0f), 1.0f);
    double sin_a = std::sqrt(1.0 - (cos_a * cos_a));
    double sin_b = std::sqrt(1.0 - (cos_b * cos_b));
    double sin_c = std::sqrt(1.0 - (cos_c * cos_c));
    if (cos_a == 1.0 || cos_b == 1.0 || cos_c == 1.0) return va;
    double cos_va = clampd((cos_a - (cos_b * cos_c)) / (sin_b * sin_c));
    double cos_vb = clampd((cos_b - (cos_c * cos_a)) / (sin_c * sin_a));
    double cos_vc = clampd((cos_c - (cos_a * cos_b)) / (sin_a * sin_b));
    double sin_va = std::sqrt(1.0 - (cos_va * cos_va));
    double ang_va = std::acos(cos_va), ang_vb = std::acos(cos_vb), ang_vc = std::acos(cos_vc);
    double area = ang_va + ang_vb + ang_vc - PI_64;
    double area_2 = area * (double)i;
    double s = std::sin(area_2 - ang_va);
    double t = std::cos(area_2 - ang_va);
    double u = t - cos_va;
    double v = s + (sin_va * cos_c);
    double q_top = (((v * t) - (u * s)) * cos_va) - v;
    double q_bottom = ((v * s) + (u * t)) * sin_va;
    double q = q_top / q_bottom;
    V3 vc_2 = (va * (real)q) + (normalized(vc - (va * dot(vc, va))) * (real)std::sqrt(1.0 - (q * q)));
    real z = 1.0f - (j * (1.0f - dot(vc_2, vb)));
    return (vb * z) + (normalized(vc_2 - (vb * dot(vc_2, vb))) * std::sqrt(1.0f - (z * z)));
}
// src/math.rs:179-207
static inline void coordinate_system_from_vector(V3 v, V3 *o1, V3 *o2, V3 *o3) {
    real sign = signum(v.z);
    real a = -1.0f / (sign + v.z);
    real b = v.x * v.y * a;
    *o1 = v;
    *o2 = v3(1.0f + sign * v.x * v.x * a, sign * b, -sign * v.x);
    *o3 = v3(b, sign + v.y * v.y * a, -v.y);
}
static inline V3 zup_to_vec(V3 from, V3 toz) {
    V3 z, x, y;
    coordinate_system_from_vector(normalized(toz), &z, &x, &y);
    return (x * from.x) + (y * from.y) + (z * from.z);
}

// ------------------------------------------------------------------ closures
// src/shading/surface_closure.rs
enum { CL_LAMBERT = 0, CL_GGX = 1, CL_EMIT = 2 };
struct Closure {
    uint32_t kind;
    Color color;
    real roughness, fresnel;
};
static inline void flip_normals(V3 inc, V3 nor, V3 nor_g, V3 *nn, V3 *fng) {
    if (dot(nor_g, inc) <= 0.0f) { *nn = normalized(nor); *fng = nor_g; }
    else { *nn = neg(normalized(nor)); *fng = neg(nor_g); }
}
static inline real schlick_fresnel_from_fac(real f, real c) {
    real c1 = 1.0f - c;
    real c2 = c1 * c1;
    return f + ((1.0f - f) * c1 * c2 * c2);
}
static inline real ggx_d(real nh, real rough) {
    if (nh <= 0.0f) return 0.0f;
    real r2 = rough * rough;
    real tmp = 1.0f + ((r2 - 1.0f) * (nh * nh));
    return r2 / (PI_32 * tmp * tmp);
}
static inline real ggx_g(real vh, real vn, real rough) {
    if ((vh * vn) <= 0.0f) return 0.0f;
    return 2.0f / (1.0f + std::sqrt(1.0f + rough * rough * (1.0f - vn * vn) / (vn * vn)));
}
static inline real half_theta_sample(real u, real rough) {
    real r2 = rough * rough;
    real top = 1.0f - u;
    real bottom = 1.0f + ((r2 - 1.0f) * u);
    return std::sqrt(top / bottom);
}
// returns filter, writes pdf
static inline V4 closure_evaluate(const Closure &cl, V3 inc, V3 out, V3 nor, V3 nor_g, real wl, real *pdf) {
    if (cl.kind == CL_EMIT) { *pdf = 1.0f; return color_to_spectral(cl.color, wl); }
    V3 nn, fng;
    if (cl.kind == CL_LAMBERT) {
        flip_normals(inc, nor, nor_g, &nn, &fng);
        if (dot(fng, out) >= 0.0f) {
            real fac = rmax(dot(nn, normalized(out)), 0.0f) * INV_PI;
            *pdf = fac;
            return color_to_spectral(cl.color, wl) * fac;
        }
        *pdf = 0.0f;
        return splat4(0.0f);
    }
    // GGX
    V3 aa = neg(normalized(inc));
    V3 bb = normalized(out);
    V3 hh = normalized(aa + bb);
    flip_normals(inc, nor, nor_g, &nn, &fng);
    if (dot(nn, aa) < 0.0f || dot(nn, bb) < 0.0f || dot(fng, bb) < 0.0f) { *pdf = 0.0f; return splat4(0.0f); }
    real na = rclamp(dot(nn, aa), -1.0f, 1.0f);
    real nb = rclamp(dot(nn, bb), -1.0f, 1.0f);
    real ha = rclamp(dot(hh, aa), -1.0f, 1.0f);
    real hb = rclamp(dot(hh, bb), -1.0f, 1.0f);
    real nh = rclamp(dot(nn, hh), -1.0f, 1.0f);
    V4 ss = color_to_spectral(cl.color, wl);
    real rev = 1.0f - cl.fresnel;
    V4 col_f;
    for (int k = 0; k < 4; k++) col_f[k] = lerpf(schlick_fresnel_from_fac(ss[k], hb), ss[k], rev);
    if (cl.roughness == 0.0f) { *pdf = 0.0f; return col_f; }
    real dist = ggx_d(nh, cl.roughness) / na;
    real g1 = ggx_g(ha, na, cl.roughness);
    real g2 = ggx_g(hb, nb, cl.roughness);
    *pdf = dist * INV_PI;
    return col_f * (dist * g1 * g2) * INV_PI;
}
static inline V4 closure_sample(const Closure &cl, V3 inc, V3 nor, V3 nor_g, real u, real v, real wl, V3 *out, real *pdf) {
    if (cl.kind == CL_EMIT) { *out = v3(0, 0, 0); *pdf = 1.0f; return color_to_spectral(cl.color, wl); }
    V3 nn, fng;
    flip_normals(inc, nor, nor_g, &nn, &fng);
    if (cl.kind == CL_LAMBERT) {
        V3 dir = cosine_sample_hemisphere(u, v);
        real p = dir.z * INV_PI;
        V3 o = zup_to_vec(dir, nn);
        *out = o;
        if (dot(fng, o) >= 0.0f) { *pdf = p; return color_to_spectral(cl.color, wl) * p; }
        *pdf = 0.0f;
        return splat4(0.0f);
    }
    real theta_cos = half_theta_sample(u, cl.roughness);
    real theta_sin = std::sqrt(1.0f - (theta_cos * theta_cos));
    real angle = v * PI_32 * 2.0f;
    V3 half_dir = v3(std::cos(angle) * theta_sin, std::sin(angle) * theta_sin, theta_cos);
    half_dir = normalized(zup_to_vec(half_dir, nn));
    V3 o = inc - (half_dir * 2.0f * dot(inc, half_dir));
    *out = o;
    if (dot(fng, o) >= 0.0f) return closure_evaluate(cl, inc, o, nor, nor_g, wl, pdf);
    *pdf = 0.0f;
    return splat4(0.0f);
}
// Snyder's analytic Lambert-from-sphere-light (surface_closure.rs:371-402)
static inline real sphere_lambert(real nlcos, real rcos) {
    real nlsin = std::sqrt(1.0f - (nlcos * nlcos));
    real rsin2 = 1.0f - (rcos * rcos);
    real rsin = std::sqrt(rsin2);
    real ysin = rcos / nlsin;
    real ycos2 = 1.0f - (ysin * ysin);
    real ycos = std::sqrt(ycos2);
    real g = (-2.0f * nlsin * rcos * ycos) + H_PI - std::asin(ysin) + (ysin * ycos);
    real h = nlcos * ((ycos * std::sqrt(rsin2 - ycos2)) + (rsin2 * std::asin(ycos / rsin)));
    real nl = std::acos(nlcos);
    real r = std::acos(rcos);
    if (nl < (H_PI - r)) return nlcos * rsin2;
    if (nl < H_PI) return (nlcos * rsin2) + g - h;
    if (nl < (H_PI + r)) return (g + h) * INV_PI;
    return 0.0f;
}
static inline real closure_estimate_sphere(const Closure &cl, V3 inc, V3 to_light, real r2l, V3 nor, V3 nor_g) {
    if (cl.kind == CL_LAMBERT) {
        real dist2 = length2(to_light);
        if (dist2 <= r2l) return rmin(r2l / dist2, 4.0f);
        real stm2 = rmin(r2l / dist2, 1.0f);
        real ctm = std::sqrt(1.0f - stm2);
        V3 v = normalized(to_light);
        V3 nn = (dot(nor_g, inc) <= 0.0f) ? normalized(nor) : neg(normalized(nor));
        real cos_nv = rmin(rmax(dot(nn, v), -1.0f), 1.0f);
        return sphere_lambert(cos_nv, ctm);
    }
    if (cl.kind == CL_GGX) {
        real dist2 = length2(to_light);
        real stm2 = rmin(r2l / dist2, 1.0f);
        real ctm = std::sqrt(1.0f - stm2);
        V3 nn = (dot(nor, inc) < 0.0f) ? normalized(nor) : neg(normalized(nor));
        V3 aa = neg(normalized(inc));
        V3 bb = normalized(to_light);
        real theta = std::acos(ctm);
        V3 hh = normalized(aa + bb);
        real nh = rclamp(dot(nn, hh), -1.0f, 1.0f);
        real fac = ggx_d(nh, rmin(1.0f, std::sqrt(cl.roughness) + (2.0f * theta / PI_32)));
        return fac * rmin(1.0f, 1.0f - ctm) * INV_PI;
    }
    return 0.0f;  // Emit: never asked (unimplemented in the reference)
}

}  // namespace psyo
