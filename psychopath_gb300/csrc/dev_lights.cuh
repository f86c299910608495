// Device light sampling: rectangle / sphere surface lights
// (src/light/rectangle_light.rs, src/light/sphere_light.rs), the distant disk
// light (src/light/distant_disk_light.rs), the 8-ary light tree selection
// (src/accel/light_tree.rs:135-201) and Scene::sample_lights
// (src/scene/mod.rs:28-99) for the root assembly.
#pragma once

#include "dev_shade.cuh"

namespace psyd {

DI float light_dim(const GScene &S, const GLight &L, int c, float time) {
    uint32_t i; float a2;
    const float2 *d = S.light_dims + L.key_base;
    if (lerp_index(L.nkeys, time, &i, &a2)) return c == 0 ? d[i].x : d[i].y;
    float a = c == 0 ? d[i].x : d[i].y, b = c == 0 ? d[i + 1].x : d[i + 1].y;
    return lerpf(a, b, a2);
}
DI Xf instance_xf_at(const GScene &S, const GInstance &in, float time) {
    return in.xc ? lerp_slice_xf(S.xforms + 3 * in.xs, in.xc, time) : xf_identity();
}
DI void rect_corners(float w, float h, const Xf &si, V3 *p1, V3 *p2, V3 *p3, V3 *p4) {
    *p1 = xf_point(v3(w * 0.5f, h * 0.5f, 0.0f), si);
    *p2 = xf_point(v3(w * -0.5f, h * 0.5f, 0.0f), si);
    *p3 = xf_point(v3(w * -0.5f, h * -0.5f, 0.0f), si);
    *p4 = xf_point(v3(w * 0.5f, h * -0.5f, 0.0f), si);
}
// The inverse of a light instance's space at `time`: precomputed by the
// host for a single-key transform (the same f32 formula as xf_inverse).
DI Xf light_inverse(const GScene &S, const GInstance &in, const Xf &space) {
    return in.xc == 1 ? xf_load(S.xforms_inv + 3 * in.xinv) : xf_inverse(space);
}
// RectangleLight::sample_pdf; si: the inverse of the light's space
template <class R>
DI float rect_sample_pdf(const GScene &S, const GLight &L, const Xf &si, V3 arr, V3 sample_dir, V3 hit, float time) {
    float w = light_dim(S, L, 0, time), h = light_dim(S, L, 1, time);
    V3 p1, p2, p3, p4;
    rect_corners(w, h, si, &p1, &p2, &p3, &p4);
    V3 sp1 = normalized(p1 - arr), sp2 = normalized(p2 - arr), sp3 = normalized(p3 - arr), sp4 = normalized(p4 - arr);
    float a1 = spherical_triangle_solid_angle<R>(sp2, sp1, sp3);
    float a2 = spherical_triangle_solid_angle<R>(sp4, sp1, sp3);
    V3 normal = xf_normal(v3(0.0f, 0.0f, 1.0f), si);
    if ((a1 + a2) < 0.01f) {
        float area = triangle_surface_area(p2, p1, p3) + triangle_surface_area(p4, p1, p3);
        return length2(hit - arr) / fabsf(dot(normalized(sample_dir), normalized(normal))) / area;
    }
    return 1.0f / (a1 + a2);
}
// SphereLight::sample_pdf
template <class R>
DI float sphere_sample_pdf(const GScene &S, const GLight &L, const Xf &space, V3 arr_w, float time) {
    V3 arr = xf_point(arr_w, space);
    R radius = (R)light_dim(S, L, 0, time);
    R d2 = (R)length2(v3(0.0f, 0.0f, 0.0f) - arr);
    R d = msqrt(d2);
    if (d > radius) {
        R st2 = mfmin((radius * radius) / d2, (R)1);
        return (float)cone_pdf_st2<R>(st2, msqrt((R)1 - st2));
    }
    return (float)((R)1 / ((R)4 * pi_r<R>()));
}

struct LightSample {
    int kind;  // 0 none, 1 distant, 2 surface
    V4 color;  // color_spectrum(lcol, wl) * s1 * s2
    V3 dir, sp, sn;
    float serr, pdf, sel_pdf;
    GColor lcol;  // the light's colour at the sample's time
    float s1, s2;  // its scale factors, applied in this order
};

// The light samples leave the colour's spectrum to the caller (o.lcol and
// its scale factors o.s1, o.s2): scene_sample_lights converts it once after
// its branches, so a warp whose lanes took different lights does not run
// the spectral upsampling once per branch (the same value: the same
// function of the same colour, scaled in the same order).  `si` is the
// inverse of the light's space.
template <class R>
DI void rect_sample(const GScene &S, const GLight &L, const Xf &space, const Xf &si, V3 arr, float u, float v,
                    float time, LightSample &o) {
    float w = light_dim(S, L, 0, time), h = light_dim(S, L, 1, time);
    GColor col = lerp_slice_color(S.light_colors + L.key_base, L.nkeys, time);
    R sai = (R)1 / ((R)w * (R)h);
    V3 p1, p2, p3, p4;
    rect_corners(w, h, si, &p1, &p2, &p3, &p4);
    V3 sp1 = normalized(p1 - arr), sp2 = normalized(p2 - arr), sp3 = normalized(p3 - arr), sp4 = normalized(p4 - arr);
    float a1 = spherical_triangle_solid_angle<R>(sp2, sp1, sp3);
    float a2 = spherical_triangle_solid_angle<R>(sp4, sp1, sp3);
    V3 normal = xf_normal(v3(0.0f, 0.0f, 1.0f), si);
    if ((a1 + a2) < 0.01f) {
        float sa1 = triangle_surface_area(p2, p1, p3);
        float sa2 = triangle_surface_area(p4, p1, p3);
        float th = sa1 / (sa1 + sa2);
        V3 spt = (u < th) ? uniform_sample_triangle(p2, p1, p3, v, u / th)
                          : uniform_sample_triangle(p4, p1, p3, v, (u - th) / (1.0f - th));
        V3 shadow_vec = spt - arr;
        o.pdf = length2(spt - arr) / fabsf(dot(normalized(shadow_vec), normalized(normal))) / (sa1 + sa2);
        o.sp = spt; o.sn = normal; o.serr = 0.0001f;
        o.lcol = col; o.s1 = (float)sai; o.s2 = 0.5f;
        return;
    }
    float prob_1 = isinf(a1) ? 1.0f : (isinf(a2) ? 0.0f : a1 / (a1 + a2));
    float prob_2 = 1.0f - prob_1;
    V3 shadow_vec = (u < prob_1) ? uniform_sample_spherical_triangle<R>(sp2, sp1, sp3, v, u / prob_1)
                                 : uniform_sample_spherical_triangle<R>(sp4, sp1, sp3, v, 1.0f - ((u - prob_1) / prob_2));
    V3 arr_local = xf_point(arr, space);
    V3 svl = xf_vector(shadow_vec, space);
    svl = svl * (-arr_local.z / svl.z);
    V3 spl = arr_local + svl;
    spl.x = rmin(rmax(spl.x, w * -0.5f), w * 0.5f);
    spl.y = rmin(rmax(spl.y, h * -0.5f), h * 0.5f);
    spl.z = 0.0f;
    o.sp = xf_point(spl, si);
    o.sn = normal;
    o.serr = 0.0001f;
    o.pdf = 1.0f / (a1 + a2);
    o.lcol = col; o.s1 = (float)sai; o.s2 = 0.5f;
}

template <class R>
DI void sphere_sample(const GScene &S, const GLight &L, const Xf &space, const Xf &inv, V3 arr_w, float u, float v,
                      float time, LightSample &o) {
    V3 arr = xf_point(arr_w, space);
    R radius = (R)light_dim(S, L, 0, time);
    GColor col = lerp_slice_color(S.light_colors + L.key_base, L.nkeys, time);
    R sai = (R)1 / ((R)4 * pi_r<R>() * radius * radius);
    V3 zv = v3(0.0f, 0.0f, 0.0f) - arr;
    R d2 = (R)length2(zv);
    R d = msqrt(d2);
    V3 z, x, y;
    coordinate_system_from_vector(zv, &z, &x, &y);
    x = normalized(x); y = normalized(y); z = normalized(z);
    float rf = (float)radius;
    o.serr = length(xf_vector(v3(rf, rf, rf), inv)) * 0.001f;
    // phi = v * 2 pi is shared by the cone sample and the point placement
    R sp, cp;
    msincos_2pi((R)v, &sp, &cp);
    if (d > radius) {
        R st2 = mfmin((radius * radius) / d2, (R)1);
        R ct2 = (R)1 - st2;
        R st = msqrt(st2);
        R ct = msqrt(ct2);
        // uniform_sample_cone(u, v, ct), normalized
        R cone_c = ((R)1 - (R)u) + ((R)u * ct);
        // in f64 cone_c <= 1 exactly (1 - u is exact); in f32 1 - u can round
        // up, so clamp (the reference's form has nothing to clamp)
        R sc2 = (R)1 - (cone_c * cone_c);
        if (sizeof(R) == sizeof(float)) sc2 = mfmax(sc2, (R)0);
        R cone_s = msqrt(sc2);
        V3 smp = normalized(v3((float)(cp * cone_s), (float)(sp * cone_s), (float)cone_c));
        R cos_theta = (R)smp.z;
        R cos_theta2 = cos_theta * cos_theta;
        R sin_theta2 = mfmax((R)1 - cos_theta2, (R)0);
        R sin_theta = msqrt(sin_theta2);
        R dd = (R)1 - (d2 * sin_theta * sin_theta / (radius * radius));
        R cos_a = (dd <= (R)0) ? st : ((d / radius) * sin_theta2) + (cos_theta * msqrt(dd));
        R sin_a = msqrt(mfmax((R)1 - (cos_a * cos_a), (R)0));
        V3 s2 = v3((float)(cp * sin_a * radius), (float)(sp * sin_a * radius), (float)(d - (cos_a * radius)));
        V3 svec = (x * s2.x) + (y * s2.y) + (z * s2.z);
        V3 normal = normalized(arr + svec);
        o.sp = xf_point(normal * rf, inv);
        o.sn = xf_normal(normal, inv);
        o.pdf = (float)cone_pdf_st2<R>(st2, ct);
        o.lcol = col; o.s1 = (float)sai; o.s2 = 1.0f;
        return;
    }
    V3 svec = uniform_sample_sphere(u, v);
    V3 normal = normalized(arr + svec);
    o.sp = xf_point(normal * rf, inv);
    o.sn = xf_normal(normal, inv);
    o.pdf = (float)((R)1 / ((R)4 * pi_r<R>()));
    o.lcol = col; o.s1 = (float)sai; o.s2 = 1.0f;
}

DI float bbox_prob(const GScene &S, const GLightTreeNode &nd, float time, V3 pos, const Closure &sc, V3 inc, V3 nor,
                   V3 nor_g) {
    // lerp_slice over the node's boxes
    uint32_t i; float a2;
    const float4 *b = S.lt_bounds + 2 * nd.bounds_base;
    V3 mn, mx;
    if (lerp_index(nd.nbounds, time, &i, &a2)) {
        mn = v3(b[2 * i]); mx = v3(b[2 * i + 1]);
    } else {
        mn = lerp3(v3(b[2 * i]), v3(b[2 * i + 2]), a2);
        mx = lerp3(v3(b[2 * i + 1]), v3(b[2 * i + 3]), a2);
    }
    V3 center = lerp3(mn, mx, 0.5f);
    V3 dd = center - pos;
    float r2 = length2(mx - mn) * 0.25f;
    float inv_sa = 1.0f / r2;
    float contrib = closure_estimate_sphere(sc, inc, dd, r2, nor, nor_g);
    return nd.energy * inv_sa * contrib;
}

DI bool lt_select(const GScene &S, V3 inc, V3 pos, V3 nor, V3 nor_g, const Closure &sc, float time, float n,
                  uint32_t *light_index, float *pdf) {
    if (S.lt_empty) return false;
    GLightTreeNode node = S.lt_nodes[0];
    float tot = 1.0f;
    while (!node.leaf) {
        float ps[8];
        float total = 0.0f;
        for (uint32_t i = 0; i < 8; i++) ps[i] = 0.0f;
        for (uint32_t i = 0; i < node.nchild; i++) {
            float p = bbox_prob(S, S.lt_nodes[node.index + i], time, pos, sc, inc, nor, nor_g);
            ps[i] = p;
            total += p;
        }
        if (total <= 0.0f) {
            float p = 1.0f / (float)node.nchild;
            for (int i = 0; i < 8; i++) ps[i] = p;
        } else {
            for (int i = 0; i < 8; i++) ps[i] /= total;
        }
        float base = 0.0f;
        uint32_t pick = node.nchild - 1;
        for (uint32_t i = 0; i < 8; i++) {
            float p = ps[i];
            if ((n <= base + p) || (i == node.nchild - 1)) {
                tot *= p;
                pick = i;
                n = (n - base) / p;
                break;
            }
            base += p;
        }
        node = S.lt_nodes[node.index + pick];
    }
    *light_index = node.index;
    *pdf = tot;
    return true;
}

// Scene::sample_lights for the root assembly.  `pos, nor, nor_g, inc` are
// the hit's world-space intersection data.
template <class R>
DI LightSample scene_sample_lights(const GScene &S, float n, float u, float v, float wl, float time, V3 inc, V3 pos,
                                   V3 nor, V3 nor_g, const Closure &cl) {
    LightSample out;
    out.kind = 0;
    float wl_energy = (S.distant_energy_total <= 0.0f) ? 0.0f : 1.0f;
    float ll_energy = (S.lt_empty || S.lt_root_energy <= 0.0f) ? 0.0f : 1.0f;
    float tot = wl_energy + ll_energy;
    if (tot <= 0.0f) return out;
    float wl_prob = wl_energy / tot;
    if (n < wl_prob) {
        float nn = n / wl_prob;
        float total = S.distant_energy_total;
        float target = nn * total;
        float x = 0.0f;
        uint32_t pick = S.n_distant - 1;
        float p = 0.0f;
        for (uint32_t i = 0; i < S.n_distant; i++) {
            float wgt = S.distant[i].energy;
            x += wgt;
            if (x > target) { pick = i; p = wgt / total; break; }
            if (i == S.n_distant - 1) p = wgt / total;
        }
        const GDistant &L = S.distant[pick];
        V3 direction = lerp_slice_v3(S.distant_dirs + L.key_base, L.nkeys, time);
        GColor col = lerp_slice_color(S.distant_colors + L.key_base, L.nkeys, time);
        R ctm;
        float sai_f, pdf_f;
        if (L.is_static) {
            // cos(radius) and the cone's solid-angle inverse, evaluated by the host
            ctm = (R)L.ctm;
            sai_f = L.sai;
            pdf_f = L.sai;
        } else {
            R radius = (R)lerp_slice_f(S.distant_radii + L.key_base, L.nkeys, time);
            ctm = mcos(radius);
            R sai = (R)1 / ((R)2 * pi_r<R>() * ((R)1 - ctm));
            sai_f = (float)sai;
            pdf_f = (float)uniform_sample_cone_pdf<R>(ctm);
        }
        V3 z, x3, y3;
        coordinate_system_from_vector(neg(normalized(direction)), &z, &x3, &y3);
        V3 smp = normalized(uniform_sample_cone<R>(u, v, ctm));
        out.kind = 1;
        out.lcol = col; out.s1 = sai_f; out.s2 = 1.0f;  // x * 1.0f is exact
        out.dir = (x3 * smp.x) + (y3 * smp.y) + (z * smp.z);
        out.pdf = pdf_f;
        out.sel_pdf = p * wl_prob;
    } else {
        float nl = (n - wl_prob) / (1.0f - wl_prob);
        Xf ident = xf_identity();
        uint32_t li;
        float sel_pdf;
        if (!lt_select(S, xf_vector(inc, ident), xf_point(pos, ident), xf_normal(nor, ident), xf_normal(nor_g, ident),
                       cl, time, nl, &li, &sel_pdf))
            return out;
        GInstance inst = S.light_instances[li];
        Xf xf = instance_xf_at(S, inst, time);
        Xf xinv = light_inverse(S, inst, xf);
        const GLight &L = S.lights[inst.obj];
        if (inst.kind == PSY_INST_RECT) rect_sample<R>(S, L, xf, xinv, pos, u, v, time, out);
        else sphere_sample<R>(S, L, xf, xinv, pos, u, v, time, out);
        out.kind = 2;
        out.sel_pdf = sel_pdf * (1.0f - wl_prob);
    }
    out.color = color_spectrum<R>(S, out.lcol, wl) * out.s1 * out.s2;
    return out;
}

}  // namespace psyd
