// Surface data of a hit (shared by the trace and shade kernels).
#pragma once

#include "dev_trace.cuh"

namespace psyd {

// ------------------------------------------------------------------ surface data
// SurfaceIntersectionData of a hit, recomputed from the hit record with the
// traversal's own arithmetic (src/surface/triangle_mesh.rs:264-318,
// src/light/*_light.rs intersect_rays).
struct SurfData {
    V3 pos, nor, nor_g;
    float pos_err, sample_pdf;
    Closure closure;
    int32_t shader;
};
// Colour of the tracer's shader for instances without one (src/tracer.rs:161-163),
// rec709_to_xyz((1, 0, 1)) computed on the host.
static __constant__ GColor c_magenta;

template <class R>
__device__ void resolve_hit(const GScene &S, const HitRec &h, V3 o, V3 d, float time, SurfData &sd) {
    GInstance in = S.instances[h.slot];
    if (h.kind == PSY_HIT_SURFACE_K) {
        GMesh M = S.meshes[in.obj];
        bool has_xf = in.xc != 0;
        Xf mat = has_xf ? instance_mat(S, in, time) : xf_identity();
        V3 p0, p1, p2;
        fetch_tri(S, M, h.prim, time, has_xf, mat, p0, p1, p2);
        surface_point(p0, p1, p2, h.b0, h.b1, h.b2, &sd.pos, &sd.pos_err);
        V3 geo = cross(p0 - p1, p0 - p2);
        V3 sn = geo;
        if (M.has_normals) {
            uint4 ix = __ldg(S.tri_idx + h.prim);
            const float4 *nb = S.normals + M.vert_base;
            V3 n0 = normalized(lerp_slice_v3(nb + (size_t)ix.x * M.ts, M.ts, time));
            V3 n1 = normalized(lerp_slice_v3(nb + (size_t)ix.y * M.ts, M.ts, time));
            V3 n2 = normalized(lerp_slice_v3(nb + (size_t)ix.z * M.ts, M.ts, time));
            V3 snn = xf_normal((n0 * h.b0) + (n1 * h.b1) + (n2 * h.b2), mat);
            sn = (dot(snn, geo) >= 0.0f) ? snn : neg(snn);
        }
        sd.nor = sn;
        sd.nor_g = geo;
        sd.sample_pdf = 0.0f;
        sd.shader = in.shader;
        if (in.shader >= 0) {
            sd.closure = closure_from_shader(S.shaders[in.shader]);
        } else {
            sd.closure.kind = PSY_CL_EMIT;
            sd.closure.color = c_magenta;
            sd.closure.roughness = 0.0f;
            sd.closure.fresnel = 0.0f;
        }
        return;
    }
    // light surfaces
    const GLight L = S.lights[in.obj];
    Xf xf = instance_xf_at(S, in, time);
    sd.shader = -1;
    sd.closure.kind = PSY_CL_EMIT;
    sd.closure.roughness = 0.0f;
    sd.closure.fresnel = 0.0f;
    GColor col = lerp_slice_color(S.light_colors + L.key_base, L.nkeys, time);
    if (in.kind == PSY_INST_RECT) {
        float w = light_dim(S, L, 0, time), hh = light_dim(S, L, 1, time);
        Xf si = light_inverse(S, in, xf);
        V3 p1, p2, p3, p4;
        rect_corners(w, hh, si, &p1, &p2, &p3, &p4);
        V3 a = h.prim == 0 ? p1 : p3, b = h.prim == 0 ? p2 : p4, c = h.prim == 0 ? p3 : p1;
        surface_point(a, b, c, h.b0, h.b1, h.b2, &sd.pos, &sd.pos_err);
        V3 nn = cross(a - b, a - c);
        sd.nor = nn;
        sd.nor_g = nn;
        sd.sample_pdf = rect_sample_pdf<R>(S, L, si, o, d, sd.pos, time);
        float isa = (float)(1.0 / ((double)w * (double)hh));
        sd.closure.color = color_mul(col, isa);
    } else {
        float radius = light_dim(S, L, 0, time);
        Xf ixf = light_inverse(S, in, xf);
        V3 ol = in.xc ? xf_point(o, xf) : xf_point(o, xf_identity());
        V3 dir = xf_vector(d, xf);
        V3 unit = normalized(ol + (dir * h.t));
        sd.pos = xf_vector(unit * radius, ixf);  // as the reference: a vector transform
        sd.pos_err = 0.001f;
        V3 nrm = xf_normal(unit, ixf);
        sd.nor = nrm;
        sd.nor_g = nrm;
        sd.sample_pdf = sphere_sample_pdf<R>(S, L, xf, o, time);
        float isa = (float)(1.0 / (4.0 * PSY_PI_64 * (double)radius * (double)radius));
        sd.closure.color = color_mul(col, isa);
    }
}


}  // namespace psyd
