// Per-ray BVH4 traversal of the two-level scene (instance BVH -> mesh BVH),
// replacing Tracer::trace (src/tracer.rs:51-190), BVH4::traverse
// (src/accel/bvh4.rs:101-184), TriangleMesh::intersect_rays
// (src/surface/triangle_mesh.rs:124-322) and the light surfaces'
// intersect_rays (src/light/{rectangle,sphere}_light.rs).
//
// The reference traverses packets: a task of ray indices walks the tree and
// each node's BBox4 test fans the task out into the children's lanes.  Here
// every thread walks its own ray through the same tree with a private stack
// and visits the hit children in the reference's front-to-back table order
// (TRAVERSAL_TABLE row of the ray's own direction octant).  Each ray meets
// the same nodes and triangles with the same arithmetic, so closest hits and
// their t are identical to the reference except for exact t ties between
// triangles (where the visit order decides).
#pragma once

#include "dev_lights.cuh"

namespace psyd {

// Child visit order per direction octant and node topology (filled by the host).
static __constant__ uint8_t c_traversal_table[8][48];

struct HitRec {
    uint32_t kind;  // PSY_HIT_*
    uint32_t prim;  // BVH-order global triangle index (mesh) or 0/1 (rect light)
    uint32_t slot;  // instance slot (instance-BVH order)
    float t, b0, b1, b2;
};

#define PSY_HIT_MISS_K 0u
#define PSY_HIT_OCCLUDE_K 1u
#define PSY_HIT_SURFACE_K 2u
#define PSY_HIT_LIGHT_K 3u

// Child bounds of one node at the ray's time.  Static nodes use the inline
// key; motion nodes lerp between keys like lerp_slice(bounds, time).
struct NodeBounds {
    float4 xlo, xhi, ylo, yhi, zlo, zhi;
};
DI void load_key(const GScene &S, const GNode *n, uint32_t ext, uint32_t k, NodeBounds &b) {
    if (k == 0) {
        b.xlo = __ldg(&n->xlo); b.xhi = __ldg(&n->xhi); b.ylo = __ldg(&n->ylo);
        b.yhi = __ldg(&n->yhi); b.zlo = __ldg(&n->zlo); b.zhi = __ldg(&n->zhi);
    } else {
        const GBounds4 *e = S.bounds_ext + ext + (k - 1);
        b.xlo = __ldg(&e->xlo); b.xhi = __ldg(&e->xhi); b.ylo = __ldg(&e->ylo);
        b.yhi = __ldg(&e->yhi); b.zlo = __ldg(&e->zlo); b.zhi = __ldg(&e->zhi);
    }
}
DI float4 lerp4(float4 a, float4 b, float al) {
    float ia = 1.0f - al;
    return make_float4((a.x * ia) + (b.x * al), (a.y * ia) + (b.y * al), (a.z * ia) + (b.z * al), (a.w * ia) + (b.w * al));
}

// Test the (up to 4) children of a node; returns the hit mask.
// Child hit mask of BVH4 node ni.  safe: the ray passes slab_safe and the
// scene's boxes are ordered (ordered_slabs); oct: ray_code(di).
DI uint32_t node_hits(const GScene &S, uint32_t ni, V3 o, V3 di, float tmax, float time, uint32_t oct, bool safe,
                      uint32_t &code, uint32_t &count, uint4 &child) {
    const GNode *n = S.nodes + ni;
    uint4 meta = __ldg(&n->meta);
    child = __ldg(&n->child);
    code = meta.z & 0xFFu;
    count = meta.z >> 8;
    if (safe) {
        // near / far planes picked by the direction's signs; with motion
        // keys, each plane is lerped between the two keys (a lerp of ordered
        // boxes stays ordered: both products and the sum round monotonically)
        uint32_t sx = oct & 1u, sy = (oct >> 1) & 1u, sz = (oct >> 2) & 1u;
        float4 nx, fx, ny, fy, nz, fz;
        auto planes = [&](const float4 *bb, float4 &px, float4 &qx, float4 &py, float4 &qy, float4 &pz, float4 &qz) {
            px = __ldg(bb + sx); qx = __ldg(bb + (sx ^ 1u));
            py = __ldg(bb + 2 + sy); qy = __ldg(bb + 2 + (sy ^ 1u));
            pz = __ldg(bb + 4 + sz); qz = __ldg(bb + 4 + (sz ^ 1u));
        };
        auto key_ptr = [&](uint32_t k) -> const float4 * {  // xlo, xhi, ylo, yhi, zlo, zhi of key k
            return k == 0 ? reinterpret_cast<const float4 *>(n)
                          : reinterpret_cast<const float4 *>(S.bounds_ext + meta.x + (k - 1));
        };
        if (meta.y <= 1) {
            planes(key_ptr(0), nx, fx, ny, fy, nz, fz);
        } else {
            uint32_t i; float a2;
            if (lerp_index(meta.y, time, &i, &a2)) {
                planes(key_ptr(i), nx, fx, ny, fy, nz, fz);
            } else {
                float4 ax, bx, ay, by, az, bz, cx, dx, cy, dy, cz, dz;
                planes(key_ptr(i), ax, bx, ay, by, az, bz);
                planes(key_ptr(i + 1), cx, dx, cy, dy, cz, dz);
                nx = lerp4(ax, cx, a2); fx = lerp4(bx, dx, a2);
                ny = lerp4(ay, cy, a2); fy = lerp4(by, dy, a2);
                nz = lerp4(az, cz, a2); fz = lerp4(bz, dz, a2);
            }
        }
        // slab distances of all four children, two per packed operation
        // (bit-identical to slab_hit_ordered's scalar arithmetic)
        float tnx[4], tfx[4], tny[4], tfy[4], tnz[4], tfz[4];
        f32x2 ox = pk2(o.x, o.x), oy = pk2(o.y, o.y), oz = pk2(o.z, o.z);
        f32x2 dx = pk2(di.x, di.x), dy = pk2(di.y, di.y), dz = pk2(di.z, di.z);
        slab_axis4(nx, ox, dx, tnx); slab_axis4(fx, ox, dx, tfx);
        slab_axis4(ny, oy, dy, tny); slab_axis4(fy, oy, dy, tfy);
        slab_axis4(nz, oz, dz, tnz); slab_axis4(fz, oz, dz, tfz);
        uint32_t m = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float far_t = fminf(fmin3f(tfx[c], tfy[c], tfz[c]) * PSY_BBOX_MAXT_ADJUST, tmax);
            float near_t = fmax3f(tnx[c], tny[c], fmaxf(tnz[c], 0.0f));
            m |= near_t < far_t ? (1u << c) : 0u;
        }
        return m & ((1u << count) - 1u);
    }
    NodeBounds b;
    if (meta.y <= 1) {
        load_key(S, n, meta.x, 0, b);
    } else {
        uint32_t i; float a2;
        if (lerp_index(meta.y, time, &i, &a2)) {
            load_key(S, n, meta.x, i, b);
        } else {
            NodeBounds b0, b1;
            load_key(S, n, meta.x, i, b0);
            load_key(S, n, meta.x, i + 1, b1);
            b.xlo = lerp4(b0.xlo, b1.xlo, a2); b.xhi = lerp4(b0.xhi, b1.xhi, a2);
            b.ylo = lerp4(b0.ylo, b1.ylo, a2); b.yhi = lerp4(b0.yhi, b1.yhi, a2);
            b.zlo = lerp4(b0.zlo, b1.zlo, a2); b.zhi = lerp4(b0.zhi, b1.zhi, a2);
        }
    }
    uint32_t m = 0;
    if (slab_safe(o, di, tmax)) {  // finite inverse direction: one-instruction min / max
        m |= slab_hit_finite(b.xlo.x, b.xhi.x, b.ylo.x, b.yhi.x, b.zlo.x, b.zhi.x, o, di, tmax) ? 1u : 0u;
        m |= slab_hit_finite(b.xlo.y, b.xhi.y, b.ylo.y, b.yhi.y, b.zlo.y, b.zhi.y, o, di, tmax) ? 2u : 0u;
        m |= slab_hit_finite(b.xlo.z, b.xhi.z, b.ylo.z, b.yhi.z, b.zlo.z, b.zhi.z, o, di, tmax) ? 4u : 0u;
        m |= slab_hit_finite(b.xlo.w, b.xhi.w, b.ylo.w, b.yhi.w, b.zlo.w, b.zhi.w, o, di, tmax) ? 8u : 0u;
    } else {
        m |= slab_hit(b.xlo.x, b.xhi.x, b.ylo.x, b.yhi.x, b.zlo.x, b.zhi.x, o, di, tmax) ? 1u : 0u;
        m |= slab_hit(b.xlo.y, b.xhi.y, b.ylo.y, b.yhi.y, b.zlo.y, b.zhi.y, o, di, tmax) ? 2u : 0u;
        m |= slab_hit(b.xlo.z, b.xhi.z, b.ylo.z, b.yhi.z, b.zlo.z, b.zhi.z, o, di, tmax) ? 4u : 0u;
        m |= slab_hit(b.xlo.w, b.xhi.w, b.ylo.w, b.yhi.w, b.zlo.w, b.zhi.w, o, di, tmax) ? 8u : 0u;
    }
    return m & ((1u << count) - 1u);
}

// FP16 node variant: a child bound is decoded as the f32 sum corner +
// offset (the node's min corner for lower bounds, its max corner for upper
// ones), rounded to nearest, in one instruction (PTX add.rn.f32.f16: the f16
// operand converts exactly).  The build chose every offset so that this sum
// already lies outside the f32 bound (GNodeH in psy_layout.h), so the
// decoded boxes contain the f32 boxes and the same slab arithmetic hits
// every child the f32 test hits.
DI float dec_h(unsigned short h, float anchor) {
    float r;
    asm("add.rn.f32.f16 %0, %1, %2;" : "=f"(r) : "h"(h), "f"(anchor));
    return r;
}
// The four children's bounds of one slab (4 x f16 in a uint2).
DI float4 dec_plane(uint2 q, float anchor) {
    unsigned short h0, h1, h2, h3;
    asm("mov.b32 {%0, %1}, %2;" : "=h"(h0), "=h"(h1) : "r"(q.x));
    asm("mov.b32 {%0, %1}, %2;" : "=h"(h2), "=h"(h3) : "r"(q.y));
    return make_float4(dec_h(h0, anchor), dec_h(h1, anchor), dec_h(h2, anchor), dec_h(h3, anchor));
}
// Child hit mask of an FP16 node.  Lower bounds decode from the node's
// anchor a, upper bounds from its top corner, itself decoded as
// fl32(a + ext).  safe: octant-ordered planes as in node_hits (the decoded
// boxes are ordered too: lo16 <= lo32 <= hi32 <= hi16).
DI uint32_t fp16_hits(const GNodeH *n, float4 a, V3 o, V3 di, float tmax, uint32_t oct, bool safe) {
    uint2 e = __ldg(&n->ext);
    unsigned short ex, ey, ez = (unsigned short)(e.y & 0xFFFFu);
    asm("mov.b32 {%0, %1}, %2;" : "=h"(ex), "=h"(ey) : "r"(e.x));
    float tx = dec_h(ex, a.x), ty = dec_h(ey, a.y), tz = dec_h(ez, a.z);  // the max corner
    const uint2 *pl = &n->xlo;  // xlo, xhi, ylo, yhi, zlo, zhi
    if (safe) {
        uint32_t sx = oct & 1u, sy = (oct >> 1) & 1u, sz = (oct >> 2) & 1u;
        float4 nx = dec_plane(__ldg(pl + sx), sx ? tx : a.x), fx = dec_plane(__ldg(pl + (sx ^ 1u)), sx ? a.x : tx);
        float4 ny = dec_plane(__ldg(pl + 2 + sy), sy ? ty : a.y), fy = dec_plane(__ldg(pl + 2 + (sy ^ 1u)), sy ? a.y : ty);
        float4 nz = dec_plane(__ldg(pl + 4 + sz), sz ? tz : a.z), fz = dec_plane(__ldg(pl + 4 + (sz ^ 1u)), sz ? a.z : tz);
        float tnx[4], tfx[4], tny[4], tfy[4], tnz[4], tfz[4];
        f32x2 ox = pk2(o.x, o.x), oy = pk2(o.y, o.y), oz = pk2(o.z, o.z);
        f32x2 dx = pk2(di.x, di.x), dy = pk2(di.y, di.y), dz = pk2(di.z, di.z);
        slab_axis4(nx, ox, dx, tnx); slab_axis4(fx, ox, dx, tfx);
        slab_axis4(ny, oy, dy, tny); slab_axis4(fy, oy, dy, tfy);
        slab_axis4(nz, oz, dz, tnz); slab_axis4(fz, oz, dz, tfz);
        uint32_t m = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float far_t = fminf(fmin3f(tfx[c], tfy[c], tfz[c]) * PSY_BBOX_MAXT_ADJUST, tmax);
            float near_t = fmax3f(tnx[c], tny[c], fmaxf(tnz[c], 0.0f));
            m |= near_t < far_t ? (1u << c) : 0u;
        }
        return m;
    }
    float4 xl = dec_plane(__ldg(pl), a.x), xh = dec_plane(__ldg(pl + 1), tx);
    float4 yl = dec_plane(__ldg(pl + 2), a.y), yh = dec_plane(__ldg(pl + 3), ty);
    float4 zl = dec_plane(__ldg(pl + 4), a.z), zh = dec_plane(__ldg(pl + 5), tz);
    uint32_t m = 0;
    m |= slab_hit(xl.x, xh.x, yl.x, yh.x, zl.x, zh.x, o, di, tmax) ? 1u : 0u;
    m |= slab_hit(xl.y, xh.y, yl.y, yh.y, zl.y, zh.y, o, di, tmax) ? 2u : 0u;
    m |= slab_hit(xl.z, xh.z, yl.z, yh.z, zl.z, zh.z, o, di, tmax) ? 4u : 0u;
    m |= slab_hit(xl.w, xh.w, yl.w, yh.w, zl.w, zh.w, o, di, tmax) ? 8u : 0u;
    return m;
}
DI uint32_t node_hits_h(const GScene &S, uint32_t ni, V3 o, V3 di, float tmax, float time, uint32_t oct, bool safe,
                        uint32_t &code, uint32_t &count, uint4 &child) {
    const GNodeH *n = S.nodes_h + ni;
    float4 a = __ldg(&n->anchor);
    uint32_t meta = __float_as_uint(a.w);
    if (meta & PSY_NODEH_F32)  // motion keys or offsets past the f16 range: the f32 node
        return node_hits(S, ni, o, di, tmax, time, oct, safe, code, count, child);
    child = __ldg(&n->child);
    code = meta & 0xFFu;
    count = (meta >> 8) & 0xFFu;
    return fp16_hits(n, a, o, di, tmax, oct, safe) & ((1u << count) - 1u);
}

// World-space vertices of triangle `tri` (global index) of mesh `M` at
// `time`, transformed into world space by `mat` when the instance has a
// transform (the reference tests triangles in world space).
DI void fetch_tri(const GScene &S, const GMesh &M, uint32_t tri, float time, bool xf, const Xf &mat, V3 &p0, V3 &p1,
                  V3 &p2) {
    if (M.ts == 1) {
        const float4 *t = S.tris + 3 * (size_t)tri;
        p0 = v3(__ldg(t)); p1 = v3(__ldg(t + 1)); p2 = v3(__ldg(t + 2));
    } else {
        uint4 ix = __ldg(S.tri_idx + tri);
        const float4 *vb = S.verts + M.vert_base;
        p0 = lerp_slice_v3(vb + (size_t)ix.x * M.ts, M.ts, time);
        p1 = lerp_slice_v3(vb + (size_t)ix.y * M.ts, M.ts, time);
        p2 = lerp_slice_v3(vb + (size_t)ix.z * M.ts, M.ts, time);
    }
    if (xf) {
        p0 = xf_point(p0, mat);
        p1 = xf_point(p1, mat);
        p2 = xf_point(p2, mat);
    }
}

// Object->world matrix used for an instance's triangles at `time`.
DI Xf instance_mat(const GScene &S, const GInstance &in, float time) {
    if (in.xc == 1) return xf_load(S.xforms_inv + 3 * in.xinv);
    return xf_inverse(lerp_slice_xf(S.xforms + 3 * in.xs, in.xc, time));
}

// Rectangle light test (RectangleLight::intersect_rays).
DI bool rect_hit(const GScene &S, const GInstance &in, V3 o, V3 d, float tmax, float time, float &t, float &b0,
                 float &b1, float &b2, uint32_t &which) {
    const GLight L = S.lights[in.obj];
    float w = light_dim(S, L, 0, time), h = light_dim(S, L, 1, time);
    Xf si = light_inverse(S, in, instance_xf_at(S, in, time));
    V3 p1, p2, p3, p4;
    rect_corners(w, h, si, &p1, &p2, &p3, &p4);
    TriPre pre = tri_precompute(d);
    if (tri_intersect(o, pre, tmax, p1, p2, p3, t, b0, b1, b2) && t < tmax) { which = 0; return true; }
    if (tri_intersect(o, pre, tmax, p3, p4, p1, t, b0, b1, b2) && t < tmax) { which = 1; return true; }
    return false;
}
// Sphere light test (SphereLight::intersect_rays).  `ol` is the ray origin
// in the light's local space.
DI bool sphere_hit(const GScene &S, const GInstance &in, V3 ol, V3 d, float tmax, float time, float &t_out) {
    const GLight L = S.lights[in.obj];
    Xf xf = instance_xf_at(S, in, time);
    float radius = light_dim(S, L, 0, time);
    V3 dir = xf_vector(d, xf);
    float a = length2(dir);
    float b = 2.0f * dot(dir, ol);
    float c = length2(ol) - (radius * radius);
    float disc = (b * b) - (4.0f * a * c);
    if (disc < 0.0f) return false;
    disc = sqrtf(disc);
    float q = (b < 0.0f) ? -0.5f * (b - disc) : -0.5f * (b + disc);
    float t0 = q / a;
    float t1 = (q != 0.0f) ? c / q : tmax;
    if (t0 > t1) { float tt = t0; t0 = t1; t1 = tt; }
    if (t0 > tmax || t1 <= 0.0f) return false;
    if (t0 > 0.0f) t_out = t0;
    else if (t1 <= tmax) t_out = t1;
    else return false;
    return true;
}

// Child push by table: for each (ray octant, traversal code) a push row
// (g_push_row) and for each row and 4-bit hit mask a 16-bit entry
// (g_push_lut): bits 0-1 the child to descend into, bits 2-7 up to three
// children to push (deepest first), bits 8-10 how many, bit 11 set when any
// child was hit.  The entries follow the traversal table's front-to-back
// order and ignore mask bits past the node's child count.
#define PSY_PUSH_ROWS 32
// Global memory (not __constant__): every block copies them with one
// coalesced 16-byte load per thread, where per-lane indexed reads of
// constant memory would be serialized across the warp.
static __device__ __align__(16) uint8_t g_push_row[8 * 48];
static __device__ __align__(16) uint16_t g_push_lut[PSY_PUSH_ROWS * 16];

// Shared-memory copies of the push tables (row: 384 bytes, lut: 1 KB; both
// 16-byte aligned); blocks of at least 88 threads.
DI void load_push_tables(uint8_t *row, uint16_t *lut) {
    int t = threadIdx.x;
    if (t < 24)
        reinterpret_cast<uint4 *>(row)[t] = reinterpret_cast<const uint4 *>(g_push_row)[t];
    else if (t < 24 + 64)
        reinterpret_cast<uint4 *>(lut)[t - 24] = reinterpret_cast<const uint4 *>(g_push_lut)[t - 24];
    __syncthreads();
}

DI uint32_t sel4(const uint4 &c, uint32_t i) {
    uint32_t lo = (i & 1u) ? c.y : c.x, hi = (i & 1u) ? c.w : c.z;
    return (i & 2u) ? hi : lo;
}

// Corners of rectangle light triangle `which` (0: p1 p2 p3, 1: p3 p4 p1), as
// rect_hit builds them.
DI void rect_tri(const GScene &S, const GInstance &in, float time, uint32_t which, V3 &a, V3 &b, V3 &c) {
    const GLight L = S.lights[in.obj];
    float w = light_dim(S, L, 0, time), h = light_dim(S, L, 1, time);
    Xf si = light_inverse(S, in, instance_xf_at(S, in, time));
    V3 p1, p2, p3, p4;
    rect_corners(w, h, si, &p1, &p2, &p3, &p4);
    if (which == 0) { a = p1; b = p2; c = p3; }
    else { a = p3; b = p4; c = p1; }
}

// The world-level ray of Tracer::trace (update_local with the identity):
// the same arithmetic as transforming by the identity matrix.
DI V3 world_origin(V3 o) { return xf_point(o, xf_identity()); }
DI V3 world_dir_inv(V3 d) { return recip(xf_vector(d, xf_identity())); }

// fetch_tri with the instance matrix read from a shared-memory slot (three
// float4 rows, the layout of Xf).
DI void fetch_tri_xfm(const GScene &S, uint32_t mts, uint32_t mvb, uint32_t tri, float time, bool xf,
                      const float4 *xfm, V3 &p0, V3 &p1, V3 &p2) {
    if (mts == 1) {
        const float4 *t = S.tris + 3 * (size_t)tri;
        p0 = v3(__ldg(t)); p1 = v3(__ldg(t + 1)); p2 = v3(__ldg(t + 2));
    } else {
        uint4 ix = __ldg(S.tri_idx + tri);
        const float4 *vb = S.verts + mvb;
        p0 = lerp_slice_v3(vb + (size_t)ix.x * mts, mts, time);
        p1 = lerp_slice_v3(vb + (size_t)ix.y * mts, mts, time);
        p2 = lerp_slice_v3(vb + (size_t)ix.z * mts, mts, time);
    }
    if (xf) {
        float4 a = xfm[0], b = xfm[1], c = xfm[2];
        Xf mat;
        mat.m[0] = a.x; mat.m[1] = a.y; mat.m[2] = a.z; mat.m[3] = a.w;
        mat.m[4] = b.x; mat.m[5] = b.y; mat.m[6] = b.z; mat.m[7] = b.w;
        mat.m[8] = c.x; mat.m[9] = c.y; mat.m[10] = c.z; mat.m[11] = c.w;
        p0 = xf_point(p0, mat);
        p1 = xf_point(p1, mat);
        p2 = xf_point(p2, mat);
    }
}

// Fills the hit record once traversal is done: t is the final max_t (each
// accepted hit set max_t to its t), and the barycentrics come from repeating
// the winning triangle test -- the same arithmetic on the same inputs, with
// an unbounded max_t, which only removes the upper bound the test already
// passed.  hprim: BVH-order triangle (surface), 0 / 1 (rectangle light
// triangle) or ~0 (sphere light).
template <bool STATIC>
DI void finish_hit(const GScene &S, V3 o, const TriPre &pre, float time, float tmax, uint32_t hkind, uint32_t hprim,
                   uint32_t hslot, HitRec &hit) {
    hit.kind = hkind;
    if (hkind == PSY_HIT_MISS_K) return;
    hit.slot = hslot;
    hit.t = tmax;
    hit.b0 = hit.b1 = hit.b2 = 0.0f;
    const float inf = __int_as_float(0x7f800000);
    float t2, b0, b1, b2;
    const GInstance in = S.instances[hslot];
    if (hkind == PSY_HIT_SURFACE_K) {
        hit.prim = hprim;
        V3 p0, p1, p2;
        if (STATIC) {  // static, untransformed meshes: pre-gathered triangles
            const float4 *tp = S.tris + 3 * (size_t)hprim;
            p0 = v3(__ldg(tp)); p1 = v3(__ldg(tp + 1)); p2 = v3(__ldg(tp + 2));
        } else {
            const GMesh M = S.meshes[in.obj];
            bool xf = in.xc != 0;
            Xf mat = xf ? instance_mat(S, in, time) : xf_identity();
            fetch_tri(S, M, hprim, time, xf, mat, p0, p1, p2);
        }
        if (tri_intersect(o, pre, inf, p0, p1, p2, t2, b0, b1, b2)) { hit.b0 = b0; hit.b1 = b1; hit.b2 = b2; }
    } else if (hprim == 0xFFFFFFFFu) {
        hit.prim = 0;  // sphere light
    } else {
        hit.prim = hprim;
        V3 a, b, c;
        rect_tri(S, in, time, hprim, a, b, c);
        if (tri_intersect(o, pre, inf, a, b, c, t2, b0, b1, b2)) { hit.b0 = b0; hit.b1 = b1; hit.b2 = b2; }
    }
}

// Traversal work counters (ray x node tests and ray x triangle tests).
struct TraceCount {
    uint32_t nodes, tris;
};

// Copies the traversal table into shared memory (per-lane indexed reads of
// __constant__ memory would serialize across the warp).
DI void load_traversal_table(uint8_t *smem) {
    for (int i = threadIdx.x; i < 8 * 48; i += blockDim.x) smem[i] = (&c_traversal_table[0][0])[i];
    __syncthreads();
}

// The general traversal's per-thread shared-memory slot: the entered
// instance's object-to-world matrix (3 float4), and with PSY_RAY_SHARED (the
// default) the world ray's origin, direction and triangle-test precompute
// (3 float4), which the loop reads only at instance entry and exit and at
// leaves -- kept there instead of in registers the node tests need.  At 8
// blocks per SM (64 registers) the spill stores fall from 520 to 396 bytes
// and the motion + instancing frame (general kernel) runs 212.7 -> 228.0 M
// samples/s.  Only the register-limited variants (more than 4 blocks per
// SM) use it: with the compiler's own budget nothing spills and the extra
// shared loads only cost.  The static-scene traversal gains nothing from it
// (its spills do not fall) and keeps its ray in registers.
#ifndef PSY_RAY_SHARED
#define PSY_RAY_SHARED 1
#endif
#define PSY_XFM_SLOT(MINB) ((PSY_RAY_SHARED && (MINB) > 4) ? 6 : 3)
DI float4 pack_pre(const TriPre &p) {
    return make_float4(p.sx, p.sy, p.sz, __int_as_float(p.ix | (p.iy << 2) | (p.iz << 4)));
}
DI TriPre unpack_pre(float4 v) {
    TriPre p;
    int k = __float_as_int(v.w);
    p.ix = k & 3; p.iy = (k >> 2) & 3; p.iz = (k >> 4) & 3;
    p.sx = v.x; p.sy = v.y; p.sz = v.z;
    return p;
}

// Trace one ray.  `occl`: any-hit (shadow ray).  Returns false on stack
// overflow (the scene needs a deeper stack than STACK).  The hit keeps only
// its kind, triangle (or light triangle) and instance while traversing
// (finish_hit completes it).  Children are pushed through the push tables:
// prow_tab is the per-octant push-row table, lut the entries
// (load_push_tables).  xfm: this thread's three-float4 shared-memory slot
// for the entered instance's object-to-world matrix.
template <int STACK, bool COUNT = false, bool RSH = false>
DI bool trace_ray(const GScene &S, const uint8_t *prow_tab, const uint16_t *lut, float4 *xfm, V3 o, V3 d, float tmax,
                  float time, bool occl, HitRec &hit, TraceCount *cnt = nullptr) {
    hit.kind = PSY_HIT_MISS_K;
    if (S.top_root == PSY_REF_NONE) return true;
    // world level: update_local(identity); recomputed when leaving an
    // instance rather than kept
    V3 lo = world_origin(o), ldi = world_dir_inv(d);
    uint32_t oct = ray_code(ldi);
    const uint8_t *prow = prow_tab + 48 * oct;
    // slab_safe holds for the whole ray in a space (tmax only shrinks to a finite t)
    bool safe = S.ordered_slabs && slab_safe(lo, ldi, tmax);
    // 3 spare entries take the unconditional stores of the child push
    uint32_t stack[STACK + 4];
    int sp = 0;
    uint32_t cur = S.top_root;
    bool in_inst = false;
    uint32_t slot = 0, hkind = PSY_HIT_MISS_K, hprim = 0, hslot = 0;
    uint32_t mts = 1, mvb = 0;  // entered mesh: vertex time samples and first vertex
    bool has_xf = false;
    const TriPre pre0 = tri_precompute(d);
    if (RSH) {
        xfm[3] = make_float4(o.x, o.y, o.z, 0.0f);
        xfm[4] = make_float4(d.x, d.y, d.z, 0.0f);
        xfm[5] = pack_pre(pre0);
    }
    // the world ray and the precompute, from the slot or the registers
    auto RO = [&]() { return RSH ? v3(xfm[3]) : o; };
    auto RD = [&]() { return RSH ? v3(xfm[4]) : d; };
    auto PRE = [&]() { return RSH ? unpack_pre(xfm[5]) : pre0; };
    while (true) {
        // descend internal nodes
        while (!psy_is_leaf(cur)) {
            uint32_t code, count;
            uint4 ch;
            uint32_t m = S.use_fp16 ? node_hits_h(S, cur, lo, ldi, tmax, time, oct, safe, code, count, ch)
                                    : node_hits(S, cur, lo, ldi, tmax, time, oct, safe, code, count, ch);
            (void)count;
            if (COUNT) cnt->nodes++;
            // children in the table's front-to-back order: descend into the
            // first hit child, push the others (deepest first); only the np
            // entries kept are stored (local-memory stores write through to
            // L2, so unused ones cost traffic)
            uint32_t e = lut[16u * prow[code] + m];
            if (!(e & 0x800u)) goto pop;
            int np = (int)((e >> 8) & 7u);
            if (sp + np > STACK) return false;
            if (np > 0) stack[sp] = sel4(ch, (e >> 2) & 3u);
            if (np > 1) stack[sp + 1] = sel4(ch, (e >> 4) & 3u);
            if (np > 2) stack[sp + 2] = sel4(ch, (e >> 6) & 3u);
            sp += np;
            cur = sel4(ch, e & 3u);
        }
        // leaf
        if (!in_inst) {
            slot = psy_leaf_first(cur);
            GInstance in = S.instances[slot];
            if (in.kind == PSY_INST_MESH) {
                const GMesh mesh = S.meshes[in.obj];
                mts = mesh.ts;
                mvb = mesh.vert_base;
                has_xf = in.xc != 0;
                if (has_xf) {
                    Xf x = lerp_slice_xf(S.xforms + 3 * in.xs, in.xc, time);
                    lo = xf_point(RO(), x);
                    ldi = recip(xf_vector(RD(), x));
                    // object -> world matrix of the triangles: kept in this
                    // thread's shared-memory slot, read by each triangle fetch
                    Xf mat = instance_mat(S, in, time);
                    xfm[0] = make_float4(mat.m[0], mat.m[1], mat.m[2], mat.m[3]);
                    xfm[1] = make_float4(mat.m[4], mat.m[5], mat.m[6], mat.m[7]);
                    xfm[2] = make_float4(mat.m[8], mat.m[9], mat.m[10], mat.m[11]);
                }
                if (sp >= STACK) return false;
                stack[sp++] = PSY_REF_NONE;  // leave-instance marker
                in_inst = true;
                oct = ray_code(ldi);
                prow = prow_tab + 48 * oct;
                safe = S.ordered_slabs && slab_safe(lo, ldi, tmax);
                cur = mesh.root;
                continue;
            } else if (in.kind == PSY_INST_RECT) {
                float t, b0, b1, b2;
                uint32_t which;
                if (rect_hit(S, in, RO(), RD(), tmax, time, t, b0, b1, b2, which)) {
                    if (occl) { hit.kind = PSY_HIT_OCCLUDE_K; return true; }
                    hkind = PSY_HIT_LIGHT_K; hprim = which; hslot = slot;
                    tmax = t;
                }
            } else {
                Xf x = instance_xf_at(S, in, time);
                V3 ol = in.xc ? xf_point(RO(), x) : lo;  // lo: the world origin at this level
                float t;
                if (sphere_hit(S, in, ol, RD(), tmax, time, t)) {
                    if (occl) { hit.kind = PSY_HIT_OCCLUDE_K; return true; }
                    hkind = PSY_HIT_LIGHT_K; hprim = 0xFFFFFFFFu; hslot = slot;
                    tmax = t;
                }
            }
        } else {
            uint32_t first = psy_leaf_first(cur), ntri = psy_leaf_count(cur);
            for (uint32_t k = 0; k < ntri; k++) {
                uint32_t tri = first + k;
                V3 p0, p1, p2;
                fetch_tri_xfm(S, mts, mvb, tri, time, has_xf, xfm, p0, p1, p2);
                float t, b0, b1, b2;
                if (COUNT) cnt->tris++;
                if (tri_intersect(RO(), PRE(), tmax, p0, p1, p2, t, b0, b1, b2)) {
                    if (occl) { hit.kind = PSY_HIT_OCCLUDE_K; return true; }
                    hkind = PSY_HIT_SURFACE_K; hprim = tri; hslot = slot;
                    tmax = t;
                }
            }
        }
    pop:
        while (true) {
            if (sp == 0) goto done;
            cur = stack[--sp];
            if (cur != PSY_REF_NONE) break;
            // leaving the instance: back to world space
            in_inst = false;
            lo = world_origin(RO());
            ldi = world_dir_inv(RD());
            oct = ray_code(ldi);
            prow = prow_tab + 48 * oct;
            safe = S.ordered_slabs && slab_safe(lo, ldi, tmax);
        }
    }
done:
    finish_hit<false>(S, RO(), PRE(), time, tmax, hkind, hprim, hslot, hit);
    return true;
}

// ------------------------------------------------------------------ short stack in shared memory
// Threads per block of the traversal kernels.
#define PSY_TRACE_BLOCK 128
// Entries of each thread's traversal stack kept in shared memory (0: the
// whole stack in local memory).  Measured on the mesh-stress frame (static
// traversal, 10 blocks per SM): 16 entries 473.9, 8 entries 472.9, none
// 494.3 M samples/s -- the L1 serves the top of a local-memory stack well,
// and the shared-memory columns take L1 capacity the node loads need -- so
// the default keeps the stack in local memory.
#ifndef PSY_SSTACK
#define PSY_SSTACK 0
#endif
// Traversal stack of one thread: entries 0 .. K-1 in shared memory, in this
// thread's column of a block-wide array (entry j at sh[j * PSY_TRACE_BLOCK],
// so the 32 lanes of a warp use 32 different banks whatever their depths),
// entries K .. STACK + 3 in local memory.
template <int STACK, int K>
struct TravStack {
    uint32_t *sh;
    uint32_t loc[STACK + 4 - K];
    DI void set(int i, uint32_t v) {
        if (K > 0 && i < K) sh[i * PSY_TRACE_BLOCK] = v;
        else loc[i - K] = v;
    }
    DI uint32_t get(int i) const { return (K > 0 && i < K) ? sh[i * PSY_TRACE_BLOCK] : loc[i - K]; }
};

// ------------------------------------------------------------------ static-scene traversal
// Scenes whose meshes are all static and untransformed, whose nodes carry no
// motion keys and whose child boxes are ordered (GScene::static_fast) take a
// traversal with a much smaller live state than trace_ray: no local space,
// no instance matrix, no mesh record, and the hit keeps only its kind,
// triangle and instance (t is the final max_t; the barycentrics are
// recomputed once at the end by repeating the winning test, which is
// deterministic and passes with an unbounded max_t).  Visit order, node and
// triangle tests and their arithmetic are trace_ray's, so hits are identical.
//
// Child hit mask of a static node (no motion keys; the count mask is applied
// by the push table).  safe: slab_safe holds for the ray (boxes are ordered).
DI uint32_t node_hits_static(const GScene &S, uint32_t ni, V3 o, V3 di, float tmax, uint32_t oct, bool safe,
                             uint32_t &code, uint4 &child) {
    const GNode *n = S.nodes + ni;
    const float4 *bb = reinterpret_cast<const float4 *>(n);
    child = __ldg(&n->child);
    code = __ldg(&n->meta.z) & 0xFFu;
    if (safe) {
        uint32_t sx = oct & 1u, sy = (oct >> 1) & 1u, sz = (oct >> 2) & 1u;
        float4 nx = __ldg(bb + sx), fx = __ldg(bb + (sx ^ 1u));
        float4 ny = __ldg(bb + 2 + sy), fy = __ldg(bb + 2 + (sy ^ 1u));
        float4 nz = __ldg(bb + 4 + sz), fz = __ldg(bb + 4 + (sz ^ 1u));
        float tnx[4], tfx[4], tny[4], tfy[4], tnz[4], tfz[4];
        f32x2 ox = pk2(o.x, o.x), oy = pk2(o.y, o.y), oz = pk2(o.z, o.z);
        f32x2 dx = pk2(di.x, di.x), dy = pk2(di.y, di.y), dz = pk2(di.z, di.z);
        slab_axis4(nx, ox, dx, tnx); slab_axis4(fx, ox, dx, tfx);
        slab_axis4(ny, oy, dy, tny); slab_axis4(fy, oy, dy, tfy);
        slab_axis4(nz, oz, dz, tnz); slab_axis4(fz, oz, dz, tfz);
        uint32_t m = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float far_t = fminf(fmin3f(tfx[c], tfy[c], tfz[c]) * PSY_BBOX_MAXT_ADJUST, tmax);
            float near_t = fmax3f(tnx[c], tny[c], fmaxf(tnz[c], 0.0f));
            m |= near_t < far_t ? (1u << c) : 0u;
        }
        return m;
    }
    float4 xl = __ldg(bb), xh = __ldg(bb + 1), yl = __ldg(bb + 2), yh = __ldg(bb + 3), zl = __ldg(bb + 4),
           zh = __ldg(bb + 5);
    uint32_t m = 0;
    m |= slab_hit(xl.x, xh.x, yl.x, yh.x, zl.x, zh.x, o, di, tmax) ? 1u : 0u;
    m |= slab_hit(xl.y, xh.y, yl.y, yh.y, zl.y, zh.y, o, di, tmax) ? 2u : 0u;
    m |= slab_hit(xl.z, xh.z, yl.z, yh.z, zl.z, zh.z, o, di, tmax) ? 4u : 0u;
    m |= slab_hit(xl.w, xh.w, yl.w, yh.w, zl.w, zh.w, o, di, tmax) ? 8u : 0u;
    return m;
}

// The static-scene test on an FP16 node (nodes flagged PSY_NODEH_F32 use
// their f32 copy); the count mask is applied by the push table.
DI uint32_t node_hits_static_h(const GScene &S, uint32_t ni, V3 o, V3 di, float tmax, uint32_t oct, bool safe,
                               uint32_t &code, uint4 &child) {
    const GNodeH *n = S.nodes_h + ni;
    float4 a = __ldg(&n->anchor);
    uint32_t meta = __float_as_uint(a.w);
    if (meta & PSY_NODEH_F32) return node_hits_static(S, ni, o, di, tmax, oct, safe, code, child);
    child = __ldg(&n->child);
    code = meta & 0xFFu;
    return fp16_hits(n, a, o, di, tmax, oct, safe);
}

// Static-scene triangle leaf: tests its (up to three) triangles.
DI void static_leaf(const GScene &S, uint32_t leaf, V3 o, const TriPre &pre, uint32_t slot, float &tmax,
                    uint32_t &hkind, uint32_t &hprim, uint32_t &hslot, bool occl, bool &occluded) {
    uint32_t first = psy_leaf_first(leaf), ntri = psy_leaf_count(leaf);
    for (uint32_t k = 0; k < ntri; k++) {
        uint32_t tri = first + k;
        const float4 *tp = S.tris + 3 * (size_t)tri;
        V3 p0 = v3(__ldg(tp)), p1 = v3(__ldg(tp + 1)), p2 = v3(__ldg(tp + 2));
        float t, b0, b1, b2;
        if (tri_intersect(o, pre, tmax, p0, p1, p2, t, b0, b1, b2)) {
            if (occl) { occluded = true; return; }
            hkind = PSY_HIT_SURFACE_K; hprim = tri; hslot = slot;
            tmax = t;
        }
    }
}

// SPEC: speculative traversal (Aila & Laine, "Understanding the Efficiency
// of Ray Traversal on GPUs", 2009): a closest-hit ray that reaches a
// triangle leaf postpones it and keeps traversing the nodes on its stack
// while other lanes of the warp are still looking for a leaf, so the warp
// tests nodes and triangles with more lanes at a time.  The postponed leaf is
// still tested before everything after it in the visit order; the nodes
// tested meanwhile use the max_t of before the leaf, so a ray can visit more
// nodes and triangles than the reference, and the closest hit differs only
// where a triangle the reference culls lies at exactly the same t (a tie).
// H16: the scene's nodes are read from the FP16 copy.  sstack: this thread's
// column of the block's shared-memory stack (PSY_SSTACK entries).
template <int STACK, bool SPEC = false, bool H16 = false>
DI bool trace_ray_static(const GScene &S, const uint8_t *prow_tab, const uint16_t *lut, uint32_t *sstack, V3 o, V3 d,
                         float tmax, float time, bool occl, HitRec &hit) {
    hit.kind = PSY_HIT_MISS_K;
    if (S.top_root == PSY_REF_NONE) return true;
    Xf ident = xf_identity();
    V3 wo = xf_point(o, ident);
    V3 di = recip(xf_vector(d, ident));
    uint32_t oct = ray_code(di);
    const uint8_t *prow = prow_tab + 48 * oct;
    bool safe = slab_safe(wo, di, tmax);
    TravStack<STACK, PSY_SSTACK> stack;
    stack.sh = sstack;
    int sp = 0;
    uint32_t cur = S.top_root;
    bool in_inst = false;
    uint32_t slot = 0, hkind = PSY_HIT_MISS_K, hprim = 0, hslot = 0;
    TriPre pre = tri_precompute(d);
    const bool spec = SPEC && !occl;  // shadow rays stop at their first hit instead
    uint32_t pleaf = PSY_REF_NONE;     // postponed triangle leaf (SPEC)
    bool occluded = false;
    while (true) {
        while (!psy_is_leaf(cur)) {
            uint32_t code;
            uint4 ch;
            uint32_t m = H16 ? node_hits_static_h(S, cur, wo, di, tmax, oct, safe, code, ch)
                             : node_hits_static(S, cur, wo, di, tmax, oct, safe, code, ch);
            uint32_t e = lut[16u * prow[code] + m];
            if (!(e & 0x800u)) {
                if (!spec || pleaf == PSY_REF_NONE) goto pop;
                // speculating: go on only with a node of this mesh on top
                if (sp > 0 && !psy_is_leaf(stack.get(sp - 1))) {
                    cur = stack.get(--sp);
                } else {
                    cur = PSY_REF_NONE;
                    break;
                }
            } else {
                int np = (int)((e >> 8) & 7u);
                if (sp + np > STACK) return false;
                // only the np entries kept are stored (local-memory stores
                // write through to L2, so unused ones cost traffic)
                if (np > 0) stack.set(sp, sel4(ch, (e >> 2) & 3u));
                if (np > 1) stack.set(sp + 1, sel4(ch, (e >> 4) & 3u));
                if (np > 2) stack.set(sp + 2, sel4(ch, (e >> 6) & 3u));
                sp += np;
                cur = sel4(ch, e & 3u);
            }
            if (spec) {
                if (in_inst && pleaf == PSY_REF_NONE && psy_is_leaf(cur)) {
                    pleaf = cur;  // postpone the first triangle leaf
                    if (sp > 0 && !psy_is_leaf(stack.get(sp - 1))) {
                        cur = stack.get(--sp);
                    } else {
                        cur = PSY_REF_NONE;
                        break;
                    }
                }
                // stop once every lane still here holds a leaf
                if (!__any_sync(__activemask(), pleaf == PSY_REF_NONE)) break;
            }
        }
        if (SPEC && pleaf != PSY_REF_NONE) {
            static_leaf(S, pleaf, o, pre, slot, tmax, hkind, hprim, hslot, false, occluded);
            pleaf = PSY_REF_NONE;
            if (!psy_is_leaf(cur)) continue;  // stopped by the vote: traverse on from cur
            if (cur == PSY_REF_NONE) goto pop;
            // else cur is the next triangle leaf of the same mesh
        }
        if (!in_inst) {
            slot = psy_leaf_first(cur);
            GInstance in = S.instances[slot];
            if (in.kind == PSY_INST_MESH) {
                if (sp >= STACK) return false;
                stack.set(sp++, PSY_REF_NONE);  // leave-instance marker
                in_inst = true;
                safe = slab_safe(wo, di, tmax);
                cur = S.meshes[in.obj].root;
                continue;
            } else if (in.kind == PSY_INST_RECT) {
                float t, b0, b1, b2;
                uint32_t which;
                if (rect_hit(S, in, o, d, tmax, time, t, b0, b1, b2, which)) {
                    if (occl) { hit.kind = PSY_HIT_OCCLUDE_K; return true; }
                    hkind = PSY_HIT_LIGHT_K; hprim = which; hslot = slot;
                    tmax = t;
                }
            } else {
                Xf x = instance_xf_at(S, in, time);
                V3 ol = in.xc ? xf_point(o, x) : wo;
                float t;
                if (sphere_hit(S, in, ol, d, tmax, time, t)) {
                    if (occl) { hit.kind = PSY_HIT_OCCLUDE_K; return true; }
                    hkind = PSY_HIT_LIGHT_K; hprim = 0xFFFFFFFFu; hslot = slot;  // prim 0, no barycentrics
                    tmax = t;
                }
            }
        } else {
            static_leaf(S, cur, o, pre, slot, tmax, hkind, hprim, hslot, occl, occluded);
            if (occluded) { hit.kind = PSY_HIT_OCCLUDE_K; return true; }
        }
    pop:
        while (true) {
            if (sp == 0) goto done;
            cur = stack.get(--sp);
            if (cur != PSY_REF_NONE) break;
            in_inst = false;  // leaving the instance (world space is the instance's space)
            safe = slab_safe(wo, di, tmax);
        }
    }
done:
    finish_hit<true>(S, o, pre, time, tmax, hkind, hprim, hslot, hit);
    return true;
}

// ------------------------------------------------------------------ static-scene traversal with lane refill
// trace_ray_static's traversal cut into steps (descend to a leaf, test it,
// pop), so that a persistent kernel can give a lane whose ray finished the
// next ray of its queue while the other lanes of the warp go on (Aila &
// Laine 2009).  Node and triangle tests, visit order and hit records are
// trace_ray_static's, so hits are identical.
struct SLane {
    V3 o, d;        // the ray as given
    V3 wo, di;      // world-level origin and inverse direction (identity transform, as trace_ray_static)
    float tmax, time;
    TriPre pre;
    uint32_t cur, slot, hkind, hprim, hslot;
    int sp;
    uint32_t oct;
    bool occl, in_inst, safe;
};
DI void slane_init(const GScene &S, SLane &L, V3 o, V3 d, float tmax, float time, bool occl) {
    Xf ident = xf_identity();
    L.o = o; L.d = d;
    L.wo = xf_point(o, ident);
    L.di = recip(xf_vector(d, ident));
    L.tmax = tmax; L.time = time;
    L.pre = tri_precompute(d);
    L.cur = S.top_root;
    L.slot = 0; L.hkind = PSY_HIT_MISS_K; L.hprim = 0; L.hslot = 0;
    L.sp = 0;
    L.oct = ray_code(L.di);
    L.occl = occl; L.in_inst = false;
    L.safe = slab_safe(L.wo, L.di, tmax);
}
// One step of lane L.  Returns 0 to go on, 1 when the ray is finished (hit
// filled), -1 on stack overflow.
template <int STACK, bool H16>
DI int slane_step(const GScene &S, const uint8_t *prow_tab, const uint16_t *lut, SLane &L, uint32_t *stack,
                  HitRec &hit) {
    if (L.cur == PSY_REF_NONE) {  // empty scene
        hit.kind = PSY_HIT_MISS_K;
        return 1;
    }
    const uint8_t *prow = prow_tab + 48 * L.oct;
    while (!psy_is_leaf(L.cur)) {
        uint32_t code;
        uint4 ch;
        uint32_t m = H16 ? node_hits_static_h(S, L.cur, L.wo, L.di, L.tmax, L.oct, L.safe, code, ch)
                         : node_hits_static(S, L.cur, L.wo, L.di, L.tmax, L.oct, L.safe, code, ch);
        uint32_t e = lut[16u * prow[code] + m];
        if (!(e & 0x800u)) goto pop;
        int np = (int)((e >> 8) & 7u);
        if (L.sp + np > STACK) return -1;
        if (np > 0) stack[L.sp] = sel4(ch, (e >> 2) & 3u);
        if (np > 1) stack[L.sp + 1] = sel4(ch, (e >> 4) & 3u);
        if (np > 2) stack[L.sp + 2] = sel4(ch, (e >> 6) & 3u);
        L.sp += np;
        L.cur = sel4(ch, e & 3u);
    }
    if (!L.in_inst) {
        L.slot = psy_leaf_first(L.cur);
        GInstance in = S.instances[L.slot];
        if (in.kind == PSY_INST_MESH) {
            if (L.sp >= STACK) return -1;
            stack[L.sp++] = PSY_REF_NONE;  // leave-instance marker
            L.in_inst = true;
            L.safe = slab_safe(L.wo, L.di, L.tmax);
            L.cur = S.meshes[in.obj].root;
            return 0;
        } else if (in.kind == PSY_INST_RECT) {
            float t, b0, b1, b2;
            uint32_t which;
            if (rect_hit(S, in, L.o, L.d, L.tmax, L.time, t, b0, b1, b2, which)) {
                if (L.occl) { hit.kind = PSY_HIT_OCCLUDE_K; return 1; }
                L.hkind = PSY_HIT_LIGHT_K; L.hprim = which; L.hslot = L.slot;
                L.tmax = t;
            }
        } else {
            Xf x = instance_xf_at(S, in, L.time);
            V3 ol = in.xc ? xf_point(L.o, x) : L.wo;
            float t;
            if (sphere_hit(S, in, ol, L.d, L.tmax, L.time, t)) {
                if (L.occl) { hit.kind = PSY_HIT_OCCLUDE_K; return 1; }
                L.hkind = PSY_HIT_LIGHT_K; L.hprim = 0xFFFFFFFFu; L.hslot = L.slot;
                L.tmax = t;
            }
        }
    } else {
        bool occluded = false;
        static_leaf(S, L.cur, L.o, L.pre, L.slot, L.tmax, L.hkind, L.hprim, L.hslot, L.occl, occluded);
        if (occluded) { hit.kind = PSY_HIT_OCCLUDE_K; return 1; }
    }
pop:
    while (true) {
        if (L.sp == 0) {
            finish_hit<true>(S, L.o, L.pre, L.time, L.tmax, L.hkind, L.hprim, L.hslot, hit);
            return 1;
        }
        L.cur = stack[--L.sp];
        if (L.cur != PSY_REF_NONE) break;
        L.in_inst = false;  // leaving the instance (world space is the instance's space)
        L.safe = slab_safe(L.wo, L.di, L.tmax);
    }
    return 0;
}

}  // namespace psyd

namespace psyd {

// ------------------------------------------------------------------ persistent traversal
// Per-lane traversal state, kept in registers across the loop of the
// persistent kernel; the stack lives in local memory and persists too.
struct Lane {
    V3 o, d;            // world ray
    V3 lo, ldi;         // ray in the current space (world or instance local)
    float tmax, time;
    TriPre pre;
    Xf mat;             // object->world of the current instance (has_xf)
    uint32_t cur;       // node or leaf reference to process next
    uint32_t slot;      // current instance slot
    uint32_t mts, mvb;  // current mesh: vertex time samples and vertex base
    int sp;
    uint8_t occl, in_inst, has_xf, octant, safe, ordered;
    HitRec hit;
};

DI void lane_init(const GScene &S, Lane &L, V3 o, V3 d, float tmax, float time, bool occl) {
    Xf ident = xf_identity();
    L.o = o;
    L.d = d;
    L.lo = xf_point(o, ident);
    L.ldi = recip(xf_vector(d, ident));
    L.tmax = tmax;
    L.time = time;
    L.pre = tri_precompute(d);
    L.cur = S.top_root;
    L.slot = 0;
    L.mts = 1;
    L.mvb = 0;
    L.sp = 0;
    L.occl = occl ? 1 : 0;
    L.in_inst = 0;
    L.has_xf = 0;
    L.octant = (uint8_t)ray_code(L.ldi);
    L.ordered = S.ordered_slabs ? 1 : 0;
    L.safe = (L.ordered && slab_safe(L.lo, L.ldi, tmax)) ? 1 : 0;
    L.hit.kind = PSY_HIT_MISS_K;
    L.hit.prim = 0;
    L.hit.slot = 0;
    L.hit.t = 0.0f;
    L.hit.b0 = L.hit.b1 = L.hit.b2 = 0.0f;
}

// Pops the next reference; returns false when the ray is finished.
template <int STACK>
DI bool lane_pop(Lane &L, const uint32_t *stack) {
    while (true) {
        if (L.sp == 0) return false;
        L.cur = stack[--L.sp];
        if (L.cur != PSY_REF_NONE) return true;
        // leaving the instance: back to world space
        Xf ident = xf_identity();
        L.in_inst = 0;
        L.lo = xf_point(L.o, ident);
        L.ldi = recip(xf_vector(L.d, ident));
        L.octant = (uint8_t)ray_code(L.ldi);
        L.safe = (L.ordered && slab_safe(L.lo, L.ldi, L.tmax)) ? 1 : 0;
    }
}

// One while-while iteration: descend to a leaf, process it, pop.  Returns
// 0 = continue, 1 = finished, -1 = stack overflow.
template <int STACK>
DI int lane_step(const GScene &S, const uint8_t *table, Lane &L, uint32_t *stack, TraceCount &tc, bool count) {
    if (L.cur == PSY_REF_NONE) return 1;  // empty scene
    while (!psy_is_leaf(L.cur)) {
        uint32_t code, cnt;
        uint4 ch;
        uint32_t m = S.use_fp16 ? node_hits_h(S, L.cur, L.lo, L.ldi, L.tmax, L.time, L.octant, L.safe, code, cnt, ch)
                                : node_hits(S, L.cur, L.lo, L.ldi, L.tmax, L.time, L.octant, L.safe, code, cnt, ch);
        if (count) tc.nodes++;
        if (m == 0) {
            if (!lane_pop<STACK>(L, stack)) return 1;
            continue;
        }
        uint32_t order = table[48 * L.octant + code];
        uint32_t next = PSY_REF_NONE;
        for (int i = (int)cnt - 1; i >= 0; i--) {
            uint32_t ci = (order >> (i * 2)) & 3u;
            if (m & (1u << ci)) {
                if (next != PSY_REF_NONE) {
                    if (L.sp >= STACK) return -1;
                    stack[L.sp++] = next;
                }
                next = ci == 0 ? ch.x : (ci == 1 ? ch.y : (ci == 2 ? ch.z : ch.w));
            }
        }
        L.cur = next;
    }
    if (!L.in_inst) {
        L.slot = psy_leaf_first(L.cur);
        const GInstance in = S.instances[L.slot];
        if (in.kind == PSY_INST_MESH) {
            const GMesh M = S.meshes[in.obj];
            L.mts = M.ts;
            L.mvb = M.vert_base;
            L.has_xf = in.xc != 0;
            if (L.has_xf) {
                Xf x = lerp_slice_xf(S.xforms + 3 * in.xs, in.xc, L.time);
                L.lo = xf_point(L.o, x);
                L.ldi = recip(xf_vector(L.d, x));
                L.mat = instance_mat(S, in, L.time);
                L.octant = (uint8_t)ray_code(L.ldi);
                L.safe = (L.ordered && slab_safe(L.lo, L.ldi, L.tmax)) ? 1 : 0;
            }
            if (L.sp >= STACK) return -1;
            stack[L.sp++] = PSY_REF_NONE;  // leave-instance marker
            L.in_inst = 1;
            L.cur = M.root;
            return 0;
        } else if (in.kind == PSY_INST_RECT) {
            float t, b0, b1, b2;
            uint32_t which;
            if (rect_hit(S, in, L.o, L.d, L.tmax, L.time, t, b0, b1, b2, which)) {
                if (L.occl) { L.hit.kind = PSY_HIT_OCCLUDE_K; return 1; }
                L.hit.kind = PSY_HIT_LIGHT_K; L.hit.prim = which; L.hit.slot = L.slot;
                L.hit.t = t; L.hit.b0 = b0; L.hit.b1 = b1; L.hit.b2 = b2;
                L.tmax = t;
            }
        } else {
            Xf x = instance_xf_at(S, in, L.time);
            V3 ol = in.xc ? xf_point(L.o, x) : L.lo;
            float t;
            if (sphere_hit(S, in, ol, L.d, L.tmax, L.time, t)) {
                if (L.occl) { L.hit.kind = PSY_HIT_OCCLUDE_K; return 1; }
                L.hit.kind = PSY_HIT_LIGHT_K; L.hit.prim = 0; L.hit.slot = L.slot;
                L.hit.t = t; L.hit.b0 = L.hit.b1 = L.hit.b2 = 0.0f;
                L.tmax = t;
            }
        }
    } else {
        uint32_t first = psy_leaf_first(L.cur), ntri = psy_leaf_count(L.cur);
        for (uint32_t k = 0; k < ntri; k++) {
            uint32_t tri = first + k;
            V3 p0, p1, p2;
            if (L.mts == 1) {
                const float4 *t = S.tris + 3 * (size_t)tri;
                p0 = v3(__ldg(t)); p1 = v3(__ldg(t + 1)); p2 = v3(__ldg(t + 2));
            } else {
                uint4 ix = __ldg(S.tri_idx + tri);
                const float4 *vb = S.verts + L.mvb;
                p0 = lerp_slice_v3(vb + (size_t)ix.x * L.mts, L.mts, L.time);
                p1 = lerp_slice_v3(vb + (size_t)ix.y * L.mts, L.mts, L.time);
                p2 = lerp_slice_v3(vb + (size_t)ix.z * L.mts, L.mts, L.time);
            }
            if (L.has_xf) {
                p0 = xf_point(p0, L.mat);
                p1 = xf_point(p1, L.mat);
                p2 = xf_point(p2, L.mat);
            }
            if (count) tc.tris++;
            float t, b0, b1, b2;
            if (tri_intersect(L.o, L.pre, L.tmax, p0, p1, p2, t, b0, b1, b2)) {
                if (L.occl) { L.hit.kind = PSY_HIT_OCCLUDE_K; return 1; }
                L.hit.kind = PSY_HIT_SURFACE_K; L.hit.prim = tri; L.hit.slot = L.slot;
                L.hit.t = t; L.hit.b0 = b0; L.hit.b1 = b1; L.hit.b2 = b2;
                L.tmax = t;
            }
        }
    }
    return lane_pop<STACK>(L, stack) ? 0 : 1;
}

}  // namespace psyd
