// Warp-packet traversal: the reference's own scheme (BVH4::traverse,
// src/accel/bvh4.rs:101-184, over the tracer's per-octant ray lanes,
// src/tracer.rs:34-85) with a warp as the packet.  The 32 lanes hold 32
// rays; a shared stack per warp holds (node, lane mask, octant) entries.  At
// a node every member lane tests its own ray against the four children, a
// ballot per child gives the lanes that enter it, and the children are
// pushed in the table order of the entry's octant -- so control flow is
// uniform across the warp and each node is loaded once for all lanes.
//
// A ray's sequence of node and leaf tests is the same as in trace_ray: it
// visits exactly the nodes it hits, in the table order of its own octant,
// with its own max_t.  That holds because every entry's lanes share one
// octant: the warp's rays are split into octant groups at the start, and
// again by local octant when they enter an instance.  Hits are therefore
// identical to the one-thread-per-ray kernels.
#pragma once

#include "dev_trace.cuh"

namespace psyd {

struct PacketEntry {
    uint32_t ref;   // node or leaf reference; PSY_REF_NONE = leave the instance
    uint32_t mask;  // lanes whose rays visit it
    uint32_t oct;   // bits 0..2: the lanes' octant (child order); bit 3: inside an instance
};

// All 32 lanes of the warp call this together (`active` false for lanes
// without a ray).  st: the warp's stack, DEPTH entries.  Returns false (on
// every lane) when the stack overflows.
template <int DEPTH, bool COUNT>
DI bool trace_packet(const GScene &S, const uint8_t *table, PacketEntry *st, bool active, V3 o, V3 d, float tmax,
                     float time, bool occl, HitRec &hit, TraceCount *cnt) {
    const uint32_t FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lbit = 1u << lane;
    hit.kind = PSY_HIT_MISS_K;
    hit.prim = 0;
    hit.slot = 0;
    hit.t = 0.0f;
    hit.b0 = hit.b1 = hit.b2 = 0.0f;
    uint32_t live = __ballot_sync(FULL, active);
    if (S.top_root == PSY_REF_NONE || live == 0) return true;
    Xf ident = xf_identity();
    V3 wo = xf_point(o, ident), wdi = recip(xf_vector(d, ident));
    V3 lo = wo, ldi = wdi;
    uint32_t octw = ray_code(wdi);
    bool safew = active && S.ordered_slabs && slab_safe(wo, wdi, tmax);
    bool safe = safew;
    TriPre pre = tri_precompute(d);
    GMesh mesh;
    mesh.ts = 1;
    mesh.vert_base = 0;
    Xf mat = ident;
    bool has_xf = false;
    uint32_t slot = 0;
    int sp = 0;
    // lane 0 writes the entries; __syncwarp before any lane reads them
    auto push = [&](uint32_t ref, uint32_t mask, uint32_t oct) -> bool {
        if (sp >= DEPTH) return false;
        if (lane == 0) {
            st[sp].ref = ref;
            st[sp].mask = mask;
            st[sp].oct = oct;
        }
        sp++;
        return true;
    };
    // one entry per octant group of the warp's rays
    for (uint32_t pending = live; pending;) {
        uint32_t og = __shfl_sync(FULL, octw, __ffs(pending) - 1);
        uint32_t grp = __ballot_sync(FULL, (pending & lbit) != 0 && octw == og);
        if (!push(S.top_root, grp, og)) return false;
        pending &= ~grp;
    }
    while (sp > 0) {
        __syncwarp();
        sp--;
        const uint32_t eref = st[sp].ref, emask = st[sp].mask, eoct = st[sp].oct;
        const bool me = (emask & live & lbit) != 0;
        if (eref == PSY_REF_NONE) {  // leaving an instance: back to world space
            if (emask & lbit) {
                lo = wo;
                ldi = wdi;
                safe = safew;
                has_xf = false;
                mat = ident;
            }
            continue;
        }
        if ((emask & live) == 0) continue;
        if (!psy_is_leaf(eref)) {
            uint32_t code, count;
            uint4 ch;
            uint32_t m = node_hits(S, eref, lo, ldi, tmax, time, eoct & 7u, safe, code, count, ch);
            if (COUNT && me) cnt->nodes++;
            if (!me) m = 0;
            uint32_t c0 = __ballot_sync(FULL, (m & 1u) != 0), c1 = __ballot_sync(FULL, (m & 2u) != 0);
            uint32_t c2 = __ballot_sync(FULL, (m & 4u) != 0), c3 = __ballot_sync(FULL, (m & 8u) != 0);
            uint32_t order = table[48 * (eoct & 7u) + code];
            // reverse table order, so the first child to visit is on top
#pragma unroll
            for (int i = 3; i >= 0; i--) {
                uint32_t ci = (order >> (i * 2)) & 3u;
                uint32_t cm = ci == 0 ? c0 : (ci == 1 ? c1 : (ci == 2 ? c2 : c3));
                if (cm) {
                    uint32_t r = ci == 0 ? ch.x : (ci == 1 ? ch.y : (ci == 2 ? ch.z : ch.w));
                    if (!push(r, cm, eoct)) return false;
                }
            }
            (void)count;
            continue;
        }
        bool done = false;  // an occlusion ray that found a blocker
        if (eoct & 8u) {
            // mesh leaf: up to three triangles
            uint32_t first = psy_leaf_first(eref), ntri = psy_leaf_count(eref);
            for (uint32_t k = 0; k < ntri; k++) {
                if (me && !done) {
                    uint32_t tri = first + k;
                    V3 p0, p1, p2;
                    fetch_tri(S, mesh, tri, time, has_xf, mat, p0, p1, p2);
                    float t, b0, b1, b2;
                    if (COUNT) cnt->tris++;
                    if (tri_intersect(o, pre, tmax, p0, p1, p2, t, b0, b1, b2)) {
                        if (occl) {
                            hit.kind = PSY_HIT_OCCLUDE_K;
                            done = true;
                        } else {
                            hit.kind = PSY_HIT_SURFACE_K; hit.prim = tri; hit.slot = slot;
                            hit.t = t; hit.b0 = b0; hit.b1 = b1; hit.b2 = b2;
                            tmax = t;
                        }
                    }
                }
            }
        } else {
            // world-level leaf: one instance
            uint32_t s = psy_leaf_first(eref);
            GInstance in = S.instances[s];
            if (in.kind == PSY_INST_MESH) {
                GMesh M = S.meshes[in.obj];
                if (me) {
                    mesh = M;
                    slot = s;
                    has_xf = in.xc != 0;
                    if (has_xf) {
                        Xf x = lerp_slice_xf(S.xforms + 3 * in.xs, in.xc, time);
                        lo = xf_point(o, x);
                        ldi = recip(xf_vector(d, x));
                        mat = instance_mat(S, in, time);
                    } else {
                        mat = ident;
                    }
                    safe = S.ordered_slabs && slab_safe(lo, ldi, tmax);
                }
                uint32_t octl = ray_code(ldi);
                uint32_t entered = emask & live;
                if (!push(PSY_REF_NONE, entered, 0u)) return false;
                for (uint32_t pending = entered; pending;) {
                    uint32_t og = __shfl_sync(FULL, octl, __ffs(pending) - 1);
                    uint32_t grp = __ballot_sync(FULL, (pending & lbit) != 0 && octl == og);
                    if (!push(M.root, grp, og | 8u)) return false;
                    pending &= ~grp;
                }
                continue;
            } else if (in.kind == PSY_INST_RECT) {
                if (me) {
                    float t, b0, b1, b2;
                    uint32_t which;
                    if (rect_hit(S, in, o, d, tmax, time, t, b0, b1, b2, which)) {
                        if (occl) {
                            hit.kind = PSY_HIT_OCCLUDE_K;
                            done = true;
                        } else {
                            hit.kind = PSY_HIT_LIGHT_K; hit.prim = which; hit.slot = s;
                            hit.t = t; hit.b0 = b0; hit.b1 = b1; hit.b2 = b2;
                            tmax = t;
                        }
                    }
                }
            } else {
                if (me) {
                    Xf x = instance_xf_at(S, in, time);
                    V3 ol = in.xc ? xf_point(o, x) : wo;
                    float t;
                    if (sphere_hit(S, in, ol, d, tmax, time, t)) {
                        if (occl) {
                            hit.kind = PSY_HIT_OCCLUDE_K;
                            done = true;
                        } else {
                            hit.kind = PSY_HIT_LIGHT_K; hit.prim = 0; hit.slot = s;
                            hit.t = t; hit.b0 = hit.b1 = hit.b2 = 0.0f;
                            tmax = t;
                        }
                    }
                }
            }
        }
        live &= ~__ballot_sync(FULL, done);
    }
    return true;
}

}  // namespace psyd
