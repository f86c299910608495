// Host-side scene build for the GB300 tracing path.
//
// Builds the reference's trees -- the binary SAH BVH of src/accel/bvh_base.rs
// and src/accel/objects_split.rs collapsed into a BVH4 as in
// src/accel/bvh4.rs:186-358, and the 8-ary light tree of
// src/accel/light_tree.rs -- and lays them out flat for the device: one
// 128-byte GNode per BVH4 node, triangles pre-gathered in BVH order.
// Host float arithmetic here must round like the reference's (this file is
// compiled with -ffp-contract=off).
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <functional>
#include <thread>

#include "scene_build.h"

namespace {

// ------------------------------------------------------------------ f32 helpers (SSE semantics)
inline float vmn(float a, float b) { return (a < b) ? a : b; }
inline float vmx(float a, float b) { return (a > b) ? a : b; }

struct BB {
    float mn[3], mx[3];
};
inline BB bb_empty() { return BB{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}}; }
inline BB bb_or(const BB &a, const BB &b) {
    BB o;
    for (int i = 0; i < 3; i++) { o.mn[i] = vmn(a.mn[i], b.mn[i]); o.mx[i] = vmx(a.mx[i], b.mx[i]); }
    return o;
}
inline BB bb_or_pt(const BB &a, const float p[3]) {
    BB o;
    for (int i = 0; i < 3; i++) { o.mn[i] = vmn(a.mn[i], p[i]); o.mx[i] = vmx(a.mx[i], p[i]); }
    return o;
}
inline float bb_area(const BB &b) {
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    return ((dx * dy) + (dy * dz) + (dz * dx)) * 2.0f;
}
inline float bb_diag(const BB &b) {
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    return std::sqrt((dx * dx + dy * dy) + dz * dz);
}
inline BB bb_lerp(const BB &a, const BB &b, float al) {
    BB o;
    float ia = 1.0f - al;
    for (int i = 0; i < 3; i++) { o.mn[i] = (a.mn[i] * ia) + (b.mn[i] * al); o.mx[i] = (a.mx[i] * ia) + (b.mx[i] * al); }
    return o;
}
inline bool lerp_idx(size_t n, float alpha, size_t *i, float *a2) {
    if (n == 1 || alpha == 1.0f) { *i = n - 1; *a2 = 0.0f; return true; }
    float t = alpha * (float)(n - 1);
    *i = (size_t)t;
    *a2 = t - (float)*i;
    return false;
}
inline BB bb_lerp_slice(const BB *s, size_t n, float alpha) {
    size_t i; float a2;
    if (lerp_idx(n, alpha, &i, &a2)) return s[i];
    return bb_lerp(s[i], s[i + 1], a2);
}

// 3x4 affine, same operation order as the device / the reference.
struct M34 {
    float m[12];
};
inline void m_point(const M34 &t, const float p[3], float o[3]) {
    const float *m = t.m;
    o[0] = ((m[0] * p[0] + m[1] * p[1]) + m[2] * p[2]) + m[3];
    o[1] = ((m[4] * p[0] + m[5] * p[1]) + m[6] * p[2]) + m[7];
    o[2] = ((m[8] * p[0] + m[9] * p[1]) + m[10] * p[2]) + m[11];
}
inline void cross3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
inline M34 m_inverse(const M34 &t) {
    const float *m = t.m;
    float c0[3] = {m[0], m[4], m[8]}, c1[3] = {m[1], m[5], m[9]}, c2[3] = {m[2], m[6], m[10]};
    float r0[3], r1[3], r2[3];
    cross3(c1, c2, r0);
    cross3(c2, c0, r1);
    cross3(c0, c1, r2);
    float det = (c2[0] * r2[0] + c2[1] * r2[1]) + c2[2] * r2[2];
    float id = 1.0f / det;
    float inv[9] = {r0[0] * id, r0[1] * id, r0[2] * id, r1[0] * id, r1[1] * id, r1[2] * id, r2[0] * id, r2[1] * id, r2[2] * id};
    M34 o;
    for (int r = 0; r < 3; r++) {
        o.m[r * 4 + 0] = inv[r * 3 + 0];
        o.m[r * 4 + 1] = inv[r * 3 + 1];
        o.m[r * 4 + 2] = inv[r * 3 + 2];
        float tr = (inv[r * 3 + 0] * m[3] + inv[r * 3 + 1] * m[7]) + inv[r * 3 + 2] * m[11];
        o.m[r * 4 + 3] = tr * -1.0f;
    }
    return o;
}
inline M34 m_lerp(const M34 &a, const M34 &b, float al) {
    M34 o;
    float ia = 1.0f - al;
    for (int i = 0; i < 12; i++) o.m[i] = a.m[i] * ia + b.m[i] * al;
    return o;
}
inline M34 m_lerp_slice(const M34 *s, size_t n, float alpha) {
    size_t i; float a2;
    if (lerp_idx(n, alpha, &i, &a2)) return s[i];
    return m_lerp(s[i], s[i + 1], a2);
}
// BBox::transformed (8 corners through the matrix)
inline BB bb_transformed(const BB &b, const M34 &x) {
    BB o = bb_empty();
    for (int c = 0; c < 8; c++) {
        float p[3] = {(c & 4) ? b.mx[0] : b.mn[0], (c & 2) ? b.mx[1] : b.mn[1], (c & 1) ? b.mx[2] : b.mn[2]};
        float q[3];
        m_point(x, p, q);
        for (int i = 0; i < 3; i++) { o.mn[i] = vmn(q[i], o.mn[i]); o.mx[i] = vmx(q[i], o.mx[i]); }
    }
    return o;
}
// transform_bbox_slice_from (src/bbox.rs:153-174)
std::vector<BB> transform_bounds(const std::vector<BB> &in, const M34 *xf, size_t nx) {
    std::vector<BB> out;
    if (nx == 0) return in;
    if (in.size() == nx) {
        for (size_t i = 0; i < nx; i++) out.push_back(bb_transformed(in[i], m_inverse(xf[i])));
    } else if (in.size() > nx) {
        float s = (float)(in.size() - 1);
        for (size_t i = 0; i < in.size(); i++) out.push_back(bb_transformed(in[i], m_inverse(m_lerp_slice(xf, nx, (float)i / s))));
    } else {
        float s = (float)(nx - 1);
        for (size_t i = 0; i < nx; i++) out.push_back(bb_transformed(bb_lerp_slice(in.data(), in.size(), (float)i / s), m_inverse(xf[i])));
    }
    return out;
}
uint64_t hash64(uint64_t n, uint64_t seed) {
    uint64_t h = n;
    const uint64_t k = 32416190071ull * 314604959ull;
    for (int i = 0; i < 4; i++) {
        h *= k;
        h ^= h >> 32;
        h ^= seed;
    }
    return h;
}

// ------------------------------------------------------------------ binary SAH build
// Objects are ids; `bounds(id)` returns their time-sampled boxes.
struct Bounds {
    const BB *p;
    size_t n;
};
using BoundsFn = std::function<Bounds(uint32_t)>;

struct Base {
    struct Node {
        bool leaf;
        uint32_t b0, b1;  // bounds range
        uint32_t c0, c1;  // children
        uint8_t axis;
        uint32_t o0, o1;  // leaf object range
    };
    std::vector<Node> nodes;
    std::vector<BB> bounds;
    const BoundsFn &bf;
    std::vector<BB> midc;  // each object's box at time 0.5 by id (prepare())
    const std::vector<BB> *midc_ref = nullptr;  // a worker's view of its parent build's cache
    bool serial = false;                        // no worker threads
    explicit Base(const BoundsFn &f, bool serial_build = false) : bf(f), serial(serial_build) {}
    // subtrees of at least kParallelMin objects above depth kParallelDepth
    // are built on two threads (up to 2^kParallelDepth at once)
    static constexpr size_t kParallelDepth = 4, kParallelMin = 1u << 15;

    // Appends another build's nodes and bounds (indices shifted); returns
    // the index of its root here.
    uint32_t splice(const Base &o, uint32_t root) {
        uint32_t nb = (uint32_t)nodes.size(), bb = (uint32_t)bounds.size();
        bounds.insert(bounds.end(), o.bounds.begin(), o.bounds.end());
        for (Node n : o.nodes) {
            n.b0 += bb;
            n.b1 += bb;
            if (!n.leaf) {
                n.c0 += nb;
                n.c1 += nb;
            }
            nodes.push_back(n);
        }
        return root + nb;
    }

    // Caches the time-0.5 boxes of objects 0..n-1, which every split of the
    // build evaluates again (the same values: a cache, not a change).
    void prepare(uint32_t n) {
        midc.resize(n);
        for (uint32_t i = 0; i < n; i++) {
            Bounds b = bf(i);
            midc[i] = bb_lerp_slice(b.p, b.n, 0.5f);
        }
    }
    BB mid(uint32_t id) const {
        const std::vector<BB> &c = midc_ref ? *midc_ref : midc;
        if (id < c.size()) return c[id];
        Bounds b = bf(id);
        return bb_lerp_slice(b.p, b.n, 0.5f);
    }

    template <class P>
    static size_t partition(uint32_t *s, size_t len, P pred) {
        size_t a = 0, b = len;
        for (;;) {
            for (;;) {
                if (a == b) return a;
                if (!pred(s[a])) break;
                a++;
            }
            for (;;) {
                b--;
                if (a == b) return a;
                if (pred(s[b])) break;
            }
            std::swap(s[a], s[b]);
            a++;
        }
    }
    void sah(uint32_t *objs, size_t len, size_t *si, uint32_t *axis) const {
        const int NB = 13;
        BB cb = bb_empty();
        std::vector<BB> mids(len);
        for (size_t i = 0; i < len; i++) {
            mids[i] = mid(objs[i]);
            float c[3];
            for (int k = 0; k < 3; k++) c[k] = (mids[i].mn[k] * 0.5f) + (mids[i].mx[k] * 0.5f);  // BBox::center
            cb = bb_or_pt(cb, c);
        }
        float divs[3][NB - 1];
        for (int d = 0; d < 3; d++) {
            float ext = cb.mx[d] - cb.mn[d];
            for (int v = 0; v < NB - 1; v++) divs[d][v] = cb.mn[d] + ext * ((float)(v + 1) / (float)NB);
        }
        // Split v of axis d puts an object left when its centroid c <= divs[d][v]
        // (src/accel/objects_split.rs:166-198).  The divisions do not decrease
        // with v, so an object is left exactly for v >= its bin (the first v
        // with c <= divs[d][v]; NB - 1 when none, NaN included): bin boxes
        // and counts, then prefix / suffix unions give every split's sides.
        // Box union is min / max, exact, so the sides equal the one-object-
        // at-a-time unions (up to the sign of a zero, which no cost
        // comparison sees).
        BB binb[3][NB];
        size_t binc[3][NB] = {};
        for (int d = 0; d < 3; d++)
            for (int k = 0; k < NB; k++) binb[d][k] = bb_empty();
        for (size_t i = 0; i < len; i++) {
            const BB &b = mids[i];
            for (int d = 0; d < 3; d++) {
                float c = (b.mn[d] + b.mx[d]) * 0.5f;
                int k = 0;
                while (k < NB - 1 && !(c <= divs[d][k])) k++;
                binb[d][k] = bb_or(binb[d][k], b);
                binc[d][k]++;
            }
        }
        BB bl[3][NB - 1], br[3][NB - 1];
        size_t cl[3][NB - 1] = {}, cr[3][NB - 1] = {};
        for (int d = 0; d < 3; d++) {
            BB acc = bb_empty();
            size_t cnt = 0;
            for (int v = 0; v < NB - 1; v++) {
                acc = bb_or(acc, binb[d][v]);
                cnt += binc[d][v];
                bl[d][v] = acc;
                cl[d][v] = cnt;
            }
            acc = bb_empty();
            cnt = 0;
            for (int v = NB - 2; v >= 0; v--) {
                acc = bb_or(acc, binb[d][v + 1]);
                cnt += binc[d][v + 1];
                br[d][v] = acc;
                cr[d][v] = cnt;
            }
        }
        int dim = 0;
        float div = 0.0f, best = INFINITY;
        for (int d = 0; d < 3; d++)
            for (int v = 0; v < NB - 1; v++) {
                float lc = bb_area(bl[d][v]) * (float)cl[d][v];
                float rc = bb_area(br[d][v]) * (float)cr[d][v];
                float tot = (lc * bb_diag(bl[d][v])) + (rc * bb_diag(br[d][v]));
                if (tot < best) { dim = d; div = divs[d][v]; best = tot; }
            }
        size_t s = partition(objs, len, [&](uint32_t o) {
            BB b = mid(o);
            return ((b.mn[dim] + b.mx[dim]) * 0.5f) < div;
        });
        if (s < 1) s = 1;
        else if (s >= len) s = len - 1;
        *si = s;
        *axis = (uint32_t)dim;
    }
    void median(uint32_t *objs, size_t len, size_t *si, uint32_t *axis) const {
        BB ub = bb_empty();
        for (size_t i = 0; i < len; i++) ub = bb_or(ub, mid(objs[i]));
        int ax = 0;
        float largest = -INFINITY;
        for (int i = 0; i < 3; i++) {
            float e = ub.mx[i] - ub.mn[i];
            if (e > largest) { largest = e; ax = i; }
        }
        size_t place = len / 2;
        if (place == 0) place = 1;
        auto key = [&](uint32_t o) { BB b = mid(o); return (b.mn[ax] + b.mx[ax]) * 0.5f; };
        size_t left = 0, right = len;
        uint64_t seed = (uint64_t)place;
        for (;;) {
            size_t i = left + (size_t)(hash64((uint64_t)right, seed) % (uint64_t)(right - left));
            std::swap(objs[i], objs[right - 1]);
            float pv = key(objs[right - 1]);
            size_t ii = left + partition(objs + left, right - 1 - left, [&](uint32_t o) { return key(o) < pv; });
            std::swap(objs[ii], objs[right - 1]);
            if (ii == place) break;
            if (ii > place) right = ii;
            else left = ii + 1;
            seed += 1;
        }
        *si = place;
        *axis = (uint32_t)ax;
    }
    void push_reduced(std::vector<BB> &s) {
        BB u = bb_empty();
        for (auto &b : s) u = bb_or(u, b);
        float avg = 0.0f;
        for (auto &b : s) avg = avg + bb_area(b);
        avg = avg / (float)s.size();
        if (bb_area(u) <= (avg * 1.4f)) bounds.push_back(u);
        else bounds.insert(bounds.end(), s.begin(), s.end());
    }
    static void merge(const BB *a, size_t na, const BB *b, size_t nb, std::vector<BB> &out) {
        if (na == 0 || nb == 0) return;
        if (na == nb) {
            for (size_t i = 0; i < na; i++) out.push_back(bb_or(a[i], b[i]));
        } else if (na > nb) {
            float s = (float)(na - 1);
            for (size_t i = 0; i < na; i++) out.push_back(bb_or(a[i], bb_lerp_slice(b, nb, (float)i / s)));
        } else {
            float s = (float)(nb - 1);
            for (size_t i = 0; i < nb; i++) out.push_back(bb_or(bb_lerp_slice(a, na, (float)i / s), b[i]));
        }
    }
    uint32_t build(uint32_t offset, size_t depth, size_t per_leaf, uint32_t *objs, size_t len) {
        uint32_t me = (uint32_t)nodes.size();
        if (len <= per_leaf) {
            size_t ml = 0;
            for (size_t i = 0; i < len; i++) ml = std::max(ml, bf(objs[i]).n);
            std::vector<BB> cache(ml, bb_empty());
            for (size_t i = 0; i < len; i++) {
                Bounds b = bf(objs[i]);
                if (b.n == ml) {
                    for (size_t k = 0; k < ml; k++) cache[k] = bb_or(cache[k], b.p[k]);
                } else {
                    float s = (float)(ml - 1);
                    for (size_t k = 0; k < ml; k++) cache[k] = bb_or(cache[k], bb_lerp_slice(b.p, b.n, (float)k / s));
                }
            }
            uint32_t b0 = (uint32_t)bounds.size();
            push_reduced(cache);
            Node n{};
            n.leaf = true; n.b0 = b0; n.b1 = (uint32_t)bounds.size(); n.o0 = offset; n.o1 = offset + (uint32_t)len;
            nodes.push_back(n);
            return me;
        }
        nodes.push_back(Node{});
        size_t si;
        uint32_t axis;
        uint64_t lg = 63 - (uint64_t)__builtin_clzll((unsigned long long)len);
        if (lg < (42 - depth)) sah(objs, len, &si, &axis);
        else median(objs, len, &si, &axis);
        uint32_t c0, c1;
        if (!serial && depth < kParallelDepth && len - si >= kParallelMin && si >= kParallelMin) {
            // the right subtree on a worker thread, into its own node and
            // bounds arrays (the two sides touch disjoint object ranges),
            // spliced in afterwards: the tree is the same, only its storage
            // order differs, and the BVH4 collapse follows the child indices
            Base right(bf);
            right.midc_ref = midc_ref ? midc_ref : &midc;
            uint32_t rroot = 0;
            std::exception_ptr failure;
            std::thread th;
            bool threaded = false;
            try {
                th = std::thread([&] {
                    try {
                        rroot = right.build(offset + (uint32_t)si, depth + 1, per_leaf, objs + si, len - si);
                    } catch (...) {
                        failure = std::current_exception();
                    }
                });
                threaded = true;
            } catch (...) {  // no thread to be had: build both sides here
            }
            if (threaded) {
                try {
                    c0 = build(offset, depth + 1, per_leaf, objs, si);
                } catch (...) {
                    th.join();
                    throw;
                }
                th.join();
                if (failure) std::rethrow_exception(failure);
                c1 = splice(right, rroot);
            } else {
                c0 = build(offset, depth + 1, per_leaf, objs, si);
                c1 = build(offset + (uint32_t)si, depth + 1, per_leaf, objs + si, len - si);
            }
        } else {
            c0 = build(offset, depth + 1, per_leaf, objs, si);
            c1 = build(offset + (uint32_t)si, depth + 1, per_leaf, objs + si, len - si);
        }
        std::vector<BB> merged;
        merge(&bounds[nodes[c0].b0], nodes[c0].b1 - nodes[c0].b0, &bounds[nodes[c1].b0], nodes[c1].b1 - nodes[c1].b0, merged);
        uint32_t b0 = (uint32_t)bounds.size();
        push_reduced(merged);
        Node &n = nodes[me];
        n.leaf = false; n.b0 = b0; n.b1 = (uint32_t)bounds.size(); n.c0 = c0; n.c1 = c1; n.axis = (uint8_t)axis;
        return me;
    }
};

// ------------------------------------------------------------------ BVH4 collapse
struct Collapser {
    const Base &base;
    HostScene &hs;
    std::function<uint32_t(uint32_t, uint32_t)> leaf_ref;  // (o0, count) -> child ref
    uint32_t node_count = 0;

    // returns the child reference of base node bn; `maxpush` = worst-case
    // stack entries pushed below it.
    uint32_t emit(uint32_t bn, uint32_t *maxpush) {
        const Base::Node &n = base.nodes[bn];
        node_count++;
        if (n.leaf) {
            *maxpush = 0;
            return leaf_ref(n.o0, n.o1 - n.o0);
        }
        const Base::Node &l = base.nodes[n.c0], &r = base.nodes[n.c1];
        uint32_t ch[4] = {0, 0, 0, 0};
        uint32_t cc;
        uint32_t code;
        if (!l.leaf && !r.leaf) {
            cc = 4; ch[0] = l.c0; ch[1] = l.c1; ch[2] = r.c0; ch[3] = r.c1;
            code = n.axis + l.axis * 3 + r.axis * 9;
        } else if (!l.leaf) {
            cc = 3; ch[0] = l.c0; ch[1] = l.c1; ch[2] = n.c1;
            code = n.axis + l.axis * 3 + 27;
        } else if (!r.leaf) {
            cc = 3; ch[0] = n.c0; ch[1] = r.c0; ch[2] = r.c1;
            code = n.axis + r.axis * 3 + 36;
        } else {
            cc = 2; ch[0] = n.c0; ch[1] = n.c1;
            code = n.axis + 45;
        }
        uint32_t me = (uint32_t)hs.nodes.size();
        hs.nodes.push_back(GNode{});
        size_t blen = 0;
        for (uint32_t i = 0; i < cc; i++) blen = std::max(blen, (size_t)(base.nodes[ch[i]].b1 - base.nodes[ch[i]].b0));
        size_t keys = blen < 2 ? 1 : blen;
        uint32_t ext = (uint32_t)hs.bounds_ext.size();
        for (size_t k = 0; k < keys; k++) {
            BB b[4];
            for (int i = 0; i < 4; i++) {
                if ((uint32_t)i >= cc) { b[i] = bb_empty(); continue; }
                const Base::Node &c = base.nodes[ch[i]];
                if (blen < 2) b[i] = base.bounds[c.b0];
                else b[i] = bb_lerp_slice(&base.bounds[c.b0], c.b1 - c.b0, (float)k / (float)(blen - 1));
            }
            GBounds4 g;
            g.xlo = make_float4(b[0].mn[0], b[1].mn[0], b[2].mn[0], b[3].mn[0]);
            g.xhi = make_float4(b[0].mx[0], b[1].mx[0], b[2].mx[0], b[3].mx[0]);
            g.ylo = make_float4(b[0].mn[1], b[1].mn[1], b[2].mn[1], b[3].mn[1]);
            g.yhi = make_float4(b[0].mx[1], b[1].mx[1], b[2].mx[1], b[3].mx[1]);
            g.zlo = make_float4(b[0].mn[2], b[1].mn[2], b[2].mn[2], b[3].mn[2]);
            g.zhi = make_float4(b[0].mx[2], b[1].mx[2], b[2].mx[2], b[3].mx[2]);
            if (k == 0) {
                GNode &gn = hs.nodes[me];
                gn.xlo = g.xlo; gn.xhi = g.xhi; gn.ylo = g.ylo; gn.yhi = g.yhi; gn.zlo = g.zlo; gn.zhi = g.zhi;
            } else {
                hs.bounds_ext.push_back(g);
            }
        }
        uint32_t refs[4] = {0, 0, 0, 0};
        uint32_t mp = 0;
        for (uint32_t i = 0; i < cc; i++) {
            uint32_t sub;
            refs[i] = emit(ch[i], &sub);
            mp = std::max(mp, sub);
        }
        *maxpush = mp + (cc - 1);
        GNode &gn = hs.nodes[me];
        gn.child = make_uint4(refs[0], refs[1], refs[2], refs[3]);
        gn.meta = make_uint4(keys > 1 ? ext : 0u, (uint32_t)keys, code | (cc << 8), 0u);
        return me;
    }
};

// ------------------------------------------------------------------ colour
float color_energy(const PsyColor &c) {
    if (c.kind == PSY_COLOR_XYZ) return c.v[1];
    if (c.kind == PSY_COLOR_BLACKBODY) {
        float t2 = c.v[0] * c.v[0];
        return t2 * t2 * c.v[1];
    }
    return c.v[1];
}
GColor to_gcolor(const PsyColor &c) { return GColor{c.kind, c.v[0], c.v[1], c.v[2]}; }

static void rgb_to_xyz_matrix_f64(double rx, double ry, double gx, double gy, double bx, double by, double wx,
                                  double wy, double m[9]) {
    double Y = 1.0;
    double X = wx * Y / wy;
    double Z = (1.0 - wx - wy) * Y / wy;
    double d = rx * (by - gy) + bx * (gy - ry) + gx * (ry - by);
    double sr = (X * (by - gy) - gx * (Y * (by - 1.0) + by * (X + Z)) + bx * (Y * (gy - 1.0) + gy * (X + Z))) / d;
    double sg = (X * (ry - by) + rx * (Y * (by - 1.0) + by * (X + Z)) - bx * (Y * (ry - 1.0) + ry * (X + Z))) / d;
    double sb = (X * (gy - ry) - rx * (Y * (gy - 1.0) + gy * (X + Z)) + gx * (Y * (ry - 1.0) + ry * (X + Z))) / d;
    double v[9] = {sr * rx, sg * gx, sb * bx, sr * ry, sg * gy, sb * by, sr * (1.0 - rx - ry), sg * (1.0 - gx - gy), sb * (1.0 - bx - by)};
    for (int i = 0; i < 9; i++) m[i] = v[i];
}
// The generated Rust source prints each coefficient with 10 decimals; the
// f32 constant is that decimal number.
static void round_10(const double m[9], float out[9]) {
    for (int i = 0; i < 9; i++) {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.10f", m[i]);
        out[i] = std::strtof(buf, nullptr);
    }
}
void rgb_to_xyz_matrix(double rx, double ry, double gx, double gy, double bx, double by, double wx, double wy, float out[9]) {
    double m[9];
    rgb_to_xyz_matrix_f64(rx, ry, gx, gy, bx, by, wx, wy, m);
    round_10(m, out);
}


float4 f4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
void push_xf(std::vector<float4> &v, const M34 &m) {
    v.push_back(f4(m.m[0], m.m[1], m.m[2], m.m[3]));
    v.push_back(f4(m.m[4], m.m[5], m.m[6], m.m[7]));
    v.push_back(f4(m.m[8], m.m[9], m.m[10], m.m[11]));
}

float f16_value(uint16_t h) { return __half2float(__ushort_as_half(h)); }

// Adjacent f16 values toward +inf / -inf (finite patterns; both zeros step
// to the smallest value on the side of the step).
uint16_t f16_step_up(uint16_t h) {
    if (h == 0x8000u || h == 0x0000u) return 0x0001u;
    return (h & 0x8000u) ? (uint16_t)(h - 1) : (uint16_t)(h + 1);
}
uint16_t f16_step_down(uint16_t h) {
    if (h == 0x0000u || h == 0x8000u) return 0x8001u;
    return (h & 0x8000u) ? (uint16_t)(h + 1) : (uint16_t)(h - 1);
}

// f16 offsets of the FP16 node copy.  The device decodes a bound as the f32
// sum anchor + offset, rounded to nearest (one instruction, PTX
// add.rn.f32.f16), so the offset is chosen for that sum to lie on the outer
// side of the f32 bound itself: fl32(a + h) <= target for a lower bound
// (dir < 0), >= target for an upper one (dir > 0).  The decoded box then
// contains the f32 box and, the slab arithmetic being monotone, every child
// the f32 test hits is hit.  Start from the f16 nearest to the exact
// difference and step outward one f16 ulp at a time until the f32 sum --
// the device's own arithmetic -- is outside.  False when the difference is
// past the f16 range (the node keeps its f32 bounds).
bool f16_offset(float a, float target, int dir, uint16_t &out) {
    double d = (double)target - (double)a;
    if (!std::isfinite(d) || std::fabs(d) > 65000.0) return false;
    uint16_t h = __half_as_ushort(__float2half_rn((float)d));
    for (int k = 0; k < 64; k++) {
        float v = a + f16_value(h);
        if (dir < 0 ? (v <= target) : (v >= target)) {
            out = h;
            return true;
        }
        h = dir < 0 ? f16_step_down(h) : f16_step_up(h);
        if ((h & 0x7C00u) == 0x7C00u) return false;  // stepped past the largest finite f16
    }
    return false;
}

}  // namespace

// xyz_to_rec709_e: the inverse of the equal-energy rec709 matrix by
// Gauss-Jordan elimination with partial pivoting in f64 (the color crate's
// build script, sub_crates/color/build.rs:162-188, 246-323), then printed
// with 10 decimals.
void xyz_to_rec709_e_matrix(float out[9]) {
    double e[9];
    rgb_to_xyz_matrix_f64(0.640, 0.330, 0.300, 0.600, 0.150, 0.060, 1.0 / 3.0, 1.0 / 3.0, e);
    double t[3][3], s[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) t[i][j] = e[i * 3 + j];
    for (int i = 0; i < 2; i++) {
        int pivot = i;
        double psize = t[i][i] < 0.0 ? -t[i][i] : t[i][i];
        for (int j = i + 1; j < 3; j++) {
            double tmp = t[j][i] < 0.0 ? -t[j][i] : t[j][i];
            if (tmp > psize) { pivot = j; psize = tmp; }
        }
        if (pivot != i)
            for (int j = 0; j < 3; j++) { std::swap(t[i][j], t[pivot][j]); std::swap(s[i][j], s[pivot][j]); }
        for (int j = i + 1; j < 3; j++) {
            double f = t[j][i] / t[i][i];
            for (int k = 0; k < 3; k++) { t[j][k] -= f * t[i][k]; s[j][k] -= f * s[i][k]; }
        }
    }
    for (int i = 2; i >= 0; i--) {
        double f = t[i][i];
        for (int j = 0; j < 3; j++) { t[i][j] /= f; s[i][j] /= f; }
        for (int j = 0; j < i; j++) {
            double g = t[j][i];
            for (int k = 0; k < 3; k++) { t[j][k] -= g * t[i][k]; s[j][k] -= g * s[i][k]; }
        }
    }
    double inv[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) inv[i * 3 + j] = s[i][j];
    round_10(inv, out);
}

void unassigned_magenta_xyz(float out[3]) {
    float m[9];
    rgb_to_xyz_matrix(0.640, 0.330, 0.300, 0.600, 0.150, 0.060, 0.3127, 0.3290, m);
    float rgb[3] = {1.0f, 0.0f, 1.0f};
    for (int r = 0; r < 3; r++) out[r] = ((rgb[0] * m[r * 3]) + (rgb[1] * m[r * 3 + 1])) + (rgb[2] * m[r * 3 + 2]);
}

// Worst-case traversal stack entries pushed below a GPU-built node (the
// host collapse returns the same figure for its own trees).
static uint32_t node_maxpush(const std::vector<GNode> &nodes, uint32_t base, uint32_t ref) {
    if (psy_is_leaf(ref)) return 0;
    const GNode &n = nodes[ref - base];
    uint32_t cc = n.meta.z >> 8, mp = 0;
    const uint32_t ch[4] = {n.child.x, n.child.y, n.child.z, n.child.w};
    for (uint32_t i = 0; i < cc; i++) mp = std::max(mp, node_maxpush(nodes, base, ch[i]));
    return mp + (cc - 1);
}

int build_host_scene(const PsySceneDesc *d, const PsySceneOptions *opts, HostScene &hs, std::string &err,
                     const GpuMeshBuild *gpu_build, bool serial) {
    if (!d) { err = "null scene description"; return PSY_E_INVALID; }
    if (d->num_objects && !d->objects) { err = "objects pointer is null"; return PSY_E_INVALID; }
    if (d->num_instances && !d->instances) { err = "instances pointer is null"; return PSY_E_INVALID; }
    if (d->num_shaders && !d->shaders) { err = "shaders pointer is null"; return PSY_E_INVALID; }
    if (d->num_xforms && !d->xforms) { err = "xforms pointer is null"; return PSY_E_INVALID; }
    if (d->camera.num_transforms == 0 || !d->camera.transforms || d->camera.num_fovs == 0 || !d->camera.fovs) {
        err = "camera needs at least one transform and one fov";
        return PSY_E_INVALID;
    }
    if (d->width == 0 || d->height == 0 || d->width > 65536 || d->height > 65536) {
        err = "resolution must be within 1..65536";
        return PSY_E_INVALID;
    }
    hs.width = d->width; hs.height = d->height; hs.spp = d->spp; hs.seed = d->seed; hs.max_bounces = d->max_bounces;
    hs.background = to_gcolor(d->background);
    bool fp16 = opts && opts->bounds_precision == PSY_BOUNDS_FP16;
    // shaders
    for (uint32_t i = 0; i < d->num_shaders; i++) {
        const PsyShaderDesc &s = d->shaders[i];
        if (s.kind > PSY_SHADER_GGX) { err = "unknown shader kind"; return PSY_E_INVALID; }
        GShader g{};
        g.kind = s.kind;
        g.roughness = s.roughness;
        g.fresnel = s.fresnel;
        g.color = to_gcolor(s.color);
        hs.shaders.push_back(g);
    }
    // objects
    struct ObjInfo {
        uint32_t kind, index;
        std::vector<BB> bounds;  // object-space bounds keys
        float energy;
    };
    std::vector<ObjInfo> objs(d->num_objects);
    hs.object_to_mesh.assign(d->num_objects, -1);
    uint32_t max_mesh_push = 0;
    for (uint32_t oi = 0; oi < d->num_objects; oi++) {
        const PsyObjectDesc &od = d->objects[oi];
        ObjInfo &info = objs[oi];
        info.kind = od.kind;
        if (od.time_samples == 0) { err = "object with zero time samples"; return PSY_E_INVALID; }
        if (od.kind == PSY_OBJ_MESH) {
            if (od.num_tris == 0 || od.num_verts == 0 || !od.verts || !od.indices) { err = "empty or null mesh"; return PSY_E_INVALID; }
            uint32_t nv = od.num_verts, nt = od.num_tris, ts = od.time_samples;
            for (size_t k = 0; k < (size_t)nt * 3; k++)
                if (od.indices[k] >= nv) { err = "triangle index out of range"; return PSY_E_INVALID; }
            if ((uint64_t)hs.tri_idx.size() + nt >= (1ull << 29)) { err = "too many triangles"; return PSY_E_UNSUPPORTED; }
            GMesh gm{};
            gm.tri_base = (uint32_t)hs.tri_idx.size();
            gm.ntris = nt;
            gm.ts = ts;
            gm.vert_base = (uint32_t)hs.verts.size();
            gm.has_normals = od.normals ? 1u : 0u;
            gm.normal_base = gm.vert_base;
            for (uint32_t v = 0; v < nv; v++)
                for (uint32_t k = 0; k < ts; k++) {
                    const float *p = od.verts + ((size_t)k * nv + v) * 3;
                    hs.verts.push_back(f4(p[0], p[1], p[2], 0.0f));
                    if (od.normals) {
                        const float *n = od.normals + ((size_t)k * nv + v) * 3;
                        hs.normals.push_back(f4(n[0], n[1], n[2], 0.0f));
                    } else {
                        hs.normals.push_back(f4(0.0f, 0.0f, 0.0f, 0.0f));
                    }
                }
            // per-triangle bounds keys, from the vertices as given
            std::vector<BB> tb((size_t)nt * ts);
            for (uint32_t t = 0; t < nt; t++) {
                const uint32_t *ix = od.indices + (size_t)t * 3;
                for (uint32_t k = 0; k < ts; k++) {
                    const float *a = od.verts + ((size_t)k * nv + ix[0]) * 3;
                    const float *b = od.verts + ((size_t)k * nv + ix[1]) * 3;
                    const float *c = od.verts + ((size_t)k * nv + ix[2]) * 3;
                    BB bb;
                    for (int q = 0; q < 3; q++) {
                        bb.mn[q] = vmn(a[q], vmn(b[q], c[q]));
                        bb.mx[q] = vmx(a[q], vmx(b[q], c[q]));
                    }
                    tb[(size_t)t * ts + k] = bb;
                }
            }
            std::vector<uint32_t> order(nt);
            for (uint32_t t = 0; t < nt; t++) order[t] = t;
            bool on_gpu = opts && opts->bvh_build == PSY_BVH_GPU && ts == 1;
            LbvhOutput lb;
            BoundsFn bf = [&](uint32_t t) { return Bounds{&tb[(size_t)t * ts], (size_t)ts}; };
            Base base(bf, serial);
            if (!on_gpu) base.prepare(nt);
            if (on_gpu) {
                if (!gpu_build) { err = "GPU BVH build needs a CUDA device"; return PSY_E_UNSUPPORTED; }
                LbvhInput li{od.verts, nv, od.indices, nt, (uint32_t)hs.nodes.size(), (uint32_t)hs.tri_idx.size()};
                int rc = (*gpu_build)(li, lb, err);
                if (rc != PSY_OK) return rc;
                order = lb.order;
            } else {
                base.build(0, 0, 3, order.data(), nt);
            }
            // triangles in BVH order: (v0, v2, v1, original) as the reference's index tuples
            for (uint32_t i = 0; i < nt; i++) {
                uint32_t t = order[i];
                const uint32_t *ix = od.indices + (size_t)t * 3;
                hs.tri_idx.push_back(make_uint4(ix[0], ix[2], ix[1], t));
                if (ts == 1) {
                    const float *a = od.verts + (size_t)ix[0] * 3, *b = od.verts + (size_t)ix[2] * 3, *c = od.verts + (size_t)ix[1] * 3;
                    float tag;
                    std::memcpy(&tag, &t, 4);
                    hs.tris.push_back(f4(a[0], a[1], a[2], tag));
                    hs.tris.push_back(f4(b[0], b[1], b[2], 0.0f));
                    hs.tris.push_back(f4(c[0], c[1], c[2], 0.0f));
                } else {
                    hs.tris.push_back(f4(0, 0, 0, 0));
                    hs.tris.push_back(f4(0, 0, 0, 0));
                    hs.tris.push_back(f4(0, 0, 0, 0));
                }
            }
            uint32_t tri_base = gm.tri_base;
            uint32_t mp, node_count;
            if (on_gpu) {
                uint32_t node_base = (uint32_t)hs.nodes.size();
                hs.nodes.insert(hs.nodes.end(), lb.nodes.begin(), lb.nodes.end());
                gm.root = lb.root;
                mp = node_maxpush(hs.nodes, 0, lb.root);
                node_count = lb.node_count;
                // object bounds: the union of the triangle bounds
                BB u = bb_empty();
                for (uint32_t t = 0; t < nt; t++) u = bb_or(u, tb[t]);
                info.bounds.assign(1, u);
                (void)node_base;
            } else {
                Collapser col{base, hs, [tri_base](uint32_t o0, uint32_t cnt) { return psy_make_leaf(tri_base + o0, cnt); }};
                gm.root = col.emit(0, &mp);
                node_count = col.node_count;
                const Base::Node &root = base.nodes[0];
                info.bounds.assign(base.bounds.begin() + root.b0, base.bounds.begin() + root.b1);
            }
            max_mesh_push = std::max(max_mesh_push, mp);
            info.index = (uint32_t)hs.meshes.size();
            hs.object_to_mesh[oi] = (int32_t)hs.meshes.size();
            hs.meshes.push_back(gm);
            hs.mesh_tri_order.push_back(order);
            hs.mesh_node_count.push_back(node_count);
        } else if (od.kind == PSY_OBJ_RECT_LIGHT || od.kind == PSY_OBJ_SPHERE_LIGHT) {
            if (!od.dims || !od.colors) { err = "light without dims or colors"; return PSY_E_INVALID; }
            GLight L{};
            L.key_base = (uint32_t)hs.light_dims.size();
            L.nkeys = od.time_samples;
            float e = 0.0f;
            for (uint32_t k = 0; k < od.time_samples; k++) {
                if (od.kind == PSY_OBJ_RECT_LIGHT) {
                    float w = od.dims[k * 2], h = od.dims[k * 2 + 1];
                    hs.light_dims.push_back(make_float2(w, h));
                    info.bounds.push_back(BB{{w * -0.5f, h * -0.5f, 0.0f}, {w * 0.5f, h * 0.5f, 0.0f}});
                } else {
                    float r = od.dims[k];
                    hs.light_dims.push_back(make_float2(r, 0.0f));
                    info.bounds.push_back(BB{{-r, -r, -r}, {r, r, r}});
                }
                hs.light_colors.push_back(to_gcolor(od.colors[k]));
                e = e + color_energy(od.colors[k]);
            }
            L.energy = e / (float)od.time_samples;
            info.energy = L.energy;
            info.index = (uint32_t)hs.lights.size();
            hs.lights.push_back(L);
        } else {
            err = "unknown object kind";
            return PSY_E_INVALID;
        }
    }
    // instances: bounds, instance BVH (one instance per leaf)
    uint32_t ni = d->num_instances;
    std::vector<M34> xforms(d->num_xforms);
    for (uint32_t i = 0; i < d->num_xforms; i++) std::memcpy(xforms[i].m, d->xforms[i].m, 48);
    std::vector<std::vector<BB>> ibounds(ni);
    for (uint32_t i = 0; i < ni; i++) {
        const PsyInstanceDesc &in = d->instances[i];
        if (in.object >= d->num_objects) { err = "instance object out of range"; return PSY_E_INVALID; }
        if (in.shader >= (int32_t)d->num_shaders) { err = "instance shader out of range"; return PSY_E_INVALID; }
        if ((uint64_t)in.xform_start + in.xform_count > d->num_xforms) { err = "instance transforms out of range"; return PSY_E_INVALID; }
        ibounds[i] = transform_bounds(objs[in.object].bounds, in.xform_count ? &xforms[in.xform_start] : nullptr, in.xform_count);
    }
    for (auto &x : xforms) push_xf(hs.xforms, x);
    {
        BB u = bb_empty();
        for (auto &v : ibounds)
            for (auto &b : v) u = bb_or(u, b);
        for (int a = 0; a < 3; a++) {
            hs.scene_min[a] = std::isfinite(u.mn[a]) ? u.mn[a] : 0.0f;
            hs.scene_max[a] = std::isfinite(u.mx[a]) ? u.mx[a] : 0.0f;
        }
    }
    std::vector<uint32_t> iorder(ni);
    for (uint32_t i = 0; i < ni; i++) iorder[i] = i;
    uint32_t top_push = 0;
    if (ni > 0) {
        BoundsFn bf = [&](uint32_t i) { return Bounds{ibounds[i].data(), ibounds[i].size()}; };
        Base base(bf, serial);
        base.prepare(ni);
        base.build(0, 0, 1, iorder.data(), ni);
        Collapser col{base, hs, [](uint32_t o0, uint32_t) { return psy_make_leaf(o0, 1); }};
        hs.top_root = col.emit(0, &top_push);
    }
    for (uint32_t s = 0; s < ni; s++) {
        const PsyInstanceDesc &in = d->instances[iorder[s]];
        GInstance g{};
        uint32_t k = d->objects[in.object].kind;
        g.kind = k == PSY_OBJ_MESH ? PSY_INST_MESH : (k == PSY_OBJ_RECT_LIGHT ? PSY_INST_RECT : PSY_INST_SPHERE);
        g.obj = objs[in.object].index;
        g.shader = in.shader;
        g.id = iorder[s];
        g.xs = in.xform_start;
        g.xc = in.xform_count;
        g.xinv = 0;
        if (in.xform_count == 1) {
            g.xinv = (uint32_t)(hs.xforms_inv.size() / 3);
            push_xf(hs.xforms_inv, m_inverse(xforms[in.xform_start]));
        }
        hs.instances.push_back(g);
    }
    if (hs.xforms.empty()) push_xf(hs.xforms, M34{{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}});
    if (hs.xforms_inv.empty()) push_xf(hs.xforms_inv, M34{{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}});
    hs.max_stack = top_push + 1 + max_mesh_push;
    // light tree over light instances, in instance-BVH order
    std::vector<uint32_t> lights;  // slots
    for (uint32_t s = 0; s < ni; s++)
        if (hs.instances[s].kind != PSY_INST_MESH) lights.push_back(s);
    if (!lights.empty()) {
        struct LTN {
            bool leaf;
            uint32_t b0, b1;
            float energy;
            uint32_t child;  // leaf: light slot offset; inner: second child
        };
        std::vector<LTN> nodes;
        std::vector<BB> lb;
        std::vector<uint32_t> lord(lights.size());
        for (size_t i = 0; i < lights.size(); i++) lord[i] = (uint32_t)i;
        auto lbounds = [&](uint32_t li) -> const std::vector<BB> & { return ibounds[hs.instances[lights[li]].id]; };
        BoundsFn bf = [&](uint32_t li) { const auto &b = lbounds(li); return Bounds{b.data(), b.size()}; };
        Base splitter(bf, serial);
        splitter.prepare((uint32_t)lights.size());
        std::function<uint32_t(uint32_t, uint32_t *, size_t)> rb = [&](uint32_t off, uint32_t *o, size_t len) -> uint32_t {
            uint32_t me = (uint32_t)nodes.size();
            if (len == 1) {
                uint32_t b0 = (uint32_t)lb.size();
                const auto &b = lbounds(o[0]);
                lb.insert(lb.end(), b.begin(), b.end());
                const GInstance &gi = hs.instances[lights[o[0]]];
                nodes.push_back(LTN{true, b0, (uint32_t)lb.size(), hs.lights[gi.obj].energy, off});
                return me;
            }
            nodes.push_back(LTN{false, 0, 0, 0.0f, 0});
            size_t si;
            uint32_t ax;
            splitter.sah(o, len, &si, &ax);
            rb(off, o, si);
            uint32_t c2 = rb(off + (uint32_t)si, o + si, len - si);
            std::vector<BB> merged;
            Base::merge(&lb[nodes[me + 1].b0], nodes[me + 1].b1 - nodes[me + 1].b0, &lb[nodes[c2].b0], nodes[c2].b1 - nodes[c2].b0, merged);
            uint32_t b0 = (uint32_t)lb.size();
            lb.insert(lb.end(), merged.begin(), merged.end());
            float e = nodes[me + 1].energy + nodes[c2].energy;
            nodes[me] = LTN{false, b0, (uint32_t)lb.size(), e, c2};
            return me;
        };
        rb(0, lord.data(), lord.size());
        for (size_t i = 0; i < lord.size(); i++) hs.light_instances.push_back(hs.instances[lights[lord[i]]]);
        // collapse to arity 8 (ARITY_LOG2 = 3)
        std::function<uint32_t(uint32_t, uint32_t)> ccount = [&](uint32_t lc, uint32_t ni2) -> uint32_t {
            if (lc > 0) {
                if (nodes[ni2].leaf) return 1;
                return ccount(lc - 1, ni2 + 1) + ccount(lc - 1, nodes[ni2].child);
            }
            return 1;
        };
        std::function<void(uint32_t, uint32_t, uint32_t, uint32_t *, uint32_t *)> nth =
            [&](uint32_t lc, uint32_t ni2, uint32_t n, uint32_t *idx, uint32_t *rem) {
                if (lc > 0 && !nodes[ni2].leaf) {
                    uint32_t i, r;
                    nth(lc - 1, ni2 + 1, n, &i, &r);
                    if (r == 0) { *idx = i; *rem = 0; return; }
                    nth(lc - 1, nodes[ni2].child, r - 1, idx, rem);
                    return;
                }
                *idx = ni2; *rem = n;
            };
        std::function<void(uint32_t, uint32_t)> emit = [&](uint32_t bn, uint32_t slot) {
            const LTN &n = nodes[bn];
            GLightTreeNode g{};
            g.bounds_base = (uint32_t)(hs.lt_bounds.size() / 2);
            g.nbounds = n.b1 - n.b0;
            for (uint32_t k = n.b0; k < n.b1; k++) {
                hs.lt_bounds.push_back(f4(lb[k].mn[0], lb[k].mn[1], lb[k].mn[2], 0.0f));
                hs.lt_bounds.push_back(f4(lb[k].mx[0], lb[k].mx[1], lb[k].mx[2], 0.0f));
            }
            g.energy = n.energy;
            if (n.leaf) {
                g.leaf = 1;
                g.index = n.child;
                g.nchild = 0;
                hs.lt_nodes[slot] = g;
                return;
            }
            uint32_t cc = ccount(3, bn);
            uint32_t c0 = (uint32_t)hs.lt_nodes.size();
            hs.lt_nodes.resize(c0 + cc);
            g.leaf = 0;
            g.index = c0;
            g.nchild = cc;
            hs.lt_nodes[slot] = g;
            for (uint32_t i = 0; i < cc; i++) {
                uint32_t idx, rem;
                nth(3, bn, i, &idx, &rem);
                emit(idx, c0 + i);
            }
        };
        hs.lt_nodes.resize(1);
        emit(0, 0);
        hs.lt_empty = false;
        hs.lt_root_energy = hs.lt_nodes[0].energy;
    }
    if (hs.lt_nodes.empty()) hs.lt_nodes.push_back(GLightTreeNode{});
    if (hs.lt_bounds.empty()) { hs.lt_bounds.push_back(f4(0, 0, 0, 0)); hs.lt_bounds.push_back(f4(0, 0, 0, 0)); }
    if (hs.light_instances.empty()) hs.light_instances.push_back(GInstance{});
    // camera (Camera::new, src/camera.rs:22-72)
    const PsyCameraDesc &c = d->camera;
    for (uint32_t i = 0; i < c.num_transforms; i++) {
        M34 m;
        std::memcpy(m.m, c.transforms[i].m, 48);
        push_xf(hs.cam_xf, m);
    }
    for (uint32_t i = 0; i < c.num_fovs; i++) {
        float n = c.fovs[i];
        hs.cam_tfov.push_back(std::sin(n / 2.0f) / std::cos(n / 2.0f));
    }
    std::vector<float> ap(c.aperture_radii, c.aperture_radii + (c.aperture_radii ? c.num_aperture_radii : 0));
    std::vector<float> fd(c.focus_distances, c.focus_distances + (c.focus_distances ? c.num_focus_distances : 0));
    if (ap.empty() || fd.empty()) { ap = {0.0f}; fd = {1.0f}; }
    for (float f : fd)
        if (f == 0.0f) { ap = {0.0f}; fd = {1.0f}; break; }
    hs.cam_ap = ap;
    hs.cam_fd = fd;
    // distant lights
    float total = 0.0f;
    for (uint32_t i = 0; i < d->num_distant_lights; i++) {
        const PsyDistantLightDesc &dl = d->distant_lights[i];
        if (dl.num_keys == 0 || !dl.radii || !dl.directions || !dl.colors) { err = "distant light without keys"; return PSY_E_INVALID; }
        GDistant g{};
        g.key_base = (uint32_t)hs.distant_radii.size();
        g.nkeys = dl.num_keys;
        float e = 0.0f;
        for (uint32_t k = 0; k < dl.num_keys; k++) {
            hs.distant_radii.push_back(dl.radii[k]);
            hs.distant_dirs.push_back(f4(dl.directions[k * 3], dl.directions[k * 3 + 1], dl.directions[k * 3 + 2], 0.0f));
            hs.distant_colors.push_back(to_gcolor(dl.colors[k]));
            e = e + color_energy(dl.colors[k]);
        }
        g.energy = e / (float)dl.num_keys;
        total = total + g.energy;
        if (dl.num_keys == 1) {
            // DistantDiskLight::sample_from_point constants (src/light/distant_disk_light.rs:67-83)
            double radius = (double)dl.radii[0];
            double ctm = std::cos(radius);
            g.is_static = 1;
            g.ctm = ctm;
            g.sai = (float)(1.0 / (2.0 * 3.14159265358979323846 * (1.0 - ctm)));
        }
        hs.distant.push_back(g);
    }
    hs.distant_energy_total = total;
    if (hs.distant.empty()) {
        hs.distant.push_back(GDistant{});
        hs.distant_radii.push_back(0.0f);
        hs.distant_dirs.push_back(f4(0, 0, 0, 0));
        hs.distant_colors.push_back(GColor{});
    }
    // FP16 node copies: child bounds as f16 offsets from an f32 anchor
    if (fp16) {
        hs.nodes_h.resize(hs.nodes.size());
        for (size_t i = 0; i < hs.nodes.size(); i++) {
            const GNode &n = hs.nodes[i];
            GNodeH &h = hs.nodes_h[i];
            uint32_t cc = n.meta.z >> 8;
            float lo[3][4] = {{n.xlo.x, n.xlo.y, n.xlo.z, n.xlo.w}, {n.ylo.x, n.ylo.y, n.ylo.z, n.ylo.w}, {n.zlo.x, n.zlo.y, n.zlo.z, n.zlo.w}};
            float hi[3][4] = {{n.xhi.x, n.xhi.y, n.xhi.z, n.xhi.w}, {n.yhi.x, n.yhi.y, n.yhi.z, n.yhi.w}, {n.zhi.x, n.zhi.y, n.zhi.z, n.zhi.w}};
            // per axis: the min corner (anchor) and max corner of the
            // children's union; lower bounds are offsets from the min
            // corner, upper bounds from the max corner (decoded on the
            // device as fl32(anchor + extent)), so every face near the
            // node's own faces -- most of them -- is encoded by a small
            // offset, i.e. nearly exactly
            //
            // A child box that is flat on an axis (lo == hi: a floor, a wall,
            // an axis-aligned quad) must decode flat: a slab of even 1e-5
            // around a ground plane holds the origins of the rays that leave
            // the plane, which would all enter its box and test its
            // triangles.  On such an axis the plane itself is the anchor
            // and the upper bounds are encoded from it too (extent 0), so
            // the plane's offsets are 0 and exact; a node where a flat face
            // still does not decode exactly keeps its f32 bounds.
            float anchor[3], top[3];
            uint16_t ext[3] = {0, 0, 0};
            bool fits = true;
            for (int a = 0; a < 3; a++) {
                float m = INFINITY, M = -INFINITY;
                int flat = -1;
                for (uint32_t l = 0; l < cc; l++) {
                    m = std::min(m, lo[a][l]);
                    M = std::max(M, hi[a][l]);
                    if (flat < 0 && lo[a][l] == hi[a][l]) flat = (int)l;
                }
                if (flat >= 0) {
                    anchor[a] = lo[a][flat];
                    ext[a] = 0;
                } else {
                    anchor[a] = std::isfinite(m) ? m : 0.0f;
                    if (std::isfinite(M) && std::isfinite(m)) fits = fits && f16_offset(anchor[a], M, +1, ext[a]);
                }
                top[a] = anchor[a] + f16_value(ext[a]);
            }
            uint16_t q[6][4];
            for (int a = 0; a < 3; a++)
                for (int l = 0; l < 4; l++) {
                    if ((uint32_t)l >= cc) {
                        q[a * 2][l] = 0x7C00;      // +inf lo
                        q[a * 2 + 1][l] = 0xFC00;  // -inf hi
                        continue;
                    }
                    fits = fits && f16_offset(anchor[a], lo[a][l], -1, q[a * 2][l]) &&
                           f16_offset(top[a], hi[a][l], +1, q[a * 2 + 1][l]);
                    if (fits && lo[a][l] == hi[a][l])  // a flat face decodes exactly, or the node stays f32
                        fits = anchor[a] + f16_value(q[a * 2][l]) == lo[a][l] &&
                               top[a] + f16_value(q[a * 2 + 1][l]) == hi[a][l];
                }
            // bit 16: motion keys, bit 17: an offset does not fit an f16; either
            // way the traversal reads this node's f32 copy
            uint32_t meta = (n.meta.z & 0xFFFFu) | ((n.meta.y > 1 ? 1u : 0u) << 16) | ((fits ? 0u : 1u) << 17);
            float metaf;
            std::memcpy(&metaf, &meta, 4);
            h.anchor = f4(anchor[0], anchor[1], anchor[2], metaf);
            h.ext = make_uint2((uint32_t)ext[0] | ((uint32_t)ext[1] << 16), (uint32_t)ext[2]);
            auto pack = [&](int s) { return make_uint2((uint32_t)q[s][0] | ((uint32_t)q[s][1] << 16), (uint32_t)q[s][2] | ((uint32_t)q[s][3] << 16)); };
            h.xlo = pack(0); h.xhi = pack(1); h.ylo = pack(2); h.yhi = pack(3); h.zlo = pack(4); h.zhi = pack(5);
            h.pad = make_uint2(0u, 0u);
            h.child = n.child;
        }
    }
    // spectrum tables: every constant XYZ colour the scene stores (shader
    // colours, light and distant-light colour keys, the background) gets an
    // index; the device builds the table of each at upload
    hs.spec_xyz.clear();
    auto index_color = [&](GColor &c) {
        if ((c.kind & PSY_COLOR_KIND_MASK) != PSY_COLOR_XYZ_K || hs.spec_xyz.size() >= 0xFFFEu) return;
        c.kind = (c.kind & PSY_COLOR_KIND_MASK) | ((uint32_t)(hs.spec_xyz.size() + 1) << 16);
        hs.spec_xyz.push_back(f4(c.a, c.b, c.c, 0.0f));
    };
    for (GShader &g : hs.shaders) index_color(g.color);
    for (GColor &c : hs.light_colors) index_color(c);
    for (GColor &c : hs.distant_colors) index_color(c);
    index_color(hs.background);
    if (hs.nodes.empty()) hs.nodes.push_back(GNode{});
    if (hs.bounds_ext.empty()) hs.bounds_ext.push_back(GBounds4{});
    if (hs.tri_idx.empty()) { hs.tri_idx.push_back(make_uint4(0, 0, 0, 0)); hs.tris.resize(3, f4(0, 0, 0, 0)); }
    if (hs.verts.empty()) { hs.verts.push_back(f4(0, 0, 0, 0)); hs.normals.push_back(f4(0, 0, 0, 0)); }
    if (hs.meshes.empty()) hs.meshes.push_back(GMesh{});
    if (hs.instances.empty()) hs.instances.push_back(GInstance{});
    if (hs.shaders.empty()) hs.shaders.push_back(GShader{});
    if (hs.lights.empty()) hs.lights.push_back(GLight{});
    if (hs.light_dims.empty()) { hs.light_dims.push_back(make_float2(0, 0)); hs.light_colors.push_back(GColor{}); }
    return PSY_OK;
}
