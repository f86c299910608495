// Oracle (test infrastructure only): CPU restatement of Psychopath's scene
// build, BVH4 packet traversal, lights, light tree, path state machine and
// bucket renderer.  Each section cites the reference file it follows.
#include "psy_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <mutex>
#include <thread>
#include <vector>

#include "oracle_shading.h"

using namespace psyo;

namespace {

// ======================================================================= bbox
// src/bbox.rs
struct BBox {
    V3 min, max;
};
static inline BBox bbox_new() { return BBox{v3(INFINITY, INFINITY, INFINITY), v3(-INFINITY, -INFINITY, -INFINITY)}; }
static inline BBox bunion(BBox a, BBox b) { return BBox{vmin3(a.min, b.min), vmax3(a.max, b.max)}; }
static inline BBox bunion_pt(BBox a, V3 p) { return BBox{vmin3(a.min, p), vmax3(a.max, p)}; }
static inline real surface_area(BBox b) {
    V3 d = b.max - b.min;
    return ((d.x * d.y) + (d.y * d.z) + (d.z * d.x)) * 2.0f;
}
static inline V3 bcenter(BBox b) { return lerp3(b.min, b.max, 0.5f); }
static inline real diagonal(BBox b) { return length(b.max - b.min); }
static inline real diagonal2(BBox b) { return length2(b.max - b.min); }
static inline BBox blerp(BBox a, BBox b, real alpha) { return BBox{lerp3(a.min, b.min, alpha), lerp3(a.max, b.max, alpha)}; }
static inline BBox lerp_slice_bbox(const BBox *s, size_t n, real alpha) {
    size_t i; real a2;
    if (lerp_slice_index(n, alpha, &i, &a2)) return s[i];
    return blerp(s[i], s[i + 1], a2);
}
// BBox::transformed (src/bbox.rs:58-81)
static BBox btransformed(BBox b, const Xf &x) {
    V3 vs[8] = {v3(b.min.x, b.min.y, b.min.z), v3(b.min.x, b.min.y, b.max.z), v3(b.min.x, b.max.y, b.min.z),
                v3(b.min.x, b.max.y, b.max.z), v3(b.max.x, b.min.y, b.min.z), v3(b.max.x, b.min.y, b.max.z),
                v3(b.max.x, b.max.y, b.min.z), v3(b.max.x, b.max.y, b.max.z)};
    BBox o = bbox_new();
    for (int i = 0; i < 8; i++) {
        V3 v = xf_point(vs[i], x);
        o.min = vmin3(v, o.min);
        o.max = vmax3(v, o.max);
    }
    return o;
}
// transform_bbox_slice_from (src/bbox.rs:153-174)
static void transform_bbox_slice_from(const std::vector<BBox> &in, const Xf *xf, size_t nx, std::vector<BBox> &out) {
    out.clear();
    if (nx == 0) {
        out = in;
    } else if (in.size() == nx) {
        for (size_t i = 0; i < nx; i++) out.push_back(btransformed(in[i], xf_inverse(xf[i])));
    } else if (in.size() > nx) {
        real s = (real)(in.size() - 1);
        for (size_t i = 0; i < in.size(); i++) out.push_back(btransformed(in[i], xf_inverse(lerp_slice_xf(xf, nx, (real)i / s))));
    } else {
        real s = (real)(nx - 1);
        for (size_t i = 0; i < nx; i++) out.push_back(btransformed(lerp_slice_bbox(in.data(), in.size(), (real)i / s), xf_inverse(xf[i])));
    }
}

// BBox4 (src/bbox4.rs)
struct BBox4 {
    real xmin[4], xmax[4], ymin[4], ymax[4], zmin[4], zmax[4];
};
static BBox4 bbox4_from(const BBox b[4]) {
    BBox4 o;
    for (int i = 0; i < 4; i++) {
        o.xmin[i] = b[i].min.x; o.xmax[i] = b[i].max.x;
        o.ymin[i] = b[i].min.y; o.ymax[i] = b[i].max.y;
        o.zmin[i] = b[i].min.z; o.zmax[i] = b[i].max.z;
    }
    return o;
}
static BBox4 bbox4_lerp(const BBox4 &a, const BBox4 &b, real alpha) {
    BBox4 o;
    real ia = 1.0f - alpha;
    for (int i = 0; i < 4; i++) {
        o.xmin[i] = (a.xmin[i] * ia) + (b.xmin[i] * alpha); o.xmax[i] = (a.xmax[i] * ia) + (b.xmax[i] * alpha);
        o.ymin[i] = (a.ymin[i] * ia) + (b.ymin[i] * alpha); o.ymax[i] = (a.ymax[i] * ia) + (b.ymax[i] * alpha);
        o.zmin[i] = (a.zmin[i] * ia) + (b.zmin[i] * alpha); o.zmax[i] = (a.zmax[i] * ia) + (b.zmax[i] * alpha);
    }
    return o;
}
static const real BBOX_MAXT_ADJUST = 1.00000024f;
// BBox4::intersect_ray (src/bbox4.rs:63-97); returns a 4-bit hit mask.
static inline uint32_t bbox4_intersect(const BBox4 &b, V3 o, V3 di, real max_t) {
    uint32_t mask = 0;
    for (int i = 0; i < 4; i++) {
        real t1x = (b.xmin[i] - o.x) * di.x, t1y = (b.ymin[i] - o.y) * di.y, t1z = (b.zmin[i] - o.z) * di.z;
        real t2x = (b.xmax[i] - o.x) * di.x, t2y = (b.ymax[i] - o.y) * di.y, t2z = (b.zmax[i] - o.z) * di.z;
        real fx = vmax(t1x, t2x), fy = vmax(t1y, t2y), fz = vmax(t1z, t2z);
        real nx = vmin(t1x, t2x), ny = vmin(t1y, t2y), nz = vmin(t1z, t2z);
        real far_t = vmin(vmin(fx, vmin(fy, fz)) * BBOX_MAXT_ADJUST, max_t);
        real near_t = vmax(vmax(nx, ny), vmax(nz, 0.0f));
        if (near_t < far_t) mask |= 1u << i;
    }
    return mask;
}

// ================================================================ BVH base build
// src/accel/bvh_base.rs, src/accel/objects_split.rs, src/algorithm.rs
static const size_t BVH_MAX_DEPTH = 42;
static const real USE_UNION_FACTOR = 1.4f;
static const int SAH_BIN_COUNT = 13;

struct BoundsSlice {
    const BBox *p;
    size_t n;
};
template <class Bounder>
struct Splitter {
    const Bounder &bounder;
    // algorithm::partition (src/algorithm.rs:44-81): two-pointer in-place partition
    template <class Pred>
    static size_t partition(uint32_t *s, size_t len, Pred pred) {
        size_t a = 0, b = len;
        while (true) {
            while (true) {
                if (a == b) return a;
                if (!pred(s[a])) break;
                a++;
            }
            while (true) {
                b--;
                if (a == b) return a;
                if (pred(s[b])) break;
            }
            std::swap(s[a], s[b]);
            a++;
        }
    }
    BBox tb(uint32_t o) const {
        BoundsSlice bs = bounder(o);
        return lerp_slice_bbox(bs.p, bs.n, 0.5f);
    }
    // sah_split (src/accel/objects_split.rs:153-238)
    void sah_split(uint32_t *objs, size_t len, size_t *split_i, size_t *split_axis) const {
        BBox bounds = bbox_new();
        for (size_t i = 0; i < len; i++) bounds = bunion_pt(bounds, bcenter(tb(objs[i])));
        real divs[3][SAH_BIN_COUNT - 1];
        for (int d = 0; d < 3; d++) {
            real extent = bounds.max[d] - bounds.min[d];
            for (int dv = 0; dv < SAH_BIN_COUNT - 1; dv++) {
                real part = extent * ((real)(dv + 1) / (real)SAH_BIN_COUNT);
                divs[d][dv] = bounds.min[d] + part;
            }
        }
        BBox binl[3][SAH_BIN_COUNT - 1], binr[3][SAH_BIN_COUNT - 1];
        size_t cntl[3][SAH_BIN_COUNT - 1] = {}, cntr[3][SAH_BIN_COUNT - 1] = {};
        for (int d = 0; d < 3; d++)
            for (int dv = 0; dv < SAH_BIN_COUNT - 1; dv++) { binl[d][dv] = bbox_new(); binr[d][dv] = bbox_new(); }
        for (size_t i = 0; i < len; i++) {
            BBox b = tb(objs[i]);
            V3 c = (b.min + b.max) * 0.5f;
            for (int d = 0; d < 3; d++)
                for (int dv = 0; dv < SAH_BIN_COUNT - 1; dv++) {
                    if (c[d] <= divs[d][dv]) { binl[d][dv] = bunion(binl[d][dv], b); cntl[d][dv]++; }
                    else { binr[d][dv] = bunion(binr[d][dv], b); cntr[d][dv]++; }
                }
        }
        int dim = 0;
        real div_n = 0.0f, smallest = INFINITY;
        for (int d = 0; d < 3; d++)
            for (int dv = 0; dv < SAH_BIN_COUNT - 1; dv++) {
                real lc = surface_area(binl[d][dv]) * (real)cntl[d][dv];
                real rc = surface_area(binr[d][dv]) * (real)cntr[d][dv];
                real ld = diagonal(binl[d][dv]), rd = diagonal(binr[d][dv]);
                real tot = (lc * ld) + (rc * rd);
                if (tot < smallest) { dim = d; div_n = divs[d][dv]; smallest = tot; }
            }
        size_t si = partition(objs, len, [&](uint32_t o) {
            BBox b = tb(o);
            real c = (b.min[dim] + b.max[dim]) * 0.5f;
            return c < div_n;
        });
        if (si < 1) si = 1;
        else if (si >= len) si = len - 1;
        *split_i = si;
        *split_axis = (size_t)dim;
    }
    // quick_select (src/algorithm.rs:134-162)
    template <class Less>
    static void quick_select(uint32_t *s, size_t len, size_t n, Less less) {
        size_t left = 0, right = len;
        uint64_t seed = (uint64_t)n;
        while (true) {
            size_t i = left + (size_t)(hash_u64((uint64_t)right, seed) % (uint64_t)(right - left));
            std::swap(s[i], s[right - 1]);
            uint32_t val = s[right - 1];
            size_t ii = left + partition(s + left, right - 1 - left, [&](uint32_t x) { return less(x, val); });
            std::swap(s[ii], s[right - 1]);
            if (ii == n) return;
            if (ii > n) right = ii;
            else left = ii + 1;
            seed += 1;
        }
    }
    // median_split (src/accel/objects_split.rs:291-341)
    void median_split(uint32_t *objs, size_t len, size_t *split_i, size_t *split_axis) const {
        BBox bounds = bbox_new();
        for (size_t i = 0; i < len; i++) bounds = bunion(bounds, tb(objs[i]));
        int axis = 0;
        real largest = -INFINITY;
        for (int i = 0; i < 3; i++) {
            real e = bounds.max[i] - bounds.min[i];
            if (e > largest) { largest = e; axis = i; }
        }
        size_t place = len / 2;
        if (place == 0) place = 1;
        quick_select(objs, len, place, [&](uint32_t a, uint32_t b) {
            BBox ta = tb(a), tbb = tb(b);
            real ca = (ta.min[axis] + ta.max[axis]) * 0.5f;
            real cb = (tbb.min[axis] + tbb.max[axis]) * 0.5f;
            return ca < cb;
        });
        *split_i = place;
        *split_axis = (size_t)axis;
    }
};

struct BaseNode {
    bool leaf;
    size_t b0, b1;      // bounds range
    size_t c0, c1;      // children (internal)
    uint8_t split_axis;
    size_t o0, o1;      // object range (leaf)
};
static size_t log2_64(uint64_t n) { return n == 0 ? 0 : (size_t)(63 - __builtin_clzll(n)); }

// merge_slices_append (src/algorithm.rs:174-203) for BBox union
static void merge_bounds(const BBox *a, size_t na, const BBox *b, size_t nb, std::vector<BBox> &out) {
    if (na == 0 || nb == 0) return;
    if (na == nb) {
        for (size_t i = 0; i < na; i++) out.push_back(bunion(a[i], b[i]));
    } else if (na > nb) {
        real s = (real)(na - 1);
        for (size_t i = 0; i < na; i++) out.push_back(bunion(a[i], lerp_slice_bbox(b, nb, (real)i / s)));
    } else {
        real s = (real)(nb - 1);
        for (size_t i = 0; i < nb; i++) out.push_back(bunion(lerp_slice_bbox(a, na, (real)i / s), b[i]));
    }
}

template <class Bounder>
struct BVHBase {
    std::vector<BaseNode> nodes;
    std::vector<BBox> bounds;
    size_t depth = 0;
    const Bounder &bounder;
    explicit BVHBase(const Bounder &b) : bounder(b) {}

    // reduce time samples to their union when that is not much bigger
    void push_reduced(std::vector<BBox> &samples) {
        BBox u = bbox_new();
        for (auto &b : samples) u = bunion(u, b);
        real avg = 0.0f;
        for (auto &b : samples) avg = avg + surface_area(b);
        avg = avg / (real)samples.size();
        if (surface_area(u) <= (avg * USE_UNION_FACTOR)) bounds.push_back(u);
        else bounds.insert(bounds.end(), samples.begin(), samples.end());
    }

    // recursive_build (src/accel/bvh_base.rs:96-215); returns (node, bounds range)
    size_t build(size_t offset, size_t d, size_t per_leaf, uint32_t *objs, size_t len, size_t *rb0, size_t *rb1) {
        size_t me = nodes.size();
        if (len == 0) { *rb0 = 0; *rb1 = 0; return 0; }
        if (len <= per_leaf) {
            size_t bi = bounds.size();
            // acc_bounds
            size_t max_len = 0;
            for (size_t i = 0; i < len; i++) max_len = std::max(max_len, bounder(objs[i]).n);
            std::vector<BBox> cache(max_len, bbox_new());
            for (size_t i = 0; i < len; i++) {
                BoundsSlice bs = bounder(objs[i]);
                if (bs.n == max_len) {
                    for (size_t k = 0; k < bs.n; k++) cache[k] = bunion(cache[k], bs.p[k]);
                } else {
                    real s = (real)(max_len - 1);
                    for (size_t k = 0; k < max_len; k++) cache[k] = bunion(cache[k], lerp_slice_bbox(bs.p, bs.n, (real)k / s));
                }
            }
            push_reduced(cache);
            BaseNode n{};
            n.leaf = true; n.b0 = bi; n.b1 = bounds.size(); n.o0 = offset; n.o1 = offset + len;
            nodes.push_back(n);
            if (depth < d) depth = d;
            *rb0 = bi; *rb1 = bounds.size();
            return me;
        }
        nodes.push_back(BaseNode{});
        Splitter<Bounder> sp{bounder};
        size_t split_i, axis;
        if (log2_64((uint64_t)len) < (BVH_MAX_DEPTH - d)) sp.sah_split(objs, len, &split_i, &axis);
        else sp.median_split(objs, len, &split_i, &axis);
        size_t c1b0, c1b1, c2b0, c2b1;
        size_t c1 = build(offset, d + 1, per_leaf, objs, split_i, &c1b0, &c1b1);
        size_t c2 = build(offset + split_i, d + 1, per_leaf, objs + split_i, len - split_i, &c2b0, &c2b1);
        size_t bi = bounds.size();
        std::vector<BBox> merged;
        merge_bounds(&bounds[c1b0], c1b1 - c1b0, &bounds[c2b0], c2b1 - c2b0, merged);
        push_reduced(merged);
        BaseNode &n = nodes[me];
        n.leaf = false; n.b0 = bi; n.b1 = bounds.size(); n.c0 = c1; n.c1 = c2; n.split_axis = (uint8_t)axis;
        *rb0 = bi; *rb1 = bounds.size();
        return me;
    }
};

// ======================================================================= BVH4
// src/accel/bvh4.rs and sub_crates/bvh_order
static uint8_t TRAVERSAL_TABLE[8][48];
static void build_traversal_table() {
    for (int raydir = 0; raydir < 8; raydir++) {
        int ray[3] = {raydir & 1, (raydir >> 1) & 1, (raydir >> 2) & 1};
        int k = 0;
        for (int s2 = 0; s2 < 3; s2++)
            for (int s1 = 0; s1 < 3; s1++)
                for (int s0 = 0; s0 < 3; s0++) {
                    int perm[4] = {0, 1, 2, 3};
                    if (ray[s1] == 1) std::swap(perm[0], perm[1]);
                    if (ray[s2] == 1) std::swap(perm[2], perm[3]);
                    if (ray[s0] == 1) { std::swap(perm[0], perm[2]); std::swap(perm[1], perm[3]); }
                    TRAVERSAL_TABLE[raydir][k++] = (uint8_t)(perm[0] + (perm[1] << 2) + (perm[2] << 4) + (perm[3] << 6));
                }
        for (int s1 = 0; s1 < 3; s1++)
            for (int s0 = 0; s0 < 3; s0++) {
                int perm[3] = {0, 1, 2};
                if (ray[s1] == 1) std::swap(perm[0], perm[1]);
                if (ray[s0] == 1) { std::swap(perm[0], perm[1]); std::swap(perm[0], perm[2]); }
                TRAVERSAL_TABLE[raydir][k++] = (uint8_t)(perm[0] + (perm[1] << 2) + (perm[2] << 4));
            }
        for (int s1 = 0; s1 < 3; s1++)
            for (int s0 = 0; s0 < 3; s0++) {
                int perm[3] = {0, 1, 2};
                if (ray[s1] == 1) std::swap(perm[1], perm[2]);
                if (ray[s0] == 1) { std::swap(perm[0], perm[2]); std::swap(perm[0], perm[1]); }
                TRAVERSAL_TABLE[raydir][k++] = (uint8_t)(perm[0] + (perm[1] << 2) + (perm[2] << 4));
            }
        for (int s0 = 0; s0 < 3; s0++) {
            int perm[2] = {0, 1};
            if (ray[s0] == 1) std::swap(perm[0], perm[1]);
            TRAVERSAL_TABLE[raydir][k++] = (uint8_t)(perm[0] + (perm[1] << 2));
        }
    }
}
static struct TableInit { TableInit() { build_traversal_table(); } } g_table_init;

struct Node4 {
    bool leaf;
    size_t o0, o1;          // leaf object range
    size_t child0;          // internal: index of first child in the node pool
    uint32_t child_count;
    size_t bounds0, nbounds;  // internal: BBox4 time keys
    uint8_t traversal_code;
};
struct BVH4 {
    std::vector<Node4> nodes;   // nodes[0] = root
    std::vector<BBox4> bounds;
    std::vector<BBox> root_bounds;
    bool empty = true;
};

template <class Bounder>
static size_t construct_from_base(BVH4 &out, const BVHBase<Bounder> &base, size_t bn, size_t slot) {
    size_t count = 0;
    const BaseNode &n = base.nodes[bn];
    if (n.leaf) {
        Node4 &o = out.nodes[slot];
        o.leaf = true; o.o0 = n.o0; o.o1 = n.o1;
        return 1;
    }
    const BaseNode &l = base.nodes[n.c0];
    const BaseNode &r = base.nodes[n.c1];
    const BaseNode *ch[4] = {nullptr, nullptr, nullptr, nullptr};
    uint32_t cc;
    uint8_t code;
    if (!l.leaf && !r.leaf) {
        cc = 4;
        ch[0] = &base.nodes[l.c0]; ch[1] = &base.nodes[l.c1]; ch[2] = &base.nodes[r.c0]; ch[3] = &base.nodes[r.c1];
        code = (uint8_t)(n.split_axis + l.split_axis * 3 + r.split_axis * 9);
    } else if (!l.leaf && r.leaf) {
        cc = 3;
        ch[0] = &base.nodes[l.c0]; ch[1] = &base.nodes[l.c1]; ch[2] = &r;
        code = (uint8_t)(n.split_axis + l.split_axis * 3 + 27);
    } else if (l.leaf && !r.leaf) {
        cc = 3;
        ch[0] = &l; ch[1] = &base.nodes[r.c0]; ch[2] = &base.nodes[r.c1];
        code = (uint8_t)(n.split_axis + r.split_axis * 3 + 27 + 9);
    } else {
        cc = 2;
        ch[0] = &l; ch[1] = &r;
        code = (uint8_t)(n.split_axis + 27 + 9 + 9);
    }
    count += cc;
    size_t blen = 0;
    for (uint32_t i = 0; i < 4; i++)
        if (ch[i]) blen = std::max(blen, ch[i]->b1 - ch[i]->b0);
    size_t b0 = out.bounds.size();
    if (blen < 2) {
        BBox bb[4];
        for (int i = 0; i < 4; i++) bb[i] = ch[i] ? base.bounds[ch[i]->b0] : bbox_new();
        out.bounds.push_back(bbox4_from(bb));
    } else {
        for (size_t k = 0; k < blen; k++) {
            real time = (real)k / (real)(blen - 1);
            BBox bb[4];
            for (int i = 0; i < 4; i++)
                bb[i] = ch[i] ? lerp_slice_bbox(&base.bounds[ch[i]->b0], ch[i]->b1 - ch[i]->b0, time) : bbox_new();
            out.bounds.push_back(bbox4_from(bb));
        }
    }
    size_t c0 = out.nodes.size();
    out.nodes.resize(out.nodes.size() + cc);
    for (uint32_t i = 0; i < cc; i++)
        count += construct_from_base(out, base, (size_t)(ch[i] - base.nodes.data()), c0 + i);
    Node4 &o = out.nodes[slot];
    o.leaf = false; o.child0 = c0; o.child_count = cc; o.bounds0 = b0; o.nbounds = blen < 2 ? 1 : blen;
    o.traversal_code = code;
    return count;
}

template <class Bounder>
static void bvh4_from_objects(BVH4 &out, uint32_t *objs, size_t len, size_t per_leaf, const Bounder &bounder) {
    out = BVH4();
    if (len == 0) return;
    BVHBase<Bounder> base(bounder);
    size_t rb0, rb1;
    base.build(0, 0, per_leaf, objs, len, &rb0, &rb1);
    out.nodes.resize(1);
    construct_from_base(out, base, 0, 0);
    const BaseNode &root = base.nodes[0];
    out.root_bounds.assign(base.bounds.begin() + root.b0, base.bounds.begin() + root.b1);
    out.empty = false;
}

// ======================================================================= rays
// src/ray.rs
static const uint8_t OCCLUSION_FLAG = 1, DONE_FLAG = 2;
struct RayBatch {
    std::vector<V3> orig_local, dir_inv_local, orig, dir;
    std::vector<real> max_t, time, wavelength;
    std::vector<uint8_t> flags;
    size_t size() const { return orig.size(); }
    void clear() {
        orig_local.clear(); dir_inv_local.clear(); orig.clear(); dir.clear();
        max_t.clear(); time.clear(); wavelength.clear(); flags.clear();
    }
    void push(V3 o, V3 d, real mt, real t, real wl, bool occl) {
        orig_local.push_back(o); dir_inv_local.push_back(d);  // placeholders, as the reference
        orig.push_back(o); dir.push_back(d);
        max_t.push_back(mt); time.push_back(t); wavelength.push_back(wl);
        flags.push_back(occl ? OCCLUSION_FLAG : 0);
    }
    void set_from_ray(size_t i, V3 o, V3 d, real mt, real t, real wl, bool occl) {
        orig_local[i] = o;
        dir_inv_local[i] = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
        max_t[i] = mt; time[i] = t;
        flags[i] = occl ? OCCLUSION_FLAG : 0;
        orig[i] = o; dir[i] = d; wavelength[i] = wl;
    }
    void swap(size_t a, size_t b) {
        std::swap(orig_local[a], orig_local[b]); std::swap(dir_inv_local[a], dir_inv_local[b]);
        std::swap(orig[a], orig[b]); std::swap(dir[a], dir[b]);
        std::swap(max_t[a], max_t[b]); std::swap(time[a], time[b]); std::swap(wavelength[a], wavelength[b]);
        std::swap(flags[a], flags[b]);
    }
    void truncate(size_t n) {
        orig_local.resize(n); dir_inv_local.resize(n); orig.resize(n); dir.resize(n);
        max_t.resize(n); time.resize(n); wavelength.resize(n); flags.resize(n);
    }
    void update_local(size_t i, const Xf &x) {
        orig_local[i] = xf_point(orig[i], x);
        V3 d = xf_vector(dir[i], x);
        dir_inv_local[i] = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    }
    bool is_occlusion(size_t i) const { return (flags[i] & OCCLUSION_FLAG) != 0; }
    bool is_done(size_t i) const { return (flags[i] & DONE_FLAG) != 0; }
    void mark_done(size_t i) { flags[i] |= DONE_FLAG; }
};

// RayStack (src/ray.rs:199-383): lanes of u16 ray indices and a task stack.
struct Lane {
    std::vector<uint16_t> buf;
    size_t len = 0, end_len = 0;
    void push(uint16_t v) {
        if (len < buf.size()) buf[len] = v;
        else buf.push_back(v);
        len++;
    }
};
struct Task {
    uint32_t lane;
    size_t start;
};
struct RayStack {
    std::vector<Lane> lanes;
    std::vector<Task> tasks;
    bool empty() const { return tasks.empty(); }
    void ensure_lanes(size_t n) { while (lanes.size() < n) lanes.emplace_back(); }
    void clear() {
        for (auto &l : lanes) { l.len = 0; l.end_len = 0; }
        tasks.clear();
    }
    size_t next_count() const { const Task &t = tasks.back(); return lanes[t.lane].end_len - t.start; }
    uint16_t next_ray(size_t i) const { const Task &t = tasks.back(); return lanes[t.lane].buf[t.start + i]; }
    bool push_lane_to_task(uint32_t l) {
        if (lanes[l].end_len < lanes[l].len) {
            tasks.push_back(Task{l, lanes[l].end_len});
            lanes[l].end_len = lanes[l].len;
            return true;
        }
        return false;
    }
    void duplicate_next_task() {
        Task t = tasks.back();
        Lane &ln = lanes[t.lane];
        size_t start = t.start, end = ln.end_len;
        for (size_t i = start; i < end; i++) ln.push(ln.buf[i]);
        tasks.push_back(Task{t.lane, end});
        ln.end_len = ln.len;
    }
    void pop_task() {
        Task t = tasks.back();
        tasks.pop_back();
        lanes[t.lane].end_len = t.start;
        lanes[t.lane].len = t.start;
    }
    template <class F>
    void do_next_task(F f) {
        Task t = tasks.back();
        size_t e = lanes[t.lane].end_len;
        for (size_t i = t.start; i < e; i++) f(lanes[t.lane].buf[i]);
    }
    template <class F>
    void pop_do_next_task(F f) { do_next_task(f); pop_task(); }
    template <class F>
    void pop_do_next_task_and_push_rays(uint32_t out_lanes, F f) {
        Task t = tasks.back();
        tasks.pop_back();
        size_t s = t.start, e = lanes[t.lane].end_len;
        lanes[t.lane].end_len = t.start;
        lanes[t.lane].len = t.start;
        for (size_t i = s; i < e; i++) {
            uint16_t idx = lanes[t.lane].buf[i];
            uint32_t m = f(idx);
            for (uint32_t l = 0; l < out_lanes; l++)
                if (m & (1u << l)) lanes[l].push(idx);
        }
    }
};
static inline uint32_t ray_code(V3 d) {
    return (uint32_t)(d.x < 0.0f) + ((uint32_t)(d.y < 0.0f) << 1) + ((uint32_t)(d.z < 0.0f) << 2);
}

// ======================================================================= triangle
// src/surface/triangle.rs
struct TriPre {
    int i[3];
    real s[3];
};
static inline TriPre tri_precompute(V3 d) {
    real xa = std::fabs(d.x), ya = std::fabs(d.y), za = std::fabs(d.z);
    TriPre p;
    if (xa > ya && xa > za) { p.i[0] = 1; p.i[1] = 2; p.i[2] = 0; }
    else if (ya > za) { p.i[0] = 2; p.i[1] = 0; p.i[2] = 1; }
    else { p.i[0] = 0; p.i[1] = 1; p.i[2] = 2; }
    real dx = d[p.i[0]], dy = d[p.i[1]], dz = d[p.i[2]];
    p.s[0] = dx / dz; p.s[1] = dy / dz; p.s[2] = 1.0f / dz;
    return p;
}
static inline real max_abs_3(real a, real b, real c) {
    a = std::fabs(a); b = std::fabs(b); c = std::fabs(c);
    if (a > b && a > c) return a;
    if (b > c) return b;
    return c;
}
static inline bool tri_intersect(V3 o, const TriPre &pre, real max_t, V3 t0, V3 t1, V3 t2, real out[4]) {
    V3 p0 = t0 - o, p1 = t1 - o, p2 = t2 - o;
    real p0x = p0[pre.i[0]] - (pre.s[0] * p0[pre.i[2]]);
    real p0y = p0[pre.i[1]] - (pre.s[1] * p0[pre.i[2]]);
    real p1x = p1[pre.i[0]] - (pre.s[0] * p1[pre.i[2]]);
    real p1y = p1[pre.i[1]] - (pre.s[1] * p1[pre.i[2]]);
    real p2x = p2[pre.i[0]] - (pre.s[0] * p2[pre.i[2]]);
    real p2y = p2[pre.i[1]] - (pre.s[1] * p2[pre.i[2]]);
    real e0 = (p1x * p2y) - (p1y * p2x);
    real e1 = (p2x * p0y) - (p2y * p0x);
    real e2 = (p0x * p1y) - (p0y * p1x);
    if (e0 == 0.0f || e1 == 0.0f || e2 == 0.0f) {
        e0 = (real)(((double)p1x * (double)p2y) - ((double)p1y * (double)p2x));
        e1 = (real)(((double)p2x * (double)p0y) - ((double)p2y * (double)p0x));
        e2 = (real)(((double)p0x * (double)p1y) - ((double)p0y * (double)p1x));
    }
    if ((e0 < 0.0f || e1 < 0.0f || e2 < 0.0f) && (e0 > 0.0f || e1 > 0.0f || e2 > 0.0f)) return false;
    real det = e0 + e1 + e2;
    if (det == 0.0f) return false;
    real p0z = pre.s[2] * p0[pre.i[2]];
    real p1z = pre.s[2] * p1[pre.i[2]];
    real p2z = pre.s[2] * p2[pre.i[2]];
    real t_scaled = (e0 * p0z) + (e1 * p1z) + (e2 * p2z);
    if ((det > 0.0f && (t_scaled <= 0.0f || t_scaled > (max_t * det))) ||
        (det < 0.0f && (t_scaled >= 0.0f || t_scaled < (max_t * det))))
        return false;
    real inv_det = 1.0f / det;
    real b0 = e0 * inv_det, b1 = e1 * inv_det, b2 = e2 * inv_det;
    real t = t_scaled * inv_det;
    real max_zt = max_abs_3(p0z, p1z, p2z);
    real dz = fp_gamma(3) * max_zt;
    real max_xt = max_abs_3(p0x, p1x, p2x);
    real max_yt = max_abs_3(p0y, p1y, p2y);
    real dx = fp_gamma(5) * (max_xt + max_zt);
    real dy = fp_gamma(5) * (max_yt + max_zt);
    real de = 2.0f * ((fp_gamma(2) * max_xt * max_yt) + (dy * max_xt + dx * max_yt));
    real max_e = max_abs_3(e0, e1, e2);
    real dt = 3.0f * ((fp_gamma(3) * max_e * max_zt) + (de * max_zt + dz * max_e)) * std::fabs(inv_det);
    if (t <= dt) return false;
    out[0] = t; out[1] = b0; out[2] = b1; out[3] = b2;
    return true;
}
static inline void surface_point(V3 t0, V3 t1, V3 t2, real b0, real b1, real b2, V3 *pos, real *err) {
    *pos = (t0 * b0) + (t1 * b1) + (t2 * b2);
    V3 e = ((vabs(t0) * b0) + (vabs(t1) * b1) + (vabs(t2) * b2)) * fp_gamma(7);
    *err = max_elem3(e);
}

// ======================================================================= scene
struct Isect {
    uint32_t kind;  // PSY_HIT_*
    uint32_t prim, inst;
    real t, b0, b1, b2;
    V3 incoming, pos, nor, nor_g;
    real pos_err, sample_pdf;
    Closure closure;
    int32_t shader;
};

struct Mesh {
    uint32_t ts;  // time samples
    std::vector<V3> verts;    // [vert][ts]
    std::vector<V3> normals;  // same, or empty
    std::vector<uint32_t> idx;  // [tri][4] = (v0, v2, v1, orig), in BVH order
    BVH4 accel;
};
struct RectLight {
    std::vector<real> dims;  // [key][2]
    std::vector<Color> colors;
    std::vector<BBox> bounds;
};
struct SphereLight {
    std::vector<real> radii;
    std::vector<Color> colors;
    std::vector<BBox> bounds;
};
struct Object {
    uint32_t kind;
    uint32_t index;  // into meshes / rects / spheres
};
struct Instance {
    uint32_t object;
    int32_t shader;
    uint32_t id;
    uint32_t xs, xc;
};
struct DistantLight {
    std::vector<real> radii;
    std::vector<V3> dirs;
    std::vector<Color> colors;
};
struct LightTreeNode {
    bool leaf;
    size_t light_index;     // leaf: index into light_instances
    size_t child0, nchild;  // inner: children in pool
    std::vector<BBox> bounds;
    real energy;
};

static Color to_color(const PsyColor &c) { return Color{c.kind, c.v[0], c.v[1], c.v[2]}; }

}  // namespace

struct PsyoScene {
    std::vector<Mesh> meshes;
    std::vector<RectLight> rects;
    std::vector<SphereLight> spheres;
    std::vector<Object> objects;
    std::vector<Closure> shaders;
    std::vector<Instance> instances;   // BVH order
    std::vector<Instance> light_instances;
    std::vector<Xf> xforms;
    BVH4 object_accel;
    std::vector<LightTreeNode> lt;  // [0] = root when non-empty
    bool lt_empty = true;
    // camera
    std::vector<Xf> cam_xf;
    std::vector<real> cam_tfov, cam_ap, cam_fd;
    Color background;
    std::vector<DistantLight> distant;
    uint32_t width, height, spp, seed, max_bounces;
};

namespace {

// ======================================================================= light tree
// src/accel/light_tree.rs
struct LTBuilderNode {
    bool leaf;
    size_t b0, b1;
    real energy;
    size_t child_index;
};
struct LTBuilder {
    std::vector<LTBuilderNode> nodes;
    std::vector<BBox> bounds;
    const std::vector<std::vector<BBox>> &inst_bounds;  // by instance id
    const std::vector<real> &inst_energy;              // by light instance slot value
    std::vector<Instance> &lights;
    LTBuilder(const std::vector<std::vector<BBox>> &ib, const std::vector<real> &ie, std::vector<Instance> &l)
        : inst_bounds(ib), inst_energy(ie), lights(l) {}

    size_t build(size_t offset, uint32_t *objs, size_t len, size_t *rb0, size_t *rb1) {
        size_t me = nodes.size();
        if (len == 0) { *rb0 = *rb1 = 0; return 0; }
        if (len == 1) {
            size_t bi = bounds.size();
            const std::vector<BBox> &ob = inst_bounds[lights[objs[0]].id];
            bounds.insert(bounds.end(), ob.begin(), ob.end());
            nodes.push_back(LTBuilderNode{true, bi, bounds.size(), inst_energy[objs[0]], offset});
            *rb0 = bi; *rb1 = bounds.size();
            return me;
        }
        nodes.push_back(LTBuilderNode{false, 0, 0, 0.0f, 0});
        auto bounder = [&](uint32_t o) {
            const std::vector<BBox> &b = inst_bounds[lights[o].id];
            return BoundsSlice{b.data(), b.size()};
        };
        Splitter<decltype(bounder)> sp{bounder};
        size_t split_i, axis;
        sp.sah_split(objs, len, &split_i, &axis);
        size_t c1b0, c1b1, c2b0, c2b1;
        build(offset, objs, split_i, &c1b0, &c1b1);
        size_t c2 = build(offset + split_i, objs + split_i, len - split_i, &c2b0, &c2b1);
        size_t bi = bounds.size();
        std::vector<BBox> merged;
        merge_bounds(&bounds[c1b0], c1b1 - c1b0, &bounds[c2b0], c2b1 - c2b0, merged);
        bounds.insert(bounds.end(), merged.begin(), merged.end());
        real e = nodes[me + 1].energy + nodes[c2].energy;
        nodes[me] = LTBuilderNode{false, bi, bounds.size(), e, c2};
        *rb0 = bi; *rb1 = bounds.size();
        return me;
    }
    size_t child_count_rec(size_t lc, size_t ni) const {
        if (lc > 0) {
            if (nodes[ni].leaf) return 1;
            return child_count_rec(lc - 1, ni + 1) + child_count_rec(lc - 1, nodes[ni].child_index);
        }
        return 1;
    }
    void nth_child_rec(size_t lc, size_t ni, size_t n, size_t *idx, size_t *rem) const {
        if (lc > 0 && !nodes[ni].leaf) {
            size_t i, r;
            nth_child_rec(lc - 1, ni + 1, n, &i, &r);
            if (r == 0) { *idx = i; *rem = 0; return; }
            nth_child_rec(lc - 1, nodes[ni].child_index, r - 1, idx, rem);
            return;
        }
        *idx = ni; *rem = n;
    }
};
static void lt_construct(PsyoScene &s, const LTBuilder &b, size_t ni, size_t slot) {
    const LTBuilderNode &n = b.nodes[ni];
    LightTreeNode &o = s.lt[slot];
    o.bounds.assign(b.bounds.begin() + n.b0, b.bounds.begin() + n.b1);
    o.energy = n.energy;
    if (n.leaf) {
        o.leaf = true;
        o.light_index = n.child_index;
        return;
    }
    size_t cc = b.child_count_rec(3, ni);
    size_t c0 = s.lt.size();
    s.lt.resize(c0 + cc);
    s.lt[slot].leaf = false;
    s.lt[slot].child0 = c0;
    s.lt[slot].nchild = cc;
    for (size_t i = 0; i < cc; i++) {
        size_t idx, rem;
        b.nth_child_rec(3, ni, i, &idx, &rem);
        lt_construct(s, b, idx, c0 + i);
    }
}

}  // namespace

// ======================================================================= scene build
static real rect_energy(const RectLight &r) {
    real a = 0.0f;
    for (auto &c : r.colors) a = a + color_energy(c);
    return a / (real)r.colors.size();
}
static real sphere_energy(const SphereLight &r) {
    real a = 0.0f;
    for (auto &c : r.colors) a = a + color_energy(c);
    return a / (real)r.colors.size();
}

extern "C" PsyoScene *psyo_scene_create(const PsySceneDesc *d) {
    if (!d) return nullptr;
    PsyoScene *s = new PsyoScene();
    s->width = d->width; s->height = d->height; s->spp = d->spp; s->seed = d->seed; s->max_bounces = d->max_bounces;
    for (uint32_t i = 0; i < d->num_shaders; i++) {
        const PsyShaderDesc &sh = d->shaders[i];
        Closure c{};
        c.kind = sh.kind == PSY_SHADER_EMIT ? CL_EMIT : (sh.kind == PSY_SHADER_LAMBERT ? CL_LAMBERT : CL_GGX);
        c.color = to_color(sh.color);
        c.roughness = sh.roughness;
        c.fresnel = sh.fresnel;
        s->shaders.push_back(c);
    }
    for (uint32_t i = 0; i < d->num_xforms; i++) {
        Xf x;
        for (int k = 0; k < 12; k++) x.m[k] = d->xforms[i].m[k];
        s->xforms.push_back(x);
    }
    // objects (TriangleMesh::from_verts_and_indices, src/surface/triangle_mesh.rs:29-115)
    for (uint32_t oi = 0; oi < d->num_objects; oi++) {
        const PsyObjectDesc &od = d->objects[oi];
        Object ob{od.kind, 0};
        if (od.kind == PSY_OBJ_MESH) {
            ob.index = (uint32_t)s->meshes.size();
            s->meshes.emplace_back();
            Mesh &m = s->meshes.back();
            m.ts = od.time_samples;
            uint32_t nv = od.num_verts, ts = od.time_samples;
            m.verts.resize((size_t)nv * ts);
            for (uint32_t v = 0; v < nv; v++)
                for (uint32_t t = 0; t < ts; t++) {
                    const float *p = od.verts + ((size_t)t * nv + v) * 3;
                    m.verts[(size_t)v * ts + t] = v3(p[0], p[1], p[2]);
                }
            if (od.normals) {
                m.normals.resize((size_t)nv * ts);
                for (uint32_t v = 0; v < nv; v++)
                    for (uint32_t t = 0; t < ts; t++) {
                        const float *p = od.normals + ((size_t)t * nv + v) * 3;
                        m.normals[(size_t)v * ts + t] = v3(p[0], p[1], p[2]);
                    }
            }
            uint32_t nt = od.num_tris;
            std::vector<uint32_t> tup((size_t)nt * 4);
            std::vector<BBox> tb((size_t)nt * ts);
            for (uint32_t t = 0; t < nt; t++) {
                uint32_t a = od.indices[t * 3 + 0], b = od.indices[t * 3 + 1], c = od.indices[t * 3 + 2];
                tup[t * 4 + 0] = a; tup[t * 4 + 1] = c; tup[t * 4 + 2] = b; tup[t * 4 + 3] = t;
                for (uint32_t k = 0; k < ts; k++) {
                    const float *pa = od.verts + ((size_t)k * nv + a) * 3;
                    const float *pb = od.verts + ((size_t)k * nv + b) * 3;
                    const float *pc = od.verts + ((size_t)k * nv + c) * 3;
                    V3 p0 = v3(pa[0], pa[1], pa[2]), p1 = v3(pb[0], pb[1], pb[2]), p2 = v3(pc[0], pc[1], pc[2]);
                    V3 mn = vmin3(p0, vmin3(p1, p2));
                    V3 mx = vmax3(p0, vmax3(p1, p2));
                    tb[(size_t)t * ts + k] = BBox{mn, mx};
                }
            }
            // objects to order are original triangle indices
            std::vector<uint32_t> order(nt);
            for (uint32_t t = 0; t < nt; t++) order[t] = t;
            auto bounder = [&](uint32_t t) { return BoundsSlice{&tb[(size_t)t * ts], (size_t)ts}; };
            bvh4_from_objects(m.accel, order.data(), nt, 3, bounder);
            m.idx.resize((size_t)nt * 4);
            for (uint32_t i = 0; i < nt; i++)
                for (int k = 0; k < 4; k++) m.idx[(size_t)i * 4 + k] = tup[(size_t)order[i] * 4 + k];
        } else if (od.kind == PSY_OBJ_RECT_LIGHT) {
            ob.index = (uint32_t)s->rects.size();
            RectLight r;
            for (uint32_t k = 0; k < od.time_samples; k++) {
                real w = od.dims[k * 2], h = od.dims[k * 2 + 1];
                r.dims.push_back(w); r.dims.push_back(h);
                r.colors.push_back(to_color(od.colors[k]));
                r.bounds.push_back(BBox{v3(w * -0.5f, h * -0.5f, 0.0f), v3(w * 0.5f, h * 0.5f, 0.0f)});
            }
            s->rects.push_back(r);
        } else {
            ob.index = (uint32_t)s->spheres.size();
            SphereLight r;
            for (uint32_t k = 0; k < od.time_samples; k++) {
                real rad = od.dims[k];
                r.radii.push_back(rad);
                r.colors.push_back(to_color(od.colors[k]));
                r.bounds.push_back(BBox{v3(-rad, -rad, -rad), v3(rad, rad, rad)});
            }
            s->spheres.push_back(r);
        }
        s->objects.push_back(ob);
    }
    // instances and instance bounds (AssemblyBuilder::build / instance_bounds,
    // src/scene/assembly.rs:288-395)
    std::vector<Instance> insts;
    for (uint32_t i = 0; i < d->num_instances; i++) {
        const PsyInstanceDesc &id = d->instances[i];
        insts.push_back(Instance{id.object, id.shader, i, id.xform_start, id.xform_count});
    }
    std::vector<std::vector<BBox>> ib(insts.size());
    for (auto &in : insts) {
        const Object &ob = s->objects[in.object];
        std::vector<BBox> bbs;
        if (ob.kind == PSY_OBJ_MESH) bbs = s->meshes[ob.index].accel.root_bounds;
        else if (ob.kind == PSY_OBJ_RECT_LIGHT) bbs = s->rects[ob.index].bounds;
        else bbs = s->spheres[ob.index].bounds;
        std::vector<BBox> out;
        transform_bbox_slice_from(bbs, in.xc ? &s->xforms[in.xs] : nullptr, in.xc, out);
        ib[in.id] = out;
    }
    std::vector<uint32_t> order(insts.size());
    for (size_t i = 0; i < insts.size(); i++) order[i] = (uint32_t)i;
    auto ibounder = [&](uint32_t o) { return BoundsSlice{ib[insts[o].id].data(), ib[insts[o].id].size()}; };
    bvh4_from_objects(s->object_accel, order.data(), order.size(), 1, ibounder);
    for (auto o : order) s->instances.push_back(insts[o]);
    // light instances + light tree
    for (auto &in : s->instances) {
        uint32_t k = s->objects[in.object].kind;
        if (k == PSY_OBJ_RECT_LIGHT || k == PSY_OBJ_SPHERE_LIGHT) s->light_instances.push_back(in);
    }
    if (!s->light_instances.empty()) {
        std::vector<Instance> lights = s->light_instances;
        std::vector<real> energy(lights.size());
        for (size_t i = 0; i < lights.size(); i++) {
            const Object &ob = s->objects[lights[i].object];
            energy[i] = ob.kind == PSY_OBJ_RECT_LIGHT ? rect_energy(s->rects[ob.index]) : sphere_energy(s->spheres[ob.index]);
        }
        std::vector<uint32_t> lorder(lights.size());
        for (size_t i = 0; i < lights.size(); i++) lorder[i] = (uint32_t)i;
        LTBuilder b(ib, energy, lights);
        size_t rb0, rb1;
        b.build(0, lorder.data(), lorder.size(), &rb0, &rb1);
        s->light_instances.clear();
        for (auto o : lorder) s->light_instances.push_back(lights[o]);
        s->lt.resize(1);
        lt_construct(*s, b, 0, 0);
        s->lt_empty = false;
    }
    // camera (Camera::new, src/camera.rs:22-72)
    const PsyCameraDesc &c = d->camera;
    for (uint32_t i = 0; i < c.num_transforms; i++) {
        Xf x;
        for (int k = 0; k < 12; k++) x.m[k] = c.transforms[i].m[k];
        s->cam_xf.push_back(x);
    }
    for (uint32_t i = 0; i < c.num_fovs; i++) {
        real n = c.fovs[i];
        s->cam_tfov.push_back(std::sin(n / 2.0f) / std::cos(n / 2.0f));
    }
    std::vector<real> ap(c.aperture_radii, c.aperture_radii + c.num_aperture_radii);
    std::vector<real> fd(c.focus_distances, c.focus_distances + c.num_focus_distances);
    if (ap.empty() || fd.empty()) { ap = {0.0f}; fd = {1.0f}; }
    for (real f : fd)
        if (f == 0.0f) { ap = {0.0f}; fd = {1.0f}; break; }
    s->cam_ap = ap; s->cam_fd = fd;
    s->background = to_color(d->background);
    for (uint32_t i = 0; i < d->num_distant_lights; i++) {
        const PsyDistantLightDesc &dl = d->distant_lights[i];
        DistantLight l;
        for (uint32_t k = 0; k < dl.num_keys; k++) {
            l.radii.push_back(dl.radii[k]);
            l.dirs.push_back(v3(dl.directions[k * 3], dl.directions[k * 3 + 1], dl.directions[k * 3 + 2]));
            l.colors.push_back(to_color(dl.colors[k]));
        }
        s->distant.push_back(l);
    }
    return s;
}

extern "C" void psyo_scene_destroy(PsyoScene *s) { delete s; }

// ======================================================================= tracer
namespace {

struct Counters {
    uint64_t node_tests = 0, tri_tests = 0;
};

// Shader of instances without one: Emit of rec709_to_xyz((1, 0, 1))
// (src/tracer.rs:161-163).
static Closure unassigned_closure() {
    float rgb[3] = {1.0f, 0.0f, 1.0f}, xyz[3];
    psyo_rec709_to_xyz(rgb, xyz);
    return Closure{CL_EMIT, Color{COL_XYZ, xyz[0], xyz[1], xyz[2]}, 0.0f, 0.0f};
}

struct Tracer {
    const PsyoScene &s;
    RayStack rs;
    std::vector<Isect> isects;
    Counters cnt;
    const Xf *space = nullptr;  // transform stack top (root assembly: one level)
    size_t nspace = 0;

    explicit Tracer(const PsyoScene &sc) : s(sc) {}

    // BVH4::traverse (src/accel/bvh4.rs:101-184)
    template <class Leaf>
    void traverse(const BVH4 &bvh, RayBatch &rays, Leaf leaf) {
        if (bvh.empty) return;
        const uint8_t *table = TRAVERSAL_TABLE[ray_code(rays.dir_inv_local[rs.next_ray(0)])];
        size_t stack[BVH_MAX_DEPTH * 3 + 2];
        for (auto &v : stack) v = 0;
        long sp = 1;
        while (sp > 0) {
            const Node4 &node = bvh.nodes[stack[sp]];
            if (!node.leaf) {
                cnt.node_tests += rs.next_count();
                uint32_t all_hits = 0;
                rs.pop_do_next_task_and_push_rays(node.child_count, [&](uint16_t ri) -> uint32_t {
                    if (rays.is_done(ri)) return 0;
                    uint32_t h;
                    if (node.nbounds == 1) {
                        h = bbox4_intersect(bvh.bounds[node.bounds0], rays.orig_local[ri], rays.dir_inv_local[ri], rays.max_t[ri]);
                    } else {
                        size_t i; real a2;
                        const BBox4 *bb = &bvh.bounds[node.bounds0];
                        BBox4 b = lerp_slice_index(node.nbounds, rays.time[ri], &i, &a2) ? bb[i] : bbox4_lerp(bb[i], bb[i + 1], a2);
                        h = bbox4_intersect(b, rays.orig_local[ri], rays.dir_inv_local[ri], rays.max_t[ri]);
                    }
                    all_hits |= h;
                    return h;
                });
                if (all_hits) {
                    uint8_t order = table[node.traversal_code];
                    long lane_count = 0;
                    for (int i = (int)node.child_count - 1; i >= 0; i--) {
                        uint32_t ci = (order >> (i * 2)) & 3u;
                        if (rs.push_lane_to_task(ci)) {
                            stack[sp + lane_count] = node.child0 + ci;
                            lane_count++;
                        }
                    }
                    sp += lane_count - 1;
                } else {
                    sp -= 1;
                }
            } else {
                leaf(node.o0, node.o1, rays);
                sp -= 1;
            }
        }
    }

    void mesh_intersect(const Mesh &m, const Closure &shader, int32_t shader_idx, uint32_t inst_id, RayBatch &rays) {
        Xf static_mat = (nspace == 1) ? xf_inverse(space[0]) : xf_identity();
        traverse(m.accel, rays, [&](size_t o0, size_t o1, RayBatch &rays) {
            size_t tri_count = o1 - o0;
            bool cached = rs.next_count() >= tri_count && m.ts == 1 && nspace <= 1;
            V3 cache[3][3];
            if (cached) {
                for (size_t ti = o0; ti < o1; ti++) {
                    const uint32_t *ix = &m.idx[ti * 4];
                    for (int k = 0; k < 3; k++) {
                        V3 p = m.verts[ix[k]];
                        cache[ti - o0][k] = (nspace != 0) ? xf_point(p, static_mat) : p;
                    }
                }
            }
            rs.do_next_task([&](uint16_t ri) {
                if (rays.is_done(ri)) return;
                real rt = rays.time[ri];
                Xf mat = (nspace > 1) ? xf_inverse(lerp_slice_xf(space, nspace, rt)) : static_mat;
                bool hit = false;
                V3 ht[3];
                const uint32_t *hix = nullptr;
                real hd[4] = {0, 0, 0, 0};
                TriPre pre = tri_precompute(rays.dir[ri]);
                for (size_t ti = o0; ti < o1; ti++) {
                    const uint32_t *ix = &m.idx[ti * 4];
                    V3 tri[3];
                    if (cached) {
                        for (int k = 0; k < 3; k++) tri[k] = cache[ti - o0][k];
                    } else {
                        for (int k = 0; k < 3; k++) {
                            tri[k] = (m.ts == 1) ? m.verts[ix[k]] : lerp_slice_v3(&m.verts[(size_t)ix[k] * m.ts], m.ts, rt);
                            if (nspace != 0) tri[k] = xf_point(tri[k], mat);
                        }
                    }
                    real r[4];
                    cnt.tri_tests++;
                    if (tri_intersect(rays.orig[ri], pre, rays.max_t[ri], tri[0], tri[1], tri[2], r)) {
                        if (rays.is_occlusion(ri)) {
                            isects[ri].kind = PSY_HIT_OCCLUDE;
                            rays.mark_done(ri);
                            break;
                        }
                        hit = true;
                        rays.max_t[ri] = r[0];
                        ht[0] = tri[0]; ht[1] = tri[1]; ht[2] = tri[2];
                        hix = ix;
                        std::memcpy(hd, r, sizeof(hd));
                    }
                }
                if (hit) {
                    Isect &is = isects[ri];
                    is.kind = PSY_HIT_SURFACE;
                    is.t = hd[0]; is.b0 = hd[1]; is.b1 = hd[2]; is.b2 = hd[3];
                    is.prim = hix[3];
                    is.inst = inst_id;
                    surface_point(ht[0], ht[1], ht[2], hd[1], hd[2], hd[3], &is.pos, &is.pos_err);
                    V3 geo = cross(ht[0] - ht[1], ht[0] - ht[2]);
                    V3 sn = geo;
                    if (!m.normals.empty()) {
                        V3 n[3];
                        for (int k = 0; k < 3; k++)
                            n[k] = normalized(lerp_slice_v3(&m.normals[(size_t)hix[k] * m.ts], m.ts, rt));
                        V3 snn = xf_normal((n[0] * hd[1]) + (n[1] * hd[2]) + (n[2] * hd[3]), mat);
                        sn = (dot(snn, geo) >= 0.0f) ? snn : neg(snn);
                    }
                    is.incoming = rays.dir[ri];
                    is.nor = sn;
                    is.nor_g = geo;
                    is.sample_pdf = 0.0f;
                    is.closure = shader;
                    is.shader = shader_idx;
                }
            });
            rs.pop_task();
        });
    }

    // RectangleLight::sample_pdf (src/light/rectangle_light.rs:52-96)
    static real rect_sample_pdf(const RectLight &L, const Xf &space_xf, V3 arr, V3 sample_dir, V3 hit, real time) {
        real w = lerp_slice_f_pair(L.dims, 0, time), h = lerp_slice_f_pair(L.dims, 1, time);
        Xf si = xf_inverse(space_xf);
        V3 p1 = xf_point(v3(w * 0.5f, h * 0.5f, 0.0f), si);
        V3 p2 = xf_point(v3(w * -0.5f, h * 0.5f, 0.0f), si);
        V3 p3 = xf_point(v3(w * -0.5f, h * -0.5f, 0.0f), si);
        V3 p4 = xf_point(v3(w * 0.5f, h * -0.5f, 0.0f), si);
        V3 sp1 = normalized(p1 - arr), sp2 = normalized(p2 - arr), sp3 = normalized(p3 - arr), sp4 = normalized(p4 - arr);
        real a1 = spherical_triangle_solid_angle(sp2, sp1, sp3);
        real a2 = spherical_triangle_solid_angle(sp4, sp1, sp3);
        V3 normal = xf_normal(v3(0.0f, 0.0f, 1.0f), si);
        if ((a1 + a2) < 0.01f) {
            real area = triangle_surface_area(p2, p1, p3) + triangle_surface_area(p4, p1, p3);
            return length2(hit - arr) / std::fabs(dot(normalized(sample_dir), normalized(normal))) / area;
        }
        return 1.0f / (a1 + a2);
    }
    static real lerp_slice_f_pair(const std::vector<real> &dims, int c, real time) {
        size_t n = dims.size() / 2;
        size_t i; real a2;
        if (lerp_slice_index(n, time, &i, &a2)) return dims[i * 2 + c];
        return lerpf(dims[i * 2 + c], dims[(i + 1) * 2 + c], a2);
    }

    Xf space_at(real t) const { return nspace ? lerp_slice_xf(space, nspace, t) : xf_identity(); }

    void rect_intersect(const RectLight &L, uint32_t inst_id, RayBatch &rays) {
        rs.pop_do_next_task([&](uint16_t ri) {
            real time = rays.time[ri];
            V3 o = rays.orig[ri], dir = rays.dir[ri];
            real max_t = rays.max_t[ri];
            real w = lerp_slice_f_pair(L.dims, 0, time), h = lerp_slice_f_pair(L.dims, 1, time);
            Xf xf = space_at(time);
            Xf si = xf_inverse(xf);
            V3 p1 = xf_point(v3(w * 0.5f, h * 0.5f, 0.0f), si);
            V3 p2 = xf_point(v3(w * -0.5f, h * 0.5f, 0.0f), si);
            V3 p3 = xf_point(v3(w * -0.5f, h * -0.5f, 0.0f), si);
            V3 p4 = xf_point(v3(w * 0.5f, h * -0.5f, 0.0f), si);
            TriPre pre = tri_precompute(dir);
            V3 tris[2][3] = {{p1, p2, p3}, {p3, p4, p1}};
            for (int k = 0; k < 2; k++) {
                real r[4];
                cnt.tri_tests++;
                if (tri_intersect(o, pre, max_t, tris[k][0], tris[k][1], tris[k][2], r) && r[0] < max_t) {
                    Isect &is = isects[ri];
                    if (rays.is_occlusion(ri)) {
                        is.kind = PSY_HIT_OCCLUDE;
                        rays.mark_done(ri);
                    } else {
                        is.kind = PSY_HIT_LIGHT;
                        is.t = r[0]; is.b0 = r[1]; is.b1 = r[2]; is.b2 = r[3];
                        is.prim = (uint32_t)k;
                        is.inst = inst_id;
                        surface_point(tris[k][0], tris[k][1], tris[k][2], r[1], r[2], r[3], &is.pos, &is.pos_err);
                        V3 nn = cross(tris[k][0] - tris[k][1], tris[k][0] - tris[k][2]);
                        is.incoming = dir;
                        is.nor = nn; is.nor_g = nn;
                        is.sample_pdf = rect_sample_pdf(L, xf, o, dir, is.pos, time);
                        real isa = (real)(1.0 / ((double)w * (double)h));
                        Color col = color_mul(lerp_slice_color(L.colors.data(), L.colors.size(), time), isa);
                        is.closure = Closure{CL_EMIT, col, 0.0f, 0.0f};
                        is.shader = -1;
                        rays.max_t[ri] = r[0];
                    }
                    break;
                }
            }
        });
    }

    // SphereLight::sample_pdf (src/light/sphere_light.rs:51-81)
    static real sphere_sample_pdf(const SphereLight &L, const Xf &space_xf, V3 arr_w, real time) {
        V3 arr = xf_point(arr_w, space_xf);
        double radius = (double)lerp_slice_f(L.radii.data(), L.radii.size(), time);
        double d2 = (double)length2(v3(0, 0, 0) - arr);
        double d = std::sqrt(d2);
        if (d > radius) {
            double st2 = std::fmin((radius * radius) / d2, 1.0);
            double ct2 = 1.0 - st2;
            return (real)uniform_sample_cone_pdf(std::sqrt(ct2));
        }
        return (real)(1.0 / (4.0 * PI_64));
    }

    void sphere_intersect(const SphereLight &L, uint32_t inst_id, RayBatch &rays) {
        rs.pop_do_next_task([&](uint16_t ri) {
            real time = rays.time[ri];
            Xf xf = space_at(time);
            real radius = lerp_slice_f(L.radii.data(), L.radii.size(), time);
            V3 o = rays.orig_local[ri];
            V3 dir = xf_vector(rays.dir[ri], xf);
            real a = length2(dir);
            real b = 2.0f * dot(dir, o);
            real c = length2(o) - (radius * radius);
            real disc = (b * b) - (4.0f * a * c);
            if (disc < 0.0f) return;
            disc = std::sqrt(disc);
            real q = (b < 0.0f) ? -0.5f * (b - disc) : -0.5f * (b + disc);
            real t0 = q / a;
            real t1 = (q != 0.0f) ? c / q : rays.max_t[ri];
            if (t0 > t1) std::swap(t0, t1);
            if (t0 > rays.max_t[ri] || t1 <= 0.0f) return;
            real t;
            if (t0 > 0.0f) t = t0;
            else if (t1 <= rays.max_t[ri]) t = t1;
            else return;
            Isect &is = isects[ri];
            if (rays.is_occlusion(ri)) {
                is.kind = PSY_HIT_OCCLUDE;
                rays.mark_done(ri);
                return;
            }
            Xf ixf = xf_inverse(xf);
            V3 tpos = o + (dir * t);
            V3 unit = normalized(tpos);
            is.kind = PSY_HIT_LIGHT;
            is.t = t; is.b0 = is.b1 = is.b2 = 0.0f;
            is.prim = 0;
            is.inst = inst_id;
            is.pos = xf_vector(unit * radius, ixf);  // the reference applies the vector transform here
            is.pos_err = 0.001f;
            V3 nrm = xf_normal(unit, ixf);
            is.incoming = rays.dir[ri];
            is.nor = nrm; is.nor_g = nrm;
            is.sample_pdf = sphere_sample_pdf(L, xf, rays.orig[ri], time);
            real isa = (real)(1.0 / (4.0 * PI_64 * (double)radius * (double)radius));
            is.closure = Closure{CL_EMIT, color_mul(lerp_slice_color(L.colors.data(), L.colors.size(), time), isa), 0.0f, 0.0f};
            is.shader = -1;
            rays.max_t[ri] = t;
        });
    }

    // TracerInner::trace_assembly (src/tracer.rs:87-150), root assembly only
    void trace_assembly(RayBatch &rays) {
        traverse(s.object_accel, rays, [&](size_t o0, size_t, RayBatch &rays) {
            const Instance &inst = s.instances[o0];
            bool has_xf = inst.xc != 0;
            if (has_xf) {
                space = &s.xforms[inst.xs];
                nspace = inst.xc;
                rs.do_next_task([&](uint16_t ri) { rays.update_local(ri, lerp_slice_xf(space, nspace, rays.time[ri])); });
                rs.duplicate_next_task();
            }
            const Object &ob = s.objects[inst.object];
            if (ob.kind == PSY_OBJ_MESH) {
                Closure sh = inst.shader >= 0 ? s.shaders[inst.shader] : unassigned_closure();
                mesh_intersect(s.meshes[ob.index], sh, inst.shader, inst.id, rays);
            } else if (ob.kind == PSY_OBJ_RECT_LIGHT) {
                rect_intersect(s.rects[ob.index], inst.id, rays);
            } else {
                sphere_intersect(s.spheres[ob.index], inst.id, rays);
            }
            if (has_xf) {
                space = nullptr;
                nspace = 0;
                Xf ident = xf_identity();
                rs.pop_do_next_task([&](uint16_t ri) { rays.update_local(ri, ident); });
            }
        });
    }

    // TracerInner::trace (src/tracer.rs:51-85)
    void trace(RayBatch &rays) {
        rs.clear();
        isects.assign(rays.size(), Isect{});
        for (auto &is : isects) is.kind = PSY_HIT_MISS;
        Xf ident = xf_identity();
        for (size_t i = 0; i < rays.size(); i++) rays.update_local(i, ident);
        rs.ensure_lanes(8);
        for (size_t i = 0; i < rays.size(); i++) rs.lanes[ray_code(rays.dir[i])].push((uint16_t)i);
        for (uint32_t l = 0; l < 8; l++) rs.push_lane_to_task(l);
        while (!rs.empty()) trace_assembly(rays);
    }
};

}  // namespace


// ======================================================================= light sampling
namespace {

// LightTree::select (src/accel/light_tree.rs:135-201)
static bool lt_select(const PsyoScene &s, V3 inc, V3 pos, V3 nor, V3 nor_g, const Closure &sc, real time, real n,
                      size_t *light_index, real *pdf, real *whittled) {
    if (s.lt_empty) return false;
    auto node_prob = [&](const LightTreeNode &nd) {
        BBox bb = lerp_slice_bbox(nd.bounds.data(), nd.bounds.size(), time);
        V3 dd = bcenter(bb) - pos;
        real r2 = diagonal2(bb) * 0.25f;
        real inv_sa = 1.0f / r2;
        real contrib = closure_estimate_sphere(sc, inc, dd, r2, nor, nor_g);
        return nd.energy * inv_sa * contrib;
    };
    const LightTreeNode *node = &s.lt[0];
    real tot = 1.0f;
    while (!node->leaf) {
        real ps[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        real total = 0.0f;
        for (size_t i = 0; i < node->nchild; i++) {
            real p = node_prob(s.lt[node->child0 + i]);
            ps[i] = p;
            total += p;
        }
        if (total <= 0.0f) {
            real p = 1.0f / (real)node->nchild;
            for (int i = 0; i < 8; i++) ps[i] = p;
        } else {
            for (int i = 0; i < 8; i++) ps[i] /= total;
        }
        real base = 0.0f;
        for (size_t i = 0; i < 8; i++) {
            real p = ps[i];
            if ((n <= base + p) || (i == node->nchild - 1)) {
                tot *= p;
                node = &s.lt[node->child0 + i];
                n = (n - base) / p;
                break;
            }
            base += p;
        }
    }
    *light_index = node->light_index;
    *pdf = tot;
    *whittled = n;
    return true;
}

// RectangleLight::sample_from_point (src/light/rectangle_light.rs:121-243)
static V4 rect_sample(const RectLight &L, const Xf &space, V3 arr, real u, real v, real wl, real time, V3 *sp,
                      V3 *sn, real *serr, real *pdf) {
    real w = Tracer::lerp_slice_f_pair(L.dims, 0, time), h = Tracer::lerp_slice_f_pair(L.dims, 1, time);
    Color col = lerp_slice_color(L.colors.data(), L.colors.size(), time);
    double sa = (double)w * (double)h;
    double sai = 1.0 / sa;
    Xf si = xf_inverse(space);
    V3 p1 = xf_point(v3(w * 0.5f, h * 0.5f, 0.0f), si);
    V3 p2 = xf_point(v3(w * -0.5f, h * 0.5f, 0.0f), si);
    V3 p3 = xf_point(v3(w * -0.5f, h * -0.5f, 0.0f), si);
    V3 p4 = xf_point(v3(w * 0.5f, h * -0.5f, 0.0f), si);
    V3 lp1 = p1 - arr, lp2 = p2 - arr, lp3 = p3 - arr, lp4 = p4 - arr;
    V3 sp1 = normalized(lp1), sp2 = normalized(lp2), sp3 = normalized(lp3), sp4 = normalized(lp4);
    real a1 = spherical_triangle_solid_angle(sp2, sp1, sp3);
    real a2 = spherical_triangle_solid_angle(sp4, sp1, sp3);
    V3 normal = xf_normal(v3(0.0f, 0.0f, 1.0f), si);
    if ((a1 + a2) < 0.01f) {
        real sa1 = triangle_surface_area(p2, p1, p3);
        real sa2 = triangle_surface_area(p4, p1, p3);
        real th = sa1 / (sa1 + sa2);
        V3 spt = (u < th) ? uniform_sample_triangle(p2, p1, p3, v, u / th)
                          : uniform_sample_triangle(p4, p1, p3, v, (u - th) / (1.0f - th));
        V3 shadow_vec = spt - arr;
        V4 ss = color_to_spectral(col, wl) * (real)sai * 0.5f;
        *pdf = length2(spt - arr) / std::fabs(dot(normalized(shadow_vec), normalized(normal))) / (sa1 + sa2);
        *sp = spt; *sn = normal; *serr = 0.0001f;
        return ss;
    }
    real prob_1 = std::isinf(a1) ? 1.0f : (std::isinf(a2) ? 0.0f : a1 / (a1 + a2));
    real prob_2 = 1.0f - prob_1;
    V3 shadow_vec = (u < prob_1) ? uniform_sample_spherical_triangle(sp2, sp1, sp3, v, u / prob_1)
                                 : uniform_sample_spherical_triangle(sp4, sp1, sp3, v, 1.0f - ((u - prob_1) / prob_2));
    V3 arr_local = xf_point(arr, space);
    V3 svl = xf_vector(shadow_vec, space);
    svl = svl * (-arr_local.z / svl.z);
    V3 spl = arr_local + svl;
    spl.x = rmin(rmax(spl.x, w * -0.5f), w * 0.5f);
    spl.y = rmin(rmax(spl.y, h * -0.5f), h * 0.5f);
    spl.z = 0.0f;
    *sp = xf_point(spl, si);
    *sn = normal;
    *serr = 0.0001f;
    *pdf = 1.0f / (a1 + a2);
    return color_to_spectral(col, wl) * (real)sai * 0.5f;
}

// SphereLight::sample_from_point (src/light/sphere_light.rs:85-192)
static V4 sphere_sample(const SphereLight &L, const Xf &space, V3 arr_w, real u, real v, real wl, real time, V3 *sp,
                        V3 *sn, real *serr, real *pdf) {
    V3 arr = xf_point(arr_w, space);
    V3 pos = v3(0, 0, 0);
    Xf inv = xf_inverse(space);
    double radius = (double)lerp_slice_f(L.radii.data(), L.radii.size(), time);
    Color col = lerp_slice_color(L.colors.data(), L.colors.size(), time);
    double sai = 1.0 / (4.0 * PI_64 * radius * radius);
    V3 zv = pos - arr;
    double d2 = (double)length2(zv);
    double d = std::sqrt(d2);
    V3 z, x, y;
    coordinate_system_from_vector(zv, &z, &x, &y);
    x = normalized(x); y = normalized(y); z = normalized(z);
    real rf = (real)radius;
    real err = length(xf_vector(v3(rf, rf, rf), inv)) * 0.001f;
    if (d > radius) {
        double st2 = std::fmin((radius * radius) / d2, 1.0);
        double ct2 = 1.0 - st2;
        double st = std::sqrt(st2);
        double ct = std::sqrt(ct2);
        V3 smp = normalized(uniform_sample_cone(u, v, ct));
        double cos_theta = (double)smp.z;
        double cos_theta2 = cos_theta * cos_theta;
        double sin_theta2 = std::fmax(1.0 - cos_theta2, 0.0);
        double sin_theta = std::sqrt(sin_theta2);
        double dd = 1.0 - (d2 * sin_theta * sin_theta / (radius * radius));
        double cos_a = (dd <= 0.0) ? st : ((d / radius) * sin_theta2) + (cos_theta * std::sqrt(dd));
        double sin_a = std::sqrt(std::fmax(1.0 - (cos_a * cos_a), 0.0));
        double phi = (double)v * 2.0 * PI_64;
        V3 s2 = v3((real)(std::cos(phi) * sin_a * radius), (real)(std::sin(phi) * sin_a * radius), (real)(d - (cos_a * radius)));
        V3 svec = (x * s2.x) + (y * s2.y) + (z * s2.z);
        V3 normal = normalized(arr + svec);
        V3 point = normal * rf;
        *sp = xf_point(point, inv);
        *sn = xf_normal(normal, inv);
        *serr = err;
        *pdf = (real)uniform_sample_cone_pdf(ct);
        return color_to_spectral(col, wl) * (real)sai;
    }
    V3 svec = uniform_sample_sphere(u, v);
    V3 normal = normalized(arr + svec);
    V3 point = normal * rf;
    *sp = xf_point(point, inv);
    *sn = xf_normal(normal, inv);
    *serr = err;
    *pdf = (real)(1.0 / (4.0 * PI_64));
    return color_to_spectral(col, wl) * (real)sai;
}

enum { LS_NONE = 0, LS_DISTANT = 1, LS_SURFACE = 2 };
struct LightSample {
    int kind;
    V4 color;
    V3 dir;            // distant
    V3 sp, sn;         // surface
    real serr;
    real pdf, sel_pdf;
};

static real distant_energy(const DistantLight &l) {
    real a = 0.0f;
    for (auto &c : l.colors) a = a + color_energy(c);
    return a / (real)l.colors.size();
}

// Scene::sample_lights (src/scene/mod.rs:28-99) + Assembly::sample_lights
// (src/scene/assembly.rs:46-140) for the root assembly.
static LightSample scene_sample_lights(const PsyoScene &s, real n, real u, real v, real w, real wl, real time,
                                       const Isect &is) {
    LightSample out{};
    out.kind = LS_NONE;
    real wle = 0.0f;
    for (auto &l : s.distant) wle = wle + distant_energy(l);
    real wl_energy = (wle <= 0.0f) ? 0.0f : 1.0f;
    real ll_energy = (s.lt_empty || s.lt[0].energy <= 0.0f) ? 0.0f : 1.0f;
    real tot = wl_energy + ll_energy;
    if (tot <= 0.0f) return out;
    real wl_prob = wl_energy / tot;
    if (n < wl_prob) {
        real nn = n / wl_prob;
        real total = 0.0f;
        for (auto &l : s.distant) total = total + distant_energy(l);
        real target = nn * total;
        real x = 0.0f;
        size_t pick = s.distant.size() - 1;
        real p = 0.0f;
        for (size_t i = 0; i < s.distant.size(); i++) {
            real wgt = distant_energy(s.distant[i]);
            x += wgt;
            if (x > target) { pick = i; p = wgt / total; break; }
            if (i == s.distant.size() - 1) p = wgt / total;
        }
        const DistantLight &L = s.distant[pick];
        double radius = (double)lerp_slice_f(L.radii.data(), L.radii.size(), time);
        V3 direction = lerp_slice_v3(L.dirs.data(), L.dirs.size(), time);
        Color col = lerp_slice_color(L.colors.data(), L.colors.size(), time);
        double sai = 1.0 / (2.0 * PI_64 * (1.0 - std::cos(radius)));
        V3 z, x3, y3;
        coordinate_system_from_vector(neg(normalized(direction)), &z, &x3, &y3);
        double ctm = std::cos(radius);
        V3 smp = normalized(uniform_sample_cone(u, v, ctm));
        out.kind = LS_DISTANT;
        out.color = color_to_spectral(col, wl) * (real)sai;
        out.dir = (x3 * smp.x) + (y3 * smp.y) + (z * smp.z);
        out.pdf = (real)uniform_sample_cone_pdf(ctm);
        out.sel_pdf = p * wl_prob;
        return out;
    }
    real nl = (n - wl_prob) / (1.0f - wl_prob);
    if (is.kind != PSY_HIT_SURFACE && is.kind != PSY_HIT_LIGHT) return out;
    Xf ident = xf_identity();
    size_t li;
    real sel_pdf, whittled;
    if (!lt_select(s, xf_vector(is.incoming, ident), xf_point(is.pos, ident), xf_normal(is.nor, ident),
                   xf_normal(is.nor_g, ident), is.closure, time, nl, &li, &sel_pdf, &whittled))
        return out;
    const Instance &inst = s.light_instances[li];
    Xf xf = inst.xc ? lerp_slice_xf(&s.xforms[inst.xs], inst.xc, time) : xf_identity();
    const Object &ob = s.objects[inst.object];
    V4 col;
    real pdf;
    if (ob.kind == PSY_OBJ_RECT_LIGHT) col = rect_sample(s.rects[ob.index], xf, is.pos, u, v, wl, time, &out.sp, &out.sn, &out.serr, &pdf);
    else col = sphere_sample(s.spheres[ob.index], xf, is.pos, u, v, wl, time, &out.sp, &out.sn, &out.serr, &pdf);
    out.kind = LS_SURFACE;
    out.color = col;
    out.pdf = pdf;
    out.sel_pdf = sel_pdf * (1.0f - wl_prob);
    return out;
}

// ======================================================================= light path
// src/renderer.rs:362-692
enum { EV_CAMERA = 0, EV_BOUNCE = 1, EV_SHADOW = 2 };
struct LightPath {
    int event;
    uint32_t bounce_count;
    uint32_t sampling_seed;
    uint32_t px, py;
    uint32_t sample_number;
    uint32_t dim_offset;
    real time, wavelength;
    bool has_next_bounce;
    V3 nb_orig, nb_dir;
    V4 next_attenuation_fac;
    real closure_sample_pdf;
    V4 light_attenuation, pending_color_addition, color;
    uint32_t rays;  // rays traced (statistics only)
};

static void camera_generate_ray(const PsyoScene &s, real x, real y, real time, real u, real v, V3 *o, V3 *d) {
    Xf xf = lerp_slice_xf(s.cam_xf.data(), s.cam_xf.size(), time);
    real tfov = lerp_slice_f(s.cam_tfov.data(), s.cam_tfov.size(), time);
    real ar = lerp_slice_f(s.cam_ap.data(), s.cam_ap.size(), time);
    real fd = lerp_slice_f(s.cam_fd.data(), s.cam_fd.size(), time);
    real cu, cv;
    square_to_circle((u * 2.0f) - 1.0f, (v * 2.0f) - 1.0f, &cu, &cv);
    V3 orig = v3(ar * cu, ar * cv, 0.0f);
    V3 dir = normalized(v3((x * tfov) - (orig.x / fd), (y * tfov) - (orig.y / fd), 1.0f));
    *o = xf_point(orig, xf);
    *d = xf_vector(dir, xf);
}

static void next_lds(LightPath &p, float out[4]) {
    uint32_t dim = p.dim_offset;
    p.dim_offset += 1;
    get_sample_4d(p.sample_number, dim, p.px, p.py, p.sampling_seed, out);
}

static bool path_next(LightPath &p, const PsyoScene &s, const Isect &is, RayBatch &rays, size_t ri) {
    if (p.event == EV_CAMERA || p.event == EV_BOUNCE) {
        if (is.kind == PSY_HIT_SURFACE || is.kind == PSY_HIT_LIGHT) {
            const Closure &cl = is.closure;
            if (cl.kind == CL_EMIT) {
                V4 c = color_to_spectral(cl.color, p.wavelength);
                if (p.event == EV_CAMERA) {
                    p.color = p.color + c;
                } else {
                    real mis = power_heuristic(p.closure_sample_pdf, is.sample_pdf);
                    p.color = p.color + c * p.light_attenuation / splat4(mis);
                }
                return false;
            }
            p.light_attenuation = p.light_attenuation / splat4(p.closure_sample_pdf);
            p.dim_offset = 0;
            p.sampling_seed += 1;
            float smp[4];
            next_lds(p, smp);
            LightSample li = scene_sample_lights(s, smp[0], smp[1], smp[2], smp[3], p.wavelength, p.time, is);
            bool found = false;
            if (li.kind != LS_NONE && !(li.pdf <= 0.0f) && !(li.sel_pdf <= 0.0f)) {
                V4 att;
                real cpdf;
                V3 so, sd;
                real smax;
                if (li.kind == LS_DISTANT) {
                    att = closure_evaluate(cl, rays.dir[ri], li.dir, is.nor, is.nor_g, p.wavelength, &cpdf);
                    so = robust_ray_origin(is.pos, is.pos_err, normalized(is.nor_g), li.dir);
                    sd = li.dir;
                    smax = INFINITY;
                } else {
                    V3 dir = li.sp - is.pos;
                    att = closure_evaluate(cl, rays.dir[ri], dir, is.nor, is.nor_g, p.wavelength, &cpdf);
                    so = robust_ray_origin(is.pos, is.pos_err, normalized(is.nor_g), dir);
                    V3 oe = robust_ray_origin(li.sp, li.serr, normalized(li.sn), neg(dir));
                    sd = oe - so;
                    smax = 1.0f;
                }
                if (!(max_elem4(att) <= 0.0f)) {
                    real lmis = power_heuristic(li.pdf, cpdf);
                    p.pending_color_addition = li.color * att * p.light_attenuation / splat4(lmis * li.sel_pdf);
                    rays.set_from_ray(ri, so, sd, smax, p.time, p.wavelength, true);
                    found = true;
                }
            }
            bool do_bounce = false;
            if (p.bounce_count < s.max_bounces) {
                p.bounce_count += 1;
                p.dim_offset = 0;
                p.sampling_seed += 1;
                float b4[4];
                next_lds(p, b4);
                V3 dir;
                real pdf;
                V4 filt = closure_sample(cl, is.incoming, is.nor, is.nor_g, b4[0], b4[1], p.wavelength, &dir, &pdf);
                if ((pdf > 0.0f) && (max_elem4(filt) > 0.0f)) {
                    p.next_attenuation_fac = filt;
                    p.closure_sample_pdf = pdf;
                    p.nb_orig = robust_ray_origin(is.pos, is.pos_err, normalized(is.nor_g), dir);
                    p.nb_dir = dir;
                    p.has_next_bounce = true;
                    do_bounce = true;
                }
            } else {
                p.has_next_bounce = false;
            }
            if (found) {
                p.event = EV_SHADOW;
                return true;
            }
            if (do_bounce) {
                rays.set_from_ray(ri, p.nb_orig, p.nb_dir, INFINITY, p.time, p.wavelength, false);
                p.event = EV_BOUNCE;
                p.light_attenuation = p.light_attenuation * p.next_attenuation_fac;
                return true;
            }
            return false;
        }
        V4 bg = color_to_spectral(s.background, p.wavelength);
        p.color = p.color + bg * p.light_attenuation / splat4(p.closure_sample_pdf);
        return false;
    }
    // shadow ray result
    if (is.kind == PSY_HIT_MISS) p.color = p.color + p.pending_color_addition;
    if (p.has_next_bounce) {
        rays.set_from_ray(ri, p.nb_orig, p.nb_dir, INFINITY, p.time, p.wavelength, false);
        p.light_attenuation = p.light_attenuation * p.next_attenuation_fac;
        p.event = EV_BOUNCE;
        return true;
    }
    return false;
}

struct BucketJob {
    uint32_t x, y, w, h;
};

struct Worker {
    const PsyoScene &s;
    Tracer tracer;
    RayBatch rays;
    std::vector<LightPath> paths;
    PsyRenderStats st{};
    explicit Worker(const PsyoScene &sc) : s(sc), tracer(sc) {}

    // ray generation of render_job (src/renderer.rs:241-275)
    void gen(const BucketJob &b, uint32_t spp, uint32_t seed) {
        paths.clear();
        rays.clear();
        real cmpx = 1.0f / (real)s.width, cmpy = 1.0f / (real)s.height;
        real min_x = -1.0f, max_x = 1.0f;
        real min_y = -((real)s.height / (real)s.width), max_y = (real)s.height / (real)s.width;
        real xe = max_x - min_x, ye = max_y - min_y;
        for (uint32_t y = b.y; y < b.y + b.h; y++)
            for (uint32_t x = b.x; x < b.x + b.w; x++)
                for (uint32_t si = 0; si < spp; si++) {
                    float d[4], d4[4];
                    get_sample_4d(si, 0, x, y, seed, d);
                    get_sample_4d(si, 1, x, y, seed, d4);
                    real fx = probit(d[3], 2.0f / 6.0f) + 0.5f;
                    real fy = probit(d4[0], 2.0f / 6.0f) + 0.5f;
                    real sx = (fx + (real)x) * cmpx;
                    real sy = (fy + (real)y) * cmpy;
                    real ix = (sx - 0.5f) * xe, iy = (0.5f - sy) * ye;
                    real wl = map_0_1_to_wavelength(golden_ratio_sample(si, hash_u32((x << 16) ^ y, seed)));
                    LightPath p{};
                    p.event = EV_CAMERA;
                    p.sampling_seed = seed ^ 0x40d4682bu;
                    p.px = x; p.py = y;
                    p.sample_number = si;
                    p.time = d[0];
                    p.wavelength = wl;
                    p.next_attenuation_fac = splat4(1.0f);
                    p.closure_sample_pdf = 1.0f;
                    p.light_attenuation = splat4(1.0f);
                    p.pending_color_addition = splat4(0.0f);
                    p.color = splat4(0.0f);
                    V3 o, dd;
                    camera_generate_ray(s, ix, iy, d[0], d[1], d[2], &o, &dd);
                    paths.push_back(p);
                    rays.push(o, dd, INFINITY, d[0], wl, false);
                }
    }
    // trace/compact loop (src/renderer.rs:279-297)
    void run() {
        size_t pi = paths.size();
        while (pi > 0) {
            auto t0 = std::chrono::steady_clock::now();
            tracer.trace(rays);
            st.ray_count += rays.size();
            auto t1 = std::chrono::steady_clock::now();
            size_t ne = 0;
            for (size_t i = 0; i < pi; i++) {
                paths[i].rays++;
                if (path_next(paths[i], s, tracer.isects[i], rays, i)) {
                    std::swap(paths[ne], paths[i]);
                    rays.swap(ne, i);
                    ne++;
                }
            }
            rays.truncate(ne);
            pi = ne;
            auto t2 = std::chrono::steady_clock::now();
            st.trace_time += std::chrono::duration<double>(t1 - t0).count();
            st.ray_generation_time += std::chrono::duration<double>(t2 - t1).count();
        }
    }
};

}  // namespace

// ======================================================================= C API
extern "C" int psyo_trace(PsyoScene *s, const PsyRay *rays, uint32_t n, PsyHit *hits, PsySurfaceHit *full,
                          uint64_t *node_tests, uint64_t *tri_tests, uint32_t nthreads) {
    if (!s || (!rays && n) || (!hits && n)) return PSY_E_INVALID;
    if (nthreads == 0) nthreads = 1;
    const uint32_t B = 65536;
    uint32_t nb = (n + B - 1) / B;
    std::atomic<uint32_t> next{0};
    std::atomic<uint64_t> nt{0}, tt{0};
    auto work = [&]() {
        Tracer tr(*s);
        RayBatch rb;
        while (true) {
            uint32_t bi = next.fetch_add(1);
            if (bi >= nb) break;
            uint32_t a = bi * B, e = std::min(n, a + B);
            rb.clear();
            for (uint32_t i = a; i < e; i++) {
                const PsyRay &r = rays[i];
                rb.push(v3(r.orig[0], r.orig[1], r.orig[2]), v3(r.dir[0], r.dir[1], r.dir[2]), r.max_t, r.time, r.wavelength,
                        (r.flags & PSY_RAY_OCCLUSION) != 0);
            }
            tr.trace(rb);
            for (uint32_t i = a; i < e; i++) {
                const Isect &is = tr.isects[i - a];
                PsyHit h{};
                h.kind = is.kind;
                if (is.kind == PSY_HIT_SURFACE || is.kind == PSY_HIT_LIGHT) {
                    h.prim = is.prim; h.inst = is.inst; h.t = is.t; h.b0 = is.b0; h.b1 = is.b1; h.b2 = is.b2;
                }
                hits[i] = h;
                if (full) {
                    PsySurfaceHit f{};
                    f.hit = h;
                    if (is.kind == PSY_HIT_SURFACE || is.kind == PSY_HIT_LIGHT) {
                        f.pos[0] = is.pos.x; f.pos[1] = is.pos.y; f.pos[2] = is.pos.z;
                        f.pos_err = is.pos_err;
                        f.nor[0] = is.nor.x; f.nor[1] = is.nor.y; f.nor[2] = is.nor.z;
                        f.nor_g[0] = is.nor_g.x; f.nor_g[1] = is.nor_g.y; f.nor_g[2] = is.nor_g.z;
                        f.sample_pdf = is.sample_pdf;
                        f.shader = is.shader;
                    } else {
                        f.shader = -1;
                    }
                    full[i] = f;
                }
            }
        }
        nt += tr.cnt.node_tests;
        tt += tr.cnt.tri_tests;
    };
    std::vector<std::thread> th;
    for (uint32_t t = 1; t < nthreads; t++) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
    if (node_tests) *node_tests = nt;
    if (tri_tests) *tri_tests = tt;
    return PSY_OK;
}

static void hilbert_rot(uint32_t n, uint32_t rx, uint32_t ry, uint32_t *x, uint32_t *y) {
    if (ry == 0) {
        if (rx == 1) { *x = (n - 1) - *x; *y = (n - 1) - *y; }
        std::swap(*x, *y);
    }
}
extern "C" void psyo_hilbert_d2xy(uint32_t d, uint32_t *ox, uint32_t *oy) {
    // src/hilbert.rs:47-63
    uint32_t x = 0, y = 0, t = d;
    for (uint32_t s = 1; s < (1u << 16); s <<= 1) {
        uint32_t rx = 1 & (t >> 1);
        uint32_t ry = 1 & (t ^ rx);
        hilbert_rot(s, rx, ry, &x, &y);
        x += s * rx;
        y += s * ry;
        t >>= 2;
    }
    *ox = x; *oy = y;
}
extern "C" uint32_t psyo_hilbert_xy2d(uint32_t x, uint32_t y) {
    uint32_t d = 0;
    for (uint32_t s = (1u << 16) >> 1; s > 0; s >>= 1) {
        uint32_t rx = (x & s) > 0 ? 1 : 0;
        uint32_t ry = (y & s) > 0 ? 1 : 0;
        d += s * s * ((3 * rx) ^ ry);
        hilbert_rot(s, rx, ry, &x, &y);
    }
    return d;
}

// Renderer::render (src/renderer.rs:76-191)
extern "C" int psyo_render(PsyoScene *s, uint32_t spb, uint32_t nthreads, const uint32_t *crop, uint32_t max_buckets,
                           float *xyz, PsyRenderStats *stats) {
    return psyo_render_sampled(s, spb, nthreads, crop, 1, max_buckets, xyz, stats);
}

extern "C" int psyo_render_sampled(PsyoScene *s, uint32_t spb, uint32_t nthreads, const uint32_t *crop,
                                   uint32_t bucket_stride, uint32_t max_buckets, float *xyz, PsyRenderStats *stats) {
    if (!s || !xyz) return PSY_E_INVALID;
    if (nthreads == 0) nthreads = 1;
    if (spb == 0) spb = 4096;
    size_t W = s->width, H = s->height;
    size_t width = W, height = H, sx = 0, sy = 0;
    if (crop) {
        size_t x1 = std::min<size_t>(crop[0], W - 1), y1 = std::min<size_t>(crop[1], H - 1);
        size_t x2 = std::min<size_t>(crop[2], W - 1), y2 = std::min<size_t>(crop[3], H - 1);
        width = x2 - x1 + 1; height = y2 - y1 + 1; sx = x1; sy = y1;
    }
    double tpp = (double)spb / (double)s->spp;
    size_t bd = std::sqrt(tpp) < 1.0 ? 1 : (size_t)std::sqrt(tpp);
    uint32_t bcx = (uint32_t)(width / bd + 1), bcy = (uint32_t)(height / bd + 1);
    uint32_t larger = std::max(bcx, bcy);
    uint32_t pow2 = 1;
    while (pow2 < larger) pow2 <<= 1;
    uint64_t bucket_n = (uint64_t)pow2 * pow2;
    std::vector<BucketJob> jobs;
    for (uint64_t hd = 0; hd < bucket_n; hd++) {
        uint32_t bx, by;
        psyo_hilbert_d2xy((uint32_t)hd, &bx, &by);
        size_t x = (size_t)bx * bd, y = (size_t)by * bd;
        size_t w = (width >= x) ? std::min(bd, width - x) : bd;
        size_t h = (height >= y) ? std::min(bd, height - y) : bd;
        if (x < width && y < height && w > 0 && h > 0)
            jobs.push_back(BucketJob{(uint32_t)(sx + x), (uint32_t)(sy + y), (uint32_t)w, (uint32_t)h});
    }
    if (bucket_stride > 1) {
        std::vector<BucketJob> kept;
        for (size_t j = 0; j < jobs.size(); j += bucket_stride) kept.push_back(jobs[j]);
        jobs.swap(kept);
    }
    if (max_buckets && jobs.size() > max_buckets) jobs.resize(max_buckets);
    std::memset(xyz, 0, sizeof(float) * W * H * 3);
    // accumulate in the arithmetic type (f64 in the FP64 oracle), store f32
    std::vector<real> acc(W * H * 3, (real)0);
    std::atomic<size_t> next{0};
    std::mutex mu;
    PsyRenderStats tot{};
    auto t_start = std::chrono::steady_clock::now();
    auto work = [&]() {
        Worker wk(*s);
        auto t0 = std::chrono::steady_clock::now();
        while (true) {
            size_t j = next.fetch_add(1);
            if (j >= jobs.size()) break;
            const BucketJob &b = jobs[j];
            auto g0 = std::chrono::steady_clock::now();
            wk.gen(b, s->spp, s->seed);
            auto g1 = std::chrono::steady_clock::now();
            wk.st.initial_ray_generation_time += std::chrono::duration<double>(g1 - g0).count();
            wk.st.samples += wk.paths.size();
            wk.run();
            auto a0 = std::chrono::steady_clock::now();
            real inv = (real)s->spp;
            for (auto &p : wk.paths) {
                V3 c = xyz_from_spectral(p.color, p.wavelength);
                real *px = acc.data() + ((size_t)p.py * W + p.px) * 3;
                px[0] += c.x / inv; px[1] += c.y / inv; px[2] += c.z / inv;
            }
            auto a1 = std::chrono::steady_clock::now();
            wk.st.sample_writing_time += std::chrono::duration<double>(a1 - a0).count();
        }
        wk.st.total_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        wk.st.accel_node_visits = wk.tracer.cnt.node_tests;
        std::lock_guard<std::mutex> g(mu);
        tot.trace_time += wk.st.trace_time;
        tot.initial_ray_generation_time += wk.st.initial_ray_generation_time;
        tot.ray_generation_time += wk.st.ray_generation_time;
        tot.sample_writing_time += wk.st.sample_writing_time;
        tot.ray_count += wk.st.ray_count;
        tot.accel_node_visits += wk.st.accel_node_visits;
        tot.samples += wk.st.samples;
    };
    std::vector<std::thread> th;
    for (uint32_t t = 1; t < nthreads; t++) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
    for (size_t i = 0; i < W * H * 3; i++) xyz[i] = (float)acc[i];
    tot.total_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    if (stats) *stats = tot;
    return PSY_OK;
}

extern "C" int psyo_render_paths(PsyoScene *s, const PsyBucket *b, float *color4, float *wavelength, uint32_t *rays_per_sample) {
    if (!s || !b || !color4) return PSY_E_INVALID;
    if ((uint64_t)b->w * b->h * s->spp > 65536) return PSY_E_INVALID;
    Worker wk(*s);
    wk.gen(BucketJob{b->x, b->y, b->w, b->h}, s->spp, s->seed);
    wk.run();
    for (auto &p : wk.paths) {
        size_t i = ((size_t)(p.py - b->y) * b->w + (p.px - b->x)) * s->spp + p.sample_number;
        for (int k = 0; k < 4; k++) color4[i * 4 + k] = p.color[k];
        if (wavelength) wavelength[i] = p.wavelength;
        if (rays_per_sample) rays_per_sample[i] = p.rays;
    }
    return PSY_OK;
}

// Shape of the scene's light tree: node count, leaf count and depth (levels
// of nodes from the root to the deepest leaf; 0 for an empty tree).
extern "C" int psyo_light_tree_info(PsyoScene *s, uint32_t *nodes, uint32_t *leaves, uint32_t *depth) {
    if (!s) return PSY_E_INVALID;
    uint32_t nl = 0, dmax = 0;
    if (!s->lt_empty) {
        std::vector<std::pair<size_t, uint32_t>> st{{0, 1}};
        while (!st.empty()) {
            auto [n, d] = st.back();
            st.pop_back();
            dmax = std::max(dmax, d);
            const LightTreeNode &ln = s->lt[n];
            if (ln.leaf) { nl++; continue; }
            for (size_t c = 0; c < ln.nchild; c++) st.push_back({ln.child0 + c, d + 1});
        }
    }
    if (nodes) *nodes = s->lt_empty ? 0u : (uint32_t)s->lt.size();
    if (leaves) *leaves = nl;
    if (depth) *depth = dmax;
    return PSY_OK;
}

extern "C" int psyo_mesh_bvh_info(PsyoScene *s, uint32_t object, uint32_t *tri_order, uint32_t *node_count) {
    if (!s || object >= s->objects.size() || s->objects[object].kind != PSY_OBJ_MESH) return PSY_E_INVALID;
    const Mesh &m = s->meshes[s->objects[object].index];
    if (tri_order)
        for (size_t i = 0; i < m.idx.size() / 4; i++) tri_order[i] = m.idx[i * 4 + 3];
    if (node_count) *node_count = (uint32_t)m.accel.nodes.size();
    return PSY_OK;
}

// ----------------------------------------------------------------------- KAT helpers
extern "C" uint32_t psyo_hash_u32(uint32_t n, uint32_t seed) { return hash_u32(n, seed); }
extern "C" uint64_t psyo_hash_u64(uint64_t n, uint64_t seed) { return hash_u64(n, seed); }
extern "C" float psyo_hash_u32_to_f32(uint32_t n, uint32_t seed) { return hash_u32_to_f32(n, seed); }
extern "C" void psyo_get_sample_4d(uint32_t i, uint32_t set, uint32_t px, uint32_t py, uint32_t seed, float *out4) {
    get_sample_4d(i, set, px, py, seed, out4);
}
extern "C" float psyo_golden_ratio_sample(uint32_t i, uint32_t scramble) { return golden_ratio_sample(i, scramble); }
// The 4 wavelengths render_job gives sample si of pixel (x, y)
// (src/renderer.rs:261-265 with src/color.rs:20-43).
extern "C" void psyo_wavelengths(uint32_t si, uint32_t x, uint32_t y, uint32_t seed, float *out4) {
    float hero = (float)map_0_1_to_wavelength(golden_ratio_sample(si, hash_u32((x << 16) ^ y, seed)));
    for (int k = 0; k < 4; k++) out4[k] = (float)nth_wavelength(hero, k);
}
extern "C" float psyo_probit(float n, float width) { return probit(n, width); }
extern "C" float psyo_fast_exp(float p) { return fast_exp(p); }
extern "C" void psyo_traversal_table(uint8_t *out) { std::memcpy(out, TRAVERSAL_TABLE, sizeof(TRAVERSAL_TABLE)); }
#ifndef PSYO_F64  // f32 known-answer hooks (the FP64 oracle exports renders only)
extern "C" void psyo_xf_mul(const float *a, const float *b, float *out) {
    Xf x, y;
    std::memcpy(x.m, a, 48); std::memcpy(y.m, b, 48);
    Xf r = xf_mul(x, y);
    std::memcpy(out, r.m, 48);
}
extern "C" void psyo_xf_inverse(const float *a, float *out) {
    Xf x;
    std::memcpy(x.m, a, 48);
    Xf r = xf_inverse(x);
    std::memcpy(out, r.m, 48);
}
extern "C" void psyo_xf_lerp(const float *a, const float *b, float alpha, float *out) {
    Xf x, y;
    std::memcpy(x.m, a, 48); std::memcpy(y.m, b, 48);
    Xf r = xf_lerp(x, y, alpha);
    std::memcpy(out, r.m, 48);
}
extern "C" void psyo_xf_point(const float *m, const float *p, float *out) {
    Xf x;
    std::memcpy(x.m, m, 48);
    V3 r = xf_point(v3(p[0], p[1], p[2]), x);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
extern "C" void psyo_xf_vector(const float *m, const float *v, float *out) {
    Xf x;
    std::memcpy(x.m, m, 48);
    V3 r = xf_vector(v3(v[0], v[1], v[2]), x);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
extern "C" void psyo_lerp3(const float *a, const float *b, float alpha, float *out) {
    V3 r = lerp3(v3(a[0], a[1], a[2]), v3(b[0], b[1], b[2]), alpha);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
extern "C" float psyo_lerp(float a, float b, float alpha) { return lerpf(a, b, alpha); }
extern "C" void psyo_xf_normal(const float *m, const float *n, float *out) {
    Xf x;
    std::memcpy(x.m, m, 48);
    V3 r = xf_normal(v3(n[0], n[1], n[2]), x);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
extern "C" float psyo_lerp_slice(const float *s, uint32_t n, float alpha) { return lerp_slice_f(s, n, alpha); }
#endif
extern "C" void psyo_xyz_to_spectrum(const float *xyz, float hero, float *out4) {
    V4 r = color_to_spectral(Color{COL_XYZ, xyz[0], xyz[1], xyz[2]}, hero);
    for (int k = 0; k < 4; k++) out4[k] = r[k];
}
extern "C" void psyo_spectrum_to_xyz(const float *e4, float hero, float *xyz) {
    V3 r = xyz_from_spectral(v4(e4[0], e4[1], e4[2], e4[3]), hero);
    xyz[0] = r.x; xyz[1] = r.y; xyz[2] = r.z;
}

// sub_crates/color/build.rs: RGB->XYZ matrix from chromaticities (ACES CTL
// RGBtoXYZ), printed with 10 decimals into the generated Rust source and
// therefore rounded to 10 decimals before becoming f32 constants.
static void rgb_to_xyz_matrix(double rx, double ry, double gx, double gy, double bx, double by, double wx, double wy, float out[9]) {
    double Y = 1.0;
    double X = wx * Y / wy;
    double Z = (1.0 - wx - wy) * Y / wy;
    double d = rx * (by - gy) + bx * (gy - ry) + gx * (ry - by);
    double sr = (X * (by - gy) - gx * (Y * (by - 1.0) + by * (X + Z)) + bx * (Y * (gy - 1.0) + gy * (X + Z))) / d;
    double sg = (X * (ry - by) + rx * (Y * (by - 1.0) + by * (X + Z)) - bx * (Y * (ry - 1.0) + ry * (X + Z))) / d;
    double sb = (X * (gy - ry) - rx * (Y * (gy - 1.0) + gy * (X + Z)) + gx * (Y * (ry - 1.0) + ry * (X + Z))) / d;
    double m[9] = {sr * rx, sg * gx, sb * bx, sr * ry, sg * gy, sb * by, sr * (1.0 - rx - ry), sg * (1.0 - gx - gy), sb * (1.0 - bx - by)};
    for (int i = 0; i < 9; i++) {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.10f", m[i]);
        out[i] = std::strtof(buf, nullptr);
    }
}
static void apply3(const float m[9], const float *rgb, float *xyz) {
    for (int r = 0; r < 3; r++) xyz[r] = ((rgb[0] * m[r * 3]) + (rgb[1] * m[r * 3 + 1])) + (rgb[2] * m[r * 3 + 2]);
}
extern "C" void psyo_rec709_e_to_xyz(const float *rgb, float *xyz) {
    float m[9];
    rgb_to_xyz_matrix(0.640, 0.330, 0.300, 0.600, 0.150, 0.060, 1.0 / 3.0, 1.0 / 3.0, m);
    apply3(m, rgb, xyz);
}
extern "C" void psyo_rec709_to_xyz(const float *rgb, float *xyz) {
    float m[9];
    rgb_to_xyz_matrix(0.640, 0.330, 0.300, 0.600, 0.150, 0.060, 0.3127, 0.3290, m);
    apply3(m, rgb, xyz);
}
// Image::write_png's pixel conversion (src/image.rs:138-164, 275-305) with
// the xyz_to_rec709_e matrix of sub_crates/color/build.rs:162-188 (inverse of
// the equal-energy rec709 matrix by Gauss-Jordan elimination with partial
// pivoting, :246-323, in f64, printed with 10 decimals).
static void xyz_to_rec709_e_m(float out[9]) {
    const double rx = 0.640, ry = 0.330, gx = 0.300, gy = 0.600, bx = 0.150, by = 0.060;
    const double wx = 1.0 / 3.0, wy = 1.0 / 3.0, Y = 1.0;
    double X = wx * Y / wy, Z = (1.0 - wx - wy) * Y / wy;
    double d = rx * (by - gy) + bx * (gy - ry) + gx * (ry - by);
    double sr = (X * (by - gy) - gx * (Y * (by - 1.0) + by * (X + Z)) + bx * (Y * (gy - 1.0) + gy * (X + Z))) / d;
    double sg = (X * (ry - by) + rx * (Y * (by - 1.0) + by * (X + Z)) - bx * (Y * (ry - 1.0) + ry * (X + Z))) / d;
    double sb = (X * (gy - ry) - rx * (Y * (gy - 1.0) + gy * (X + Z)) + gx * (Y * (ry - 1.0) + ry * (X + Z))) / d;
    double a[3][3] = {{sr * rx, sg * gx, sb * bx}, {sr * ry, sg * gy, sb * by},
                      {sr * (1.0 - rx - ry), sg * (1.0 - gx - gy), sb * (1.0 - bx - by)}};
    double inv[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 2; i++) {  // forward elimination, largest pivot
        int p = i;
        double best = std::fabs(a[i][i]);
        for (int j = i + 1; j < 3; j++)
            if (std::fabs(a[j][i]) > best) { best = std::fabs(a[j][i]); p = j; }
        if (p != i)
            for (int k = 0; k < 3; k++) { std::swap(a[i][k], a[p][k]); std::swap(inv[i][k], inv[p][k]); }
        for (int j = i + 1; j < 3; j++) {
            double f = a[j][i] / a[i][i];
            for (int k = 0; k < 3; k++) { a[j][k] -= f * a[i][k]; inv[j][k] -= f * inv[i][k]; }
        }
    }
    for (int i = 2; i >= 0; i--) {  // back substitution
        double f = a[i][i];
        for (int k = 0; k < 3; k++) { a[i][k] /= f; inv[i][k] /= f; }
        for (int j = 0; j < i; j++) {
            double g = a[j][i];
            for (int k = 0; k < 3; k++) { a[j][k] -= g * a[i][k]; inv[j][k] -= g * inv[i][k]; }
        }
    }
    for (int i = 0; i < 9; i++) {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.10f", inv[i / 3][i % 3]);
        out[i] = std::strtof(buf, nullptr);
    }
}
extern "C" void psyo_xyz_to_srgb8(const float *xyz, uint32_t w, uint32_t h, uint8_t *rgba) {
    float m[9];
    xyz_to_rec709_e_m(m);
    auto gamma = [](float n) { return n < 0.0031308f ? n * 12.92f : (1.055f * std::pow(n, 1.0f / 2.4f)) - 0.055f; };
    auto q = [](float n) {
        float v = std::fmin(1.0f, std::fmax(0.0f, n)) * 255.0f;
        return (uint8_t)v;
    };
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            float rgb[3];
            apply3(m, xyz + ((size_t)(h - 1 - y) * w + x) * 3, rgb);
            uint8_t *o = rgba + ((size_t)y * w + x) * 4;
            o[0] = q(gamma(rgb[0])); o[1] = q(gamma(rgb[1])); o[2] = q(gamma(rgb[2])); o[3] = 255;
        }
}
#ifndef PSYO_F64
extern "C" int psyo_intersect_triangle(const float *o, const float *d, float max_t, const float *p0, const float *p1,
                                       const float *p2, float *out) {
    TriPre pre = tri_precompute(v3(d[0], d[1], d[2]));
    return tri_intersect(v3(o[0], o[1], o[2]), pre, max_t, v3(p0[0], p0[1], p0[2]), v3(p1[0], p1[1], p1[2]),
                         v3(p2[0], p2[1], p2[2]), out)
               ? 1
               : 0;
}
#endif
extern "C" uint32_t psyo_quick_select_ints(int32_t *list, uint32_t n, uint32_t place) {
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; i++) idx[i] = i;
    std::vector<int32_t> vals(list, list + n);
    Splitter<int>::quick_select(idx.data(), n, place, [&](uint32_t a, uint32_t b) { return vals[a] < vals[b]; });
    for (uint32_t i = 0; i < n; i++) list[i] = vals[idx[i]];
    return (uint32_t)list[place];
}
extern "C" int psyo_increment_ulp_check(void) {
    // src/fp_utils.rs:84-131 known answers
    int ok = 1;
    ok &= increment_ulp(1.0f) > 1.0f;
    ok &= increment_ulp(-1.0f) > -1.0f;
    ok &= decrement_ulp(1.0f) < 1.0f;
    ok &= decrement_ulp(-1.0f) < -1.0f;
    ok &= increment_ulp(0.0f) > 0.0f && increment_ulp(-0.0f) > 0.0f;
    ok &= decrement_ulp(0.0f) < 0.0f && decrement_ulp(-0.0f) < 0.0f;
    ok &= decrement_ulp(increment_ulp(1.2f)) == 1.2f && increment_ulp(decrement_ulp(-1.2f)) == -1.2f;
    return ok;
}
