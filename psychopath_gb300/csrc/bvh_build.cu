// GPU build of a static triangle mesh's BVH4 (an LBVH): Morton codes of the
// triangle centroids, a stable LSD radix sort, the binary radix tree of the
// sorted codes (Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees", HPG 2012), bottom-up bounds, then a top-down
// collapse into the BVH4 node layout the traversal reads (psy_layout.h).
//
// The tree differs from the SAH tree of the reference's build
// (src/accel/bvh_base.rs), so ray hits agree with it except for exact ties
// between primitives; its purpose is scene creation time.  Nodes follow the
// same conventions as the host collapse: children in binary-tree order, the
// traversal code from the split axes of the node and its expanded children,
// leaves of up to three triangles.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "bvh_build.h"
#include "radix_sort.h"

namespace {

constexpr uint32_t kLeafBit = 0x80000000u;  // binary child reference: sorted primitive index

__device__ __forceinline__ uint32_t ordered_bits(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered(uint32_t b) {
    return __uint_as_float((b & 0x80000000u) ? (b & 0x7FFFFFFFu) : ~b);
}
__device__ __forceinline__ uint32_t expand10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Triangle bounds and centroids (original triangle order); the centroid box
// is reduced into gbox (6 ordered-bit words: min xyz, max xyz).
__global__ void k_prep(const float4 *__restrict__ verts, uint32_t vbase, const uint32_t *__restrict__ idx, uint32_t n,
                       float4 *__restrict__ bmin, float4 *__restrict__ bmax, float4 *__restrict__ cent,
                       uint32_t *gbox) {
    __shared__ uint32_t sb[6];
    if (threadIdx.x < 6) sb[threadIdx.x] = threadIdx.x < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        float4 a = verts[vbase + idx[3 * t]], b = verts[vbase + idx[3 * t + 1]], c = verts[vbase + idx[3 * t + 2]];
        float4 lo = make_float4(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)), 0.0f);
        float4 hi = make_float4(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)), 0.0f);
        bmin[t] = lo;
        bmax[t] = hi;
        float4 ce = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.0f);
        cent[t] = ce;
        atomicMin(&sb[0], ordered_bits(ce.x)); atomicMin(&sb[1], ordered_bits(ce.y)); atomicMin(&sb[2], ordered_bits(ce.z));
        atomicMax(&sb[3], ordered_bits(ce.x)); atomicMax(&sb[4], ordered_bits(ce.y)); atomicMax(&sb[5], ordered_bits(ce.z));
    }
    __syncthreads();
    if (threadIdx.x < 3) atomicMin(&gbox[threadIdx.x], sb[threadIdx.x]);
    else if (threadIdx.x < 6) atomicMax(&gbox[threadIdx.x], sb[threadIdx.x]);
}

// 30-bit Morton code (x in bits 3k+2, y in 3k+1, z in 3k) of the centroid in
// the centroid box.
__global__ void k_morton(const float4 *__restrict__ cent, uint32_t n, const uint32_t *gbox, uint32_t *keys,
                         uint32_t *vals) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float lo[3], ext[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = from_ordered(gbox[a]);
        ext[a] = from_ordered(gbox[3 + a]) - lo[a];
    }
    float4 c = cent[t];
    float v[3] = {c.x, c.y, c.z};
    uint32_t q[3];
    for (int a = 0; a < 3; a++) {
        float u = ext[a] > 0.0f ? (v[a] - lo[a]) / ext[a] : 0.0f;
        q[a] = (uint32_t)fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);  // NaN -> 0
    }
    keys[t] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
    vals[t] = t;
}

// ---------------------------------------------------------------- radix tree
__device__ __forceinline__ int common_prefix(const uint32_t *keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = keys[i], b = keys[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);  // equal codes: the index breaks the tie
    return __clz(a ^ b);
}
// Internal node i of the n - 1: its range [first, last] and children
// (kLeafBit | sorted index for single primitives).
__global__ void k_radix_tree(const uint32_t *__restrict__ keys, int n, uint32_t *left, uint32_t *right,
                             uint32_t *first, uint32_t *last, uint32_t *parent, uint32_t *leaf_parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (common_prefix(keys, n, i, i + 1) - common_prefix(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = common_prefix(keys, n, i, i - d);
    int lmax = 2;
    while (common_prefix(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (common_prefix(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = common_prefix(keys, n, i, j);
    int s = 0;
    for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
        if (common_prefix(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    int split = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    uint32_t lc = (lo == split) ? (kLeafBit | (uint32_t)split) : (uint32_t)split;
    uint32_t rc = (hi == split + 1) ? (kLeafBit | (uint32_t)(split + 1)) : (uint32_t)(split + 1);
    left[i] = lc;
    right[i] = rc;
    first[i] = (uint32_t)lo;
    last[i] = (uint32_t)hi;
    if (lc & kLeafBit) leaf_parent[lc & ~kLeafBit] = (uint32_t)i; else parent[lc] = (uint32_t)i;
    if (rc & kLeafBit) leaf_parent[rc & ~kLeafBit] = (uint32_t)i; else parent[rc] = (uint32_t)i;
}
// Bounds of the internal nodes, bottom-up: the second child to arrive at a
// node computes its union (flag counts arrivals).
__global__ void k_tree_bounds(const uint32_t *__restrict__ vals, int n, const float4 *__restrict__ tmin,
                              const float4 *__restrict__ tmax, const uint32_t *__restrict__ left,
                              const uint32_t *__restrict__ right, const uint32_t *__restrict__ parent,
                              const uint32_t *__restrict__ leaf_parent, uint32_t *flag, float4 *nmin, float4 *nmax) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n || n < 2) return;
    uint32_t node = leaf_parent[j];
    while (true) {
        __threadfence();
        if (atomicAdd(&flag[node], 1u) == 0) return;  // first arrival: the sibling finishes the node
        __threadfence();
        float4 lo[2], hi[2];
        uint32_t ch[2] = {left[node], right[node]};
        for (int c = 0; c < 2; c++) {
            if (ch[c] & kLeafBit) {
                uint32_t t = vals[ch[c] & ~kLeafBit];
                lo[c] = tmin[t];
                hi[c] = tmax[t];
            } else {
                lo[c] = __ldcg(&nmin[ch[c]]);
                hi[c] = __ldcg(&nmax[ch[c]]);
            }
        }
        __stcg(&nmin[node], make_float4(fminf(lo[0].x, lo[1].x), fminf(lo[0].y, lo[1].y), fminf(lo[0].z, lo[1].z), 0.0f));
        __stcg(&nmax[node], make_float4(fmaxf(hi[0].x, hi[1].x), fmaxf(hi[0].y, hi[1].y), fmaxf(hi[0].z, hi[1].z), 0.0f));
        if (node == 0) return;
        node = parent[node];
    }
}

// ---------------------------------------------------------------- collapse into BVH4 nodes
struct TreeView {
    const uint32_t *keys, *vals, *left, *right, *first, *last;
    const float4 *tmin, *tmax, *nmin, *nmax;
};
__device__ __forceinline__ uint32_t prim_count(const TreeView &T, uint32_t c) {
    return (c & kLeafBit) ? 1u : T.last[c] - T.first[c] + 1u;
}
__device__ __forceinline__ uint32_t prim_first(const TreeView &T, uint32_t c) {
    return (c & kLeafBit) ? (c & ~kLeafBit) : T.first[c];
}
// Split axis of an internal node: the axis of the highest bit in which its
// first and last codes differ (0 when all codes are equal).
__device__ __forceinline__ uint32_t split_axis(const TreeView &T, uint32_t c) {
    uint32_t diff = T.keys[T.first[c]] ^ T.keys[T.last[c]];
    if (diff == 0) return 0;
    uint32_t p = 31u - __clz(diff);
    uint32_t m = p % 3u;
    return m == 2u ? 0u : (m == 1u ? 1u : 2u);
}
__device__ __forceinline__ void child_box(const TreeView &T, uint32_t c, float4 &lo, float4 &hi) {
    if (c & kLeafBit) {
        uint32_t t = T.vals[c & ~kLeafBit];
        lo = T.tmin[t];
        hi = T.tmax[t];
    } else {
        lo = T.nmin[c];
        hi = T.nmax[c];
    }
}
// One frontier entry per BVH4 node to write: binary node b (more than three
// primitives) at output slot slot[k].  Children with at most three
// primitives become leaves; larger ones get a slot and join the next
// frontier.
__global__ void k_collapse(TreeView T, const uint32_t *__restrict__ front, const uint32_t *__restrict__ slots,
                           uint32_t nfront, uint32_t node_base, uint32_t tri_base, GNode *out, uint32_t *next,
                           uint32_t *next_slots, uint32_t *counters /* [0] next frontier size, [1] slots used, [2] disorder */) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nfront) return;
    uint32_t b = front[k], me = slots[k];
    uint32_t l = T.left[b], r = T.right[b];
    bool le = !(l & kLeafBit) && prim_count(T, l) > 3u;
    bool re = !(r & kLeafBit) && prim_count(T, r) > 3u;
    uint32_t ch[4], cc, code, ab = split_axis(T, b);
    if (le && re) {
        cc = 4; ch[0] = T.left[l]; ch[1] = T.right[l]; ch[2] = T.left[r]; ch[3] = T.right[r];
        code = ab + split_axis(T, l) * 3u + split_axis(T, r) * 9u;
    } else if (le) {
        cc = 3; ch[0] = T.left[l]; ch[1] = T.right[l]; ch[2] = r;
        code = ab + split_axis(T, l) * 3u + 27u;
    } else if (re) {
        cc = 3; ch[0] = l; ch[1] = T.left[r]; ch[2] = T.right[r];
        code = ab + split_axis(T, r) * 3u + 36u;
    } else {
        cc = 2; ch[0] = l; ch[1] = r;
        code = ab + 45u;
    }
    float lo[3][4], hi[3][4];
    uint32_t refs[4] = {0, 0, 0, 0};
    bool ordered = true;
    for (uint32_t i = 0; i < 4; i++) {
        if (i >= cc) {
            for (int a = 0; a < 3; a++) { lo[a][i] = INFINITY; hi[a][i] = -INFINITY; }
            continue;
        }
        uint32_t c = ch[i];
        float4 blo, bhi;
        child_box(T, c, blo, bhi);
        lo[0][i] = blo.x; lo[1][i] = blo.y; lo[2][i] = blo.z;
        hi[0][i] = bhi.x; hi[1][i] = bhi.y; hi[2][i] = bhi.z;
        for (int a = 0; a < 3; a++) ordered = ordered && (lo[a][i] <= hi[a][i]);
        uint32_t cnt = prim_count(T, c);
        if ((c & kLeafBit) || cnt <= 3u) {
            refs[i] = psy_make_leaf(tri_base + prim_first(T, c), cnt);
        } else {
            uint32_t s = atomicAdd(&counters[1], 1u);
            uint32_t q = atomicAdd(&counters[0], 1u);
            next[q] = c;
            next_slots[q] = s;
            refs[i] = node_base + s;
        }
    }
    if (!ordered) atomicOr(&counters[2], 1u);
    GNode g;
    g.xlo = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
    g.xhi = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
    g.ylo = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
    g.yhi = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
    g.zlo = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
    g.zhi = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
    g.child = make_uint4(refs[0], refs[1], refs[2], refs[3]);
    g.meta = make_uint4(0u, 1u, code | (cc << 8), 0u);
    out[me] = g;
}

struct DevBuf {
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T *get(size_t count) {
        void *p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (err == cudaSuccess) ptrs.push_back(p);
        return static_cast<T *>(p);
    }
    ~DevBuf() {
        for (void *p : ptrs) cudaFree(p);
    }
};

}  // namespace

cudaError_t lbvh_build_mesh(const LbvhInput &in, LbvhOutput &out, cudaStream_t st) {
    const uint32_t n = in.ntris;
    out = LbvhOutput{};
    DevBuf B;
    float4 *verts = B.get<float4>(in.num_verts);
    uint32_t *idx = B.get<uint32_t>(3 * (size_t)n);
    float4 *tmin = B.get<float4>(n), *tmax = B.get<float4>(n), *cent = B.get<float4>(n);
    uint32_t *gbox = B.get<uint32_t>(8), *keys = B.get<uint32_t>(n), *vals = B.get<uint32_t>(n);
    uint32_t *keys2 = B.get<uint32_t>(n), *vals2 = B.get<uint32_t>(n);
    uint32_t *sort_scratch = B.get<uint32_t>(radix_sort_scratch_words(n));
    size_t ni = n > 1 ? n - 1 : 1;
    uint32_t *left = B.get<uint32_t>(ni), *right = B.get<uint32_t>(ni), *first = B.get<uint32_t>(ni);
    uint32_t *last = B.get<uint32_t>(ni), *parent = B.get<uint32_t>(ni), *lparent = B.get<uint32_t>(n);
    uint32_t *flag = B.get<uint32_t>(ni);
    float4 *nmin = B.get<float4>(ni), *nmax = B.get<float4>(ni);
    uint32_t *front = B.get<uint32_t>(ni), *fslots = B.get<uint32_t>(ni);
    uint32_t *next = B.get<uint32_t>(ni), *nslots = B.get<uint32_t>(ni), *counters = B.get<uint32_t>(4);
    GNode *nodes = B.get<GNode>(ni);
    if (B.err != cudaSuccess) return B.err;
    std::vector<float4> hv(in.num_verts);
    for (uint32_t v = 0; v < in.num_verts; v++)
        hv[v] = make_float4(in.verts[3 * v], in.verts[3 * v + 1], in.verts[3 * v + 2], 0.0f);
    cudaError_t e = cudaMemcpyAsync(verts, hv.data(), hv.size() * sizeof(float4), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(idx, in.indices, 3 * (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    uint32_t box0[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpyAsync(gbox, box0, sizeof(box0), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    uint32_t g = (n + 255) / 256;
    k_prep<<<g, 256, 0, st>>>(verts, 0, idx, n, tmin, tmax, cent, gbox);
    k_morton<<<g, 256, 0, st>>>(cent, n, gbox, keys, vals);
    uint32_t *ka = nullptr, *va = nullptr;  // 30-bit Morton codes
    if ((e = radix_sort_pairs(keys, vals, keys2, vals2, sort_scratch, n, 30, &ka, &va, st)) != cudaSuccess) return e;
    out.order.resize(n);
    if ((e = cudaMemcpyAsync(out.order.data(), va, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    if (n <= 3) {  // the whole mesh is one leaf
        out.root = psy_make_leaf(in.tri_base, n);
        out.depth = 0;
        return cudaStreamSynchronize(st);
    }
    int gi = (int)((ni + 255) / 256);
    k_radix_tree<<<gi, 256, 0, st>>>(ka, (int)n, left, right, first, last, parent, lparent);
    if ((e = cudaMemsetAsync(flag, 0, ni * sizeof(uint32_t), st)) != cudaSuccess) return e;
    k_tree_bounds<<<g, 256, 0, st>>>(va, (int)n, tmin, tmax, left, right, parent, lparent, flag, nmin, nmax);
    TreeView T{ka, va, left, right, first, last, tmin, tmax, nmin, nmax};
    // frontier waves: the root (binary node 0) is BVH4 slot 0
    uint32_t zero = 0, init[4] = {0u, 1u, 0u, 0u};
    if ((e = cudaMemcpyAsync(front, &zero, 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(fslots, &zero, 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(counters, init, sizeof(init), cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    uint32_t nfront = 1, depth = 0, host_ctr[4];
    while (nfront > 0) {
        depth++;
        if ((e = cudaMemsetAsync(counters, 0, 4, st)) != cudaSuccess) return e;  // next frontier size
        k_collapse<<<(nfront + 127) / 128, 128, 0, st>>>(T, front, fslots, nfront, in.node_base, in.tri_base, nodes,
                                                         next, nslots, counters);
        if ((e = cudaMemcpyAsync(host_ctr, counters, sizeof(host_ctr), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        nfront = host_ctr[0];
        std::swap(front, next);
        std::swap(fslots, nslots);
    }
    out.root = in.node_base;  // slot 0
    out.node_count = host_ctr[1];
    out.depth = depth;
    out.ordered = host_ctr[2] == 0;
    out.nodes.resize(out.node_count);
    e = cudaMemcpyAsync(out.nodes.data(), nodes, out.node_count * sizeof(GNode), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}
