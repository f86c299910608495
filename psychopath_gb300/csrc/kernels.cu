// Kernels of the GB300 tracing path: ray tracing (closest / any hit),
// camera ray generation, the light-path state machine and accumulation.
#include <cuda_fp16.h>

#include <algorithm>

#include "dev_trace.cuh"
#include "kernels.cuh"

using namespace psyd;

// ------------------------------------------------------------------ constants
// Sobol direction numbers: dimension 1 is van der Corput, dimensions 2..8
// follow Joe & Kuo's primitive polynomials and initial direction numbers.
static void sobol_dirs_host(uint32_t d[8][32]) {
    static const uint32_t s_[7] = {1, 2, 3, 3, 4, 4, 5};
    static const uint32_t a_[7] = {0, 1, 1, 2, 1, 4, 2};
    static const uint32_t m_[7][5] = {{1}, {1, 3}, {1, 3, 1}, {1, 1, 1}, {1, 1, 3, 3}, {1, 3, 5, 13}, {1, 1, 5, 5, 17}};
    for (int k = 0; k < 32; k++) d[0][k] = 1u << (31 - k);
    for (int j = 1; j < 8; j++) {
        uint32_t s = s_[j - 1], a = a_[j - 1];
        for (uint32_t k = 0; k < 32; k++) {
            if (k < s) {
                d[j][k] = m_[j - 1][k] << (31 - k);
            } else {
                uint32_t x = d[j][k - s] ^ (d[j][k - s] >> s);
                for (uint32_t i = 1; i < s; i++)
                    if ((a >> (s - 1 - i)) & 1u) x ^= d[j][k - i];
                d[j][k] = x;
            }
        }
    }
}
// Child visit order per ray octant and node topology (sub_crates/bvh_order).
static void traversal_table_host(uint8_t t[8][48]) {
    for (int rd = 0; rd < 8; rd++) {
        int ray[3] = {rd & 1, (rd >> 1) & 1, (rd >> 2) & 1};
        int k = 0;
        auto sw = [](int &a, int &b) { int x = a; a = b; b = x; };
        for (int s2 = 0; s2 < 3; s2++)
            for (int s1 = 0; s1 < 3; s1++)
                for (int s0 = 0; s0 < 3; s0++) {
                    int p[4] = {0, 1, 2, 3};
                    if (ray[s1]) sw(p[0], p[1]);
                    if (ray[s2]) sw(p[2], p[3]);
                    if (ray[s0]) { sw(p[0], p[2]); sw(p[1], p[3]); }
                    t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2) | (p[2] << 4) | (p[3] << 6));
                }
        for (int s1 = 0; s1 < 3; s1++)
            for (int s0 = 0; s0 < 3; s0++) {
                int p[3] = {0, 1, 2};
                if (ray[s1]) sw(p[0], p[1]);
                if (ray[s0]) { sw(p[0], p[1]); sw(p[0], p[2]); }
                t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2) | (p[2] << 4));
            }
        for (int s1 = 0; s1 < 3; s1++)
            for (int s0 = 0; s0 < 3; s0++) {
                int p[3] = {0, 1, 2};
                if (ray[s1]) sw(p[1], p[2]);
                if (ray[s0]) { sw(p[0], p[2]); sw(p[0], p[1]); }
                t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2) | (p[2] << 4));
            }
        for (int s0 = 0; s0 < 3; s0++) {
            int p[2] = {0, 1};
            if (ray[s0]) sw(p[0], p[1]);
            t[rd][k++] = (uint8_t)(p[0] | (p[1] << 2));
        }
    }
}
void psy_upload_constants() {
    uint32_t d[8][32];
    uint8_t t[8][48];
    sobol_dirs_host(d);
    traversal_table_host(t);
    cudaMemcpyToSymbol(c_sobol_dirs, d, sizeof(d));
    cudaMemcpyToSymbol(c_traversal_table, t, sizeof(t));
}

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
__constant__ GColor c_magenta;

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
        Xf si = xf_inverse(xf);
        V3 p1, p2, p3, p4;
        rect_corners(w, hh, si, &p1, &p2, &p3, &p4);
        V3 a = h.prim == 0 ? p1 : p3, b = h.prim == 0 ? p2 : p4, c = h.prim == 0 ? p3 : p1;
        surface_point(a, b, c, h.b0, h.b1, h.b2, &sd.pos, &sd.pos_err);
        V3 nn = cross(a - b, a - c);
        sd.nor = nn;
        sd.nor_g = nn;
        sd.sample_pdf = rect_sample_pdf<R>(S, L, xf, o, d, sd.pos, time);
        float isa = (float)(1.0 / ((double)w * (double)hh));
        sd.closure.color = color_mul(col, isa);
    } else {
        float radius = light_dim(S, L, 0, time);
        Xf ixf = xf_inverse(xf);
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

// ------------------------------------------------------------------ ray tracing
template <int STACK, bool COUNT>
__global__ void __launch_bounds__(128) k_trace_rays(GScene S, const PsyRay *__restrict__ rays, uint32_t n,
                                                    PsyHit *__restrict__ hits, PsySurfaceHit *__restrict__ full,
                                                    int *err, unsigned long long *counters) {
    __shared__ uint8_t table[8 * 48];
    load_traversal_table(table);
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    TraceCount tc{0, 0};
    if (i < n) {
        const float *r = reinterpret_cast<const float *>(rays + i);
        V3 o = v3(r[0], r[1], r[2]), d = v3(r[3], r[4], r[5]);
        float tmax = r[6], time = r[7];
        uint32_t flags = reinterpret_cast<const uint32_t *>(r)[9];
        HitRec h;
        if (!trace_ray<STACK, COUNT>(S, table, o, d, tmax, time, (flags & PSY_RAY_OCCLUSION) != 0, h, &tc)) {
            atomicExch(err, PSY_E_OVERFLOW);
            h.kind = PSY_HIT_MISS_K;
        }
        PsyHit out;
        out.kind = h.kind;
        out.prim = 0; out.inst = 0; out.t = 0.0f; out.b0 = 0.0f; out.b1 = 0.0f; out.b2 = 0.0f; out.pad = 0.0f;
        if (h.kind == PSY_HIT_SURFACE_K || h.kind == PSY_HIT_LIGHT_K) {
            GInstance in = S.instances[h.slot];
            out.prim = h.kind == PSY_HIT_SURFACE_K ? __ldg(S.tri_idx + h.prim).w : h.prim;
            out.inst = in.id;
            out.t = h.t; out.b0 = h.b0; out.b1 = h.b1; out.b2 = h.b2;
        }
        hits[i] = out;
        if (full) {
            PsySurfaceHit f;
            f.hit = out;
            f.shader = -1;
            f.pos[0] = f.pos[1] = f.pos[2] = 0.0f;
            f.nor[0] = f.nor[1] = f.nor[2] = 0.0f;
            f.nor_g[0] = f.nor_g[1] = f.nor_g[2] = 0.0f;
            f.pos_err = 0.0f;
            f.sample_pdf = 0.0f;
            if (h.kind == PSY_HIT_SURFACE_K || h.kind == PSY_HIT_LIGHT_K) {
                SurfData sd;
                resolve_hit<double>(S, h, o, d, time, sd);
                f.pos[0] = sd.pos.x; f.pos[1] = sd.pos.y; f.pos[2] = sd.pos.z;
                f.nor[0] = sd.nor.x; f.nor[1] = sd.nor.y; f.nor[2] = sd.nor.z;
                f.nor_g[0] = sd.nor_g.x; f.nor_g[1] = sd.nor_g.y; f.nor_g[2] = sd.nor_g.z;
                f.pos_err = sd.pos_err;
                f.sample_pdf = sd.sample_pdf;
                f.shader = sd.shader;
            }
            full[i] = f;
        }
    }
    if (COUNT) {
        unsigned long long a = tc.nodes, b = tc.tris, c = (i < n) ? 1ull : 0ull;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, off);
            b += __shfl_down_sync(0xffffffffu, b, off);
            c += __shfl_down_sync(0xffffffffu, c, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(counters, a);
            atomicAdd(counters + 1, b);
            atomicAdd(counters + 2, c);
        }
    }
}

cudaError_t launch_trace_rays(const GScene &S, const PsyRay *rays, uint32_t n, PsyHit *hits, PsySurfaceHit *full,
                              int stack, int block, int *d_err, unsigned long long *counters, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    (void)block;
    dim3 b(128), g((n + 127) / 128);
    bool c = counters != nullptr;
#define TR(SZ)                                                                                        \
    if (c) k_trace_rays<SZ, true><<<g, b, 0, st>>>(S, rays, n, hits, full, d_err, counters);         \
    else k_trace_rays<SZ, false><<<g, b, 0, st>>>(S, rays, n, hits, full, d_err, counters)
    if (stack <= 32) { TR(32); }
    else if (stack <= 64) { TR(64); }
    else { TR(192); }
#undef TR
    return cudaGetLastError();
}

// ------------------------------------------------------------------ persistent traversal
// Ray sources / sinks of the persistent traversal kernel.
struct IOQueue {  // wavefront: rays of the paths listed in queue[0 .. *count)
    const uint32_t *queue;
    const uint32_t *count;
    const float4 *ro, *rd;
    const uint8_t *occl;
    uint4 *ki;
    float4 *tb;
    __device__ __forceinline__ uint32_t n() const { return *count; }
    __device__ __forceinline__ uint32_t load(uint32_t q, V3 &o, V3 &d, float &tmax, float &time, bool &oc) const {
        uint32_t p = queue[q];
        float4 a = ro[p], b = rd[p];
        o = v3(a); d = v3(b); tmax = a.w; time = b.w; oc = occl[p] != 0;
        return p;
    }
    __device__ __forceinline__ void store(const GScene &, uint32_t p, const HitRec &h) const {
        ki[p] = make_uint4(h.kind, h.prim, h.slot, 0u);
        tb[p] = make_float4(h.t, h.b0, h.b1, h.b2);
    }
};
struct IORays {  // PsyRay records in, PsyHit records out
    const PsyRay *rays;
    uint32_t count;
    PsyHit *hits;
    __device__ __forceinline__ uint32_t n() const { return count; }
    __device__ __forceinline__ uint32_t load(uint32_t q, V3 &o, V3 &d, float &tmax, float &time, bool &oc) const {
        const float *r = reinterpret_cast<const float *>(rays + q);
        o = v3(r[0], r[1], r[2]); d = v3(r[3], r[4], r[5]); tmax = r[6]; time = r[7];
        oc = (reinterpret_cast<const uint32_t *>(r)[9] & PSY_RAY_OCCLUSION) != 0;
        return q;
    }
    __device__ __forceinline__ void store(const GScene &S, uint32_t q, const HitRec &h) const {
        PsyHit out;
        out.kind = h.kind;
        out.prim = 0; out.inst = 0; out.t = 0.0f; out.b0 = 0.0f; out.b1 = 0.0f; out.b2 = 0.0f; out.pad = 0.0f;
        if (h.kind == PSY_HIT_SURFACE_K || h.kind == PSY_HIT_LIGHT_K) {
            out.prim = h.kind == PSY_HIT_SURFACE_K ? __ldg(S.tri_idx + h.prim).w : h.prim;
            out.inst = S.instances[h.slot].id;
            out.t = h.t; out.b0 = h.b0; out.b1 = h.b1; out.b2 = h.b2;
        }
        hits[q] = out;
    }
};

// Persistent traversal: each warp keeps its lanes busy by refilling lanes
// whose ray finished with the next rays of a global work counter (one
// aggregated atomic per warp), so long and short rays no longer idle the
// rest of the warp (Aila & Laine, "Understanding the Efficiency of Ray
// Traversal on GPUs", 2009).
template <int STACK, int MINB, class IO>
__global__ void __launch_bounds__(128, MINB) k_trace_persist(GScene S, IO io, uint32_t *work, int *err,
                                                            unsigned long long *counters) {
    __shared__ uint8_t table[8 * 48];
    load_traversal_table(table);
    const uint32_t n = io.n();
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint32_t stack[STACK];
    Lane L;
    bool active = false, exhausted = false;
    uint32_t id = 0, nr = 0;
    TraceCount tc{0, 0};
    const bool count = counters != nullptr;
    while (true) {
        unsigned idle = __ballot_sync(FULL, !active);
        if (idle && !exhausted) {
            int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(work, (uint32_t)__popc(idle));
            base = __shfl_sync(FULL, base, leader);
            if (base + (uint32_t)__popc(idle) >= n) exhausted = true;
            if (!active) {
                uint32_t my = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (my < n) {
                    V3 o, d;
                    float tmax, time;
                    bool oc;
                    id = io.load(my, o, d, tmax, time, oc);
                    lane_init(S, L, o, d, tmax, time, oc);
                    active = true;
                    nr++;
                }
            }
        }
        if (!__any_sync(FULL, active)) break;
        if (active) {
            int r = lane_step<STACK>(S, table, L, stack, tc, count);
            if (r != 0) {
                if (r < 0) {
                    atomicExch(err, PSY_E_OVERFLOW);
                    L.hit.kind = PSY_HIT_MISS_K;
                }
                io.store(S, id, L.hit);
                active = false;
            }
        }
    }
    if (count) {
        unsigned long long a = tc.nodes, b = tc.tris, c = nr;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_down_sync(FULL, a, off);
            b += __shfl_down_sync(FULL, b, off);
            c += __shfl_down_sync(FULL, c, off);
        }
        if (lane == 0) {
            atomicAdd(counters, a);
            atomicAdd(counters + 1, b);
            atomicAdd(counters + 2, c);
        }
    }
}

template <class IO, int STACK, int MINB>
static int persist_grid() {
    static int g = 0;
    if (g == 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trace_persist<STACK, MINB, IO>, 128, 0);
        g = sms * (per > 0 ? per : 1);
    }
    return g;
}

template <class IO>
static cudaError_t launch_persist(const GScene &S, const IO &io, uint32_t max_count, int stack, int minb,
                                  uint32_t *work, int *d_err, unsigned long long *counters, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(work, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
#define TP(SZ, MB)                                                                          \
    {                                                                                       \
        int g = persist_grid<IO, SZ, MB>();                                                 \
        uint32_t need = (max_count + 127) / 128;                                            \
        if ((uint32_t)g > need) g = (int)need;                                              \
        if (g > 0) k_trace_persist<SZ, MB, IO><<<g, 128, 0, st>>>(S, io, work, d_err, counters); \
    }
    if (minb >= 8) {
        if (stack <= 32) TP(32, 8) else if (stack <= 64) TP(64, 8) else TP(192, 8)
    } else if (minb >= 6) {
        if (stack <= 32) TP(32, 6) else if (stack <= 64) TP(64, 6) else TP(192, 6)
    } else {
        if (stack <= 32) TP(32, 4) else if (stack <= 64) TP(64, 4) else TP(192, 4)
    }
#undef TP
    return cudaGetLastError();
}

cudaError_t launch_trace_persist_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue,
                                       const uint32_t *count, uint32_t max_count, int stack, int minb, uint32_t *work,
                                       int *d_err, unsigned long long *counters, cudaStream_t st) {
    IOQueue io{queue, count, R.o, R.d, R.occl, H.ki, H.tb};
    return launch_persist(S, io, max_count, stack, minb, work, d_err, counters, st);
}
cudaError_t launch_trace_persist_rays(const GScene &S, const PsyRay *rays, uint32_t n, PsyHit *hits, int stack,
                                      int minb, uint32_t *work, int *d_err, unsigned long long *counters,
                                      cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    IORays io{rays, n, hits};
    return launch_persist(S, io, n, stack, minb, work, d_err, counters, st);
}

// Queue-driven trace for the render wavefront: a grid-stride loop over the
// live paths listed in queue[0 .. *count).  COUNT adds the work counters
// (node visits, triangle tests, rays) into counters[0..2].
template <int STACK, bool COUNT>
__global__ void __launch_bounds__(128) k_trace_queue(GScene S, RayBuf R, HitBuf H, const uint32_t *__restrict__ queue,
                                                     const uint32_t *__restrict__ count, int *err,
                                                     unsigned long long *counters) {
    __shared__ uint8_t table[8 * 48];
    load_traversal_table(table);
    uint32_t n = *count;
    TraceCount tc{0, 0};
    uint32_t nr = 0;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        uint32_t p = queue[q];
        float4 ro = R.o[p], rd = R.d[p];
        HitRec h;
        if (!trace_ray<STACK, COUNT>(S, table, v3(ro), v3(rd), ro.w, rd.w, R.occl[p] != 0, h, &tc)) {
            atomicExch(err, PSY_E_OVERFLOW);
            h.kind = PSY_HIT_MISS_K;
        }
        nr++;
        H.ki[p] = make_uint4(h.kind, h.prim, h.slot, 0u);
        H.tb[p] = make_float4(h.t, h.b0, h.b1, h.b2);
    }
    if (COUNT) {
        unsigned long long a = tc.nodes, b = tc.tris, c = nr;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, off);
            b += __shfl_down_sync(0xffffffffu, b, off);
            c += __shfl_down_sync(0xffffffffu, c, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(counters, a);
            atomicAdd(counters + 1, b);
            atomicAdd(counters + 2, c);
        }
    }
}

cudaError_t launch_trace_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue, const uint32_t *count,
                               uint32_t max_count, int stack, int block, int grid, int *d_err,
                               unsigned long long *counters, cudaStream_t st) {
    (void)block;
    if (grid <= 0) grid = (int)((max_count + 127) / 128);
    if (grid == 0) return cudaSuccess;
    bool c = counters != nullptr;
#define TQ(SZ)                                                                                            \
    if (c) k_trace_queue<SZ, true><<<grid, 128, 0, st>>>(S, R, H, queue, count, d_err, counters);        \
    else k_trace_queue<SZ, false><<<grid, 128, 0, st>>>(S, R, H, queue, count, d_err, counters)
    if (stack <= 32) { TQ(32); }
    else if (stack <= 64) { TQ(64); }
    else { TQ(192); }
#undef TQ
    return cudaGetLastError();
}

// ------------------------------------------------------------------ wave segments
// Copies the wave descriptor into shared memory (one read per block).
__device__ __forceinline__ void load_wave(const WaveDesc *__restrict__ g, WaveDesc &sm) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g);
    uint32_t *dst = reinterpret_cast<uint32_t *>(&sm);
    for (int i = threadIdx.x; i < (int)(sizeof(WaveDesc) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
}
__device__ __forceinline__ int seg_of_path(const WaveDesc &wd, uint32_t p) {
    int i = 0;
    while (i + 1 < (int)wd.nseg && p >= wd.seg[i + 1].path_begin) i++;
    return i;
}
__device__ __forceinline__ int seg_of_pixel(const WaveDesc &wd, uint32_t q) {
    int i = 0;
    while (i + 1 < (int)wd.nseg && q >= wd.seg[i + 1].pix_begin) i++;
    return i;
}

// ------------------------------------------------------------------ camera
// Ray generation of Renderer::render_job (src/renderer.rs:241-275) and
// LightPath::new (src/renderer.rs:392-431) / Camera::generate_ray
// (src/camera.rs:74-102).
template <class RT>
__global__ void k_camera(GScene S, const WaveDesc *__restrict__ gwave, PathState P, RayBuf R, uint32_t *queue,
                         uint32_t *count) {
    __shared__ WaveDesc wdesc;
    load_wave(gwave, wdesc);
    uint32_t n = wdesc.npaths;
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *count = n;
    if (p >= n) return;
    const WaveSeg &w = wdesc.seg[seg_of_path(wdesc, p)];
    uint32_t lp = (p - w.path_begin) / w.spp, si = (p - w.path_begin) - lp * w.spp;
    uint32_t x = w.x0 + lp % w.w, y = w.y0 + lp / w.w;
    float cmpx = 1.0f / (float)w.img_w, cmpy = 1.0f / (float)w.img_h;
    float min_x = -1.0f, max_x = 1.0f;
    float min_y = -((float)w.img_h / (float)w.img_w), max_y = (float)w.img_h / (float)w.img_w;
    float xe = max_x - min_x, ye = max_y - min_y;
    float d[4], d4[4];
    get_sample_4d(si, 0, x, y, w.seed, d);
    get_sample_4d(si, 1, x, y, w.seed, d4);
    float fx = probit<RT>(d[3], 2.0f / 6.0f) + 0.5f;
    float fy = probit<RT>(d4[0], 2.0f / 6.0f) + 0.5f;
    float sx = (fx + (float)x) * cmpx;
    float sy = (fy + (float)y) * cmpy;
    float ix = (sx - 0.5f) * xe, iy = (0.5f - sy) * ye;
    float wl = map_0_1_to_wavelength(golden_ratio_sample(si, hash_u32((x << 16) ^ y, w.seed)));
    float time = d[0];
    // Camera::generate_ray
    Xf xf = lerp_slice_xf(S.cam_xf, S.n_cam_xf, time);
    float tfov = lerp_slice_f(S.cam_tfov, S.n_cam_tfov, time);
    float ar = lerp_slice_f(S.cam_ap, S.n_cam_ap, time);
    float fd = lerp_slice_f(S.cam_fd, S.n_cam_fd, time);
    float cu, cv;
    square_to_circle((d[1] * 2.0f) - 1.0f, (d[2] * 2.0f) - 1.0f, &cu, &cv);
    V3 orig = v3(ar * cu, ar * cv, 0.0f);
    V3 dir = normalized(v3((ix * tfov) - (orig.x / fd), (iy * tfov) - (orig.y / fd), 1.0f));
    V3 wo = xf_point(orig, xf), wd = xf_vector(dir, xf);
    P.color[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    P.latt[p] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    P.pending[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    P.nafac[p] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    P.nb_o[p] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);  // w: closure_sample_pdf = 1
    P.nb_d[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    P.tw[p] = make_float2(time, wl);
    P.seed[p] = w.seed ^ 0x40d4682bu;
    P.flags[p] = 0u;  // EV_CAMERA, bounce 0, no next bounce, 0 rays
    R.o[p] = make_float4(wo.x, wo.y, wo.z, CUDART_INF_F);
    R.d[p] = make_float4(wd.x, wd.y, wd.z, time);
    R.occl[p] = 0;
    queue[p] = p;
}

cudaError_t launch_camera(const GScene &S, const WaveDesc *d_wave, uint32_t max_paths, PathState P, RayBuf R,
                          uint32_t *queue, uint32_t *count, int prec, cudaStream_t st) {
    uint32_t n = max_paths;
    if (n == 0) return cudaSuccess;
    if (prec == 1) k_camera<float><<<(n + 255) / 256, 256, 0, st>>>(S, d_wave, P, R, queue, count);
    else k_camera<double><<<(n + 255) / 256, 256, 0, st>>>(S, d_wave, P, R, queue, count);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ shade
#define EV_CAMERA 0u
#define EV_BOUNCE 1u
#define EV_SHADOW 2u

__device__ __forceinline__ void push_live(bool alive, uint32_t p, uint32_t *next_queue, uint32_t *next_count) {
    unsigned mask = __ballot_sync(__activemask(), alive);
    if (mask == 0) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(next_count, (uint32_t)__popc(mask));
    base = __shfl_sync(__activemask(), base, leader);
    if (alive) next_queue[base + __popc(mask & ((1u << lane) - 1u))] = p;
}

// LightPath::next (src/renderer.rs:449-691).
// Sort key of a path's next ray: occlusion flag, direction octant, origin
// cell (bits/3 - 1 bits per axis of the scene box), packed into `bits` bits.
__device__ __forceinline__ uint32_t ray_sort_key(const GScene &S, float4 o, float4 d, bool occl, int bits) {
    uint32_t key = occl ? 1u : 0u;
    if (bits >= 4) key |= ray_code(v3(d)) << 1;
    if (bits >= 7) {
        int per = (bits - 4) / 3;  // 1 or 2 bits per axis
        float cells = (float)(1 << per);
        uint32_t cx = (uint32_t)fminf(fmaxf((o.x - S.bounds_min.x) * S.bounds_inv_extent.x * cells, 0.0f), cells - 1.0f);
        uint32_t cy = (uint32_t)fminf(fmaxf((o.y - S.bounds_min.y) * S.bounds_inv_extent.y * cells, 0.0f), cells - 1.0f);
        uint32_t cz = (uint32_t)fminf(fmaxf((o.z - S.bounds_min.z) * S.bounds_inv_extent.z * cells, 0.0f), cells - 1.0f);
        key |= ((cx << (2 * per)) | (cy << per) | cz) << 4;
    }
    return key;
}

template <class RT, bool SORT>
__global__ void __launch_bounds__(128) k_shade(GScene S, const WaveDesc *__restrict__ gwave, PathState P, RayBuf R,
                                               HitBuf H, const uint32_t *__restrict__ queue,
                                               const uint32_t *__restrict__ count, uint32_t *next_queue,
                                               uint32_t *next_count, SortBuf sb) {
    __shared__ WaveDesc wdesc;
    load_wave(gwave, wdesc);
    uint32_t n = *count;
    uint32_t stride = gridDim.x * blockDim.x;
    uint32_t nloop = (n + stride - 1) / stride * stride;  // keep whole warps in the loop for the ballot
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nloop; q += stride) {
        bool alive = false;
        uint32_t p = 0;
        if (q < n) {
            p = queue[q];
            uint32_t fl = P.flags[p];
            uint32_t ev = fl & 3u, bounce = (fl >> 2) & 0xFFu, has_nb = (fl >> 10) & 1u, nrays = fl >> 16;
            nrays += 1;
            float2 tw = P.tw[p];
            float time = tw.x, wl = tw.y;
            uint4 ki = H.ki[p];
            float4 tb = H.tb[p];
            float4 ro = R.o[p], rd = R.d[p];
            V3 o = v3(ro), d = v3(rd);
            V4 color = v4(P.color[p]);
            V4 latt = v4(P.latt[p]);
            float4 nbo = P.nb_o[p];
            float csp = nbo.w;  // closure_sample_pdf
            uint32_t seed = P.seed[p];
            const WaveSeg &w = wdesc.seg[seg_of_path(wdesc, p)];
            uint32_t lp = p - w.path_begin;
            uint32_t pix = lp / w.spp;
            uint32_t si = lp - pix * w.spp;
            uint32_t px = w.x0 + pix % w.w, py = w.y0 + pix / w.w;
            if (ev == EV_CAMERA || ev == EV_BOUNCE) {
                if (ki.x == PSY_HIT_SURFACE_K || ki.x == PSY_HIT_LIGHT_K) {
                    HitRec h;
                    h.kind = ki.x; h.prim = ki.y; h.slot = ki.z;
                    h.t = tb.x; h.b0 = tb.y; h.b1 = tb.z; h.b2 = tb.w;
                    SurfData sd;
                    resolve_hit<RT>(S, h, o, d, time, sd);
                    const Closure &cl = sd.closure;
                    if (cl.kind == PSY_CL_EMIT) {
                        V4 c = color_to_spectral(cl.color, wl);
                        if (ev == EV_CAMERA) {
                            color = color + c;
                        } else {
                            float mis = power_heuristic(csp, sd.sample_pdf);
                            color = color + c * latt / splat4(mis);
                        }
                        P.color[p] = f4(color);
                    } else {
                        latt = latt / splat4(csp);
                        seed += 1;
                        float smp[4];
                        get_sample_4d(si, 0, px, py, seed, smp);
                        LightSample li = scene_sample_lights<RT>(S, smp[0], smp[1], smp[2], wl, time, d, sd.pos,
                                                                 sd.nor, sd.nor_g, cl);
                        bool found = false;
                        if (li.kind != 0 && !(li.pdf <= 0.0f) && !(li.sel_pdf <= 0.0f)) {
                            V4 att;
                            float cpdf;
                            V3 so, sdir;
                            float smax;
                            if (li.kind == 1) {
                                att = closure_evaluate(cl, d, li.dir, sd.nor, sd.nor_g, wl, &cpdf);
                                so = robust_ray_origin(sd.pos, sd.pos_err, normalized(sd.nor_g), li.dir);
                                sdir = li.dir;
                                smax = CUDART_INF_F;
                            } else {
                                V3 dir = li.sp - sd.pos;
                                att = closure_evaluate(cl, d, dir, sd.nor, sd.nor_g, wl, &cpdf);
                                so = robust_ray_origin(sd.pos, sd.pos_err, normalized(sd.nor_g), dir);
                                V3 oe = robust_ray_origin(li.sp, li.serr, normalized(li.sn), neg(dir));
                                sdir = oe - so;
                                smax = 1.0f;
                            }
                            if (!(max_elem4(att) <= 0.0f)) {
                                float lmis = power_heuristic(li.pdf, cpdf);
                                V4 pend = li.color * att * latt / splat4(lmis * li.sel_pdf);
                                P.pending[p] = f4(pend);
                                R.o[p] = make_float4(so.x, so.y, so.z, smax);
                                R.d[p] = make_float4(sdir.x, sdir.y, sdir.z, time);
                                R.occl[p] = 1;
                                found = true;
                            }
                        }
                        bool do_bounce = false;
                        V4 nafac = v4(P.nafac[p]);
                        if (bounce < S.max_bounces) {
                            bounce += 1;
                            seed += 1;
                            float b4[4];
                            get_sample_4d(si, 0, px, py, seed, b4);
                            V3 dir;
                            float pdf;
                            V4 filt = closure_sample(cl, d, sd.nor, sd.nor_g, b4[0], b4[1], wl, &dir, &pdf);
                            if ((pdf > 0.0f) && (max_elem4(filt) > 0.0f)) {
                                nafac = filt;
                                csp = pdf;
                                V3 nb = robust_ray_origin(sd.pos, sd.pos_err, normalized(sd.nor_g), dir);
                                P.nafac[p] = f4(nafac);
                                P.nb_o[p] = make_float4(nb.x, nb.y, nb.z, csp);
                                P.nb_d[p] = make_float4(dir.x, dir.y, dir.z, 0.0f);
                                has_nb = 1;
                                do_bounce = true;
                            }
                        } else {
                            has_nb = 0;
                        }
                        if (found) {
                            ev = EV_SHADOW;
                            alive = true;
                        } else if (do_bounce) {
                            float4 nb = P.nb_o[p], nd = P.nb_d[p];
                            R.o[p] = make_float4(nb.x, nb.y, nb.z, CUDART_INF_F);
                            R.d[p] = make_float4(nd.x, nd.y, nd.z, time);
                            R.occl[p] = 0;
                            ev = EV_BOUNCE;
                            latt = latt * nafac;
                            alive = true;
                        }
                        P.latt[p] = f4(latt);
                        P.seed[p] = seed;
                    }
                } else {
                    V4 bg = color_to_spectral(S.background, wl);
                    color = color + bg * latt / splat4(csp);
                    P.color[p] = f4(color);
                }
            } else {
                // shadow ray result
                if (ki.x == PSY_HIT_MISS_K) {
                    color = color + v4(P.pending[p]);
                    P.color[p] = f4(color);
                }
                if (has_nb) {
                    float4 nb = P.nb_o[p], nd = P.nb_d[p];
                    R.o[p] = make_float4(nb.x, nb.y, nb.z, CUDART_INF_F);
                    R.d[p] = make_float4(nd.x, nd.y, nd.z, time);
                    R.occl[p] = 0;
                    latt = latt * v4(P.nafac[p]);
                    P.latt[p] = f4(latt);
                    ev = EV_BOUNCE;
                    alive = true;
                }
            }
            P.flags[p] = ev | (bounce << 2) | (has_nb << 10) | (nrays << 16);
        }
        if (SORT) {
            uint32_t key = 0;
            if (alive) key = ray_sort_key(S, R.o[p], R.d[p], R.occl[p] != 0, sb.bits);
            unsigned mask = __ballot_sync(__activemask(), alive);
            if (mask != 0) {
                int lane = threadIdx.x & 31;
                int leader = __ffs(mask) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(next_count, (uint32_t)__popc(mask));
                base = __shfl_sync(__activemask(), base, leader);
                if (alive) {
                    uint32_t pos = base + __popc(mask & ((1u << lane) - 1u));
                    sb.stage[pos] = p;
                    sb.stage_key[pos] = (uint16_t)key;
                    // one atomic per distinct key in the warp
                    unsigned same = __match_any_sync(mask, key);
                    if (lane == __ffs(same) - 1) atomicAdd(sb.bins + key, (uint32_t)__popc(same));
                }
            }
        } else {
            push_live(alive, p, next_queue, next_count);
        }
    }
}

// Scatter staged paths into the next queue grouped by sort key.
__global__ void k_bin_scatter(const uint32_t *__restrict__ stage, const uint16_t *__restrict__ stage_key,
                              const uint32_t *__restrict__ count, uint32_t *bins, int nbins, uint32_t *out) {
    __shared__ uint32_t offs[1024];
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int k = 0; k < nbins; k++) {
            offs[k] = acc;
            acc += bins[k];
        }
    }
    __syncthreads();
    uint32_t n = *count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = stage_key[i];
        uint32_t pos = offs[k] + atomicAdd(bins + nbins + k, 1u);
        out[pos] = stage[i];
    }
}

cudaError_t launch_shade(const GScene &S, const WaveDesc *d_wave, PathState P, RayBuf R, HitBuf H, const uint32_t *queue,
                         const uint32_t *count, uint32_t max_count, uint32_t *next_queue, uint32_t *next_count,
                         int block, int grid, int prec, cudaStream_t st) {
    (void)block;
    if (grid <= 0) grid = (int)((max_count + 127) / 128);
    if (grid == 0) return cudaSuccess;
    SortBuf none{nullptr, nullptr, nullptr, 0};
    if (prec == 1) k_shade<float, false><<<grid, 128, 0, st>>>(S, d_wave, P, R, H, queue, count, next_queue, next_count, none);
    else k_shade<double, false><<<grid, 128, 0, st>>>(S, d_wave, P, R, H, queue, count, next_queue, next_count, none);
    return cudaGetLastError();
}

cudaError_t launch_shade_sorted(const GScene &S, const WaveDesc *d_wave, PathState P, RayBuf R, HitBuf H, const uint32_t *queue,
                                const uint32_t *count, uint32_t max_count, SortBuf sb, uint32_t *stage_count,
                                uint32_t *next_queue, int grid, int prec, cudaStream_t st) {
    if (grid <= 0) grid = (int)((max_count + 127) / 128);
    if (grid == 0) return cudaSuccess;
    int nbins = 1 << sb.bits;
    cudaError_t e = cudaMemsetAsync(sb.bins, 0, 2 * nbins * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if (prec == 1) k_shade<float, true><<<grid, 128, 0, st>>>(S, d_wave, P, R, H, queue, count, nullptr, stage_count, sb);
    else k_shade<double, true><<<grid, 128, 0, st>>>(S, d_wave, P, R, H, queue, count, nullptr, stage_count, sb);
    int sg = (int)std::min<uint32_t>((max_count + 255) / 256, 152u * 8u);
    if (sg < 1) sg = 1;
    k_bin_scatter<<<sg, 256, 0, st>>>(sb.stage, sb.stage_key, stage_count, sb.bins, nbins, next_queue);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ accumulate
// XYZ::from_spectral_sample / spp added per pixel (src/renderer.rs:299-310),
// summing the pixel's samples in sample order.
__global__ void k_accumulate(GScene S, const WaveDesc *__restrict__ gwave, PathState P) {
    __shared__ WaveDesc wdesc;
    load_wave(gwave, wdesc);
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= wdesc.npix) return;
    const WaveSeg &w = wdesc.seg[seg_of_pixel(wdesc, q)];
    uint32_t lq = q - w.pix_begin;
    uint32_t x = w.x0 + lq % w.w, y = w.y0 + lq / w.w;
    float inv = (float)w.spp;
    V3 acc = v3(0.0f, 0.0f, 0.0f);
    for (uint32_t s = 0; s < w.spp; s++) {
        uint32_t p = w.path_begin + lq * w.spp + s;
        V3 c = xyz_from_spectral(v4(P.color[p]), P.tw[p].y);
        acc = acc + (c / inv);
    }
    float *o = w.out + ((size_t)y * w.out_stride + x) * 3;
    o[0] = acc.x; o[1] = acc.y; o[2] = acc.z;
}

cudaError_t launch_accumulate(const GScene &S, const WaveDesc *d_wave, uint32_t max_pix, PathState P, cudaStream_t st) {
    if (max_pix == 0) return cudaSuccess;
    k_accumulate<<<(max_pix + 127) / 128, 128, 0, st>>>(S, d_wave, P);
    return cudaGetLastError();
}

__global__ void k_count_rays(PathState P, uint32_t n, unsigned long long *out) {
    unsigned long long local = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) local += P.flags[i] >> 16;
    for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, local);
}
cudaError_t launch_count_rays(PathState P, uint32_t n, unsigned long long *out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_count_rays<<<152 * 4, 256, 0, st>>>(P, n, out);
    return cudaGetLastError();
}

// Host helper: set the magenta constant (rec709_to_xyz((1,0,1))) computed by
// the host with the reference's f32 arithmetic.
void psy_set_magenta(const float xyz[3]) {
    GColor c{PSY_COLOR_XYZ_K, xyz[0], xyz[1], xyz[2]};
    cudaMemcpyToSymbol(c_magenta, &c, sizeof(c));
}
