// Traversal kernels of the GB300 tracing path: closest / any hit for ray
// batches (one thread per ray, or persistent with lane refill) and for the
// render wavefront's queues.
#include <cuda_fp16.h>

#include <algorithm>

#include "dev_bins.cuh"
#include "dev_packet.cuh"
#include "dev_surface.cuh"
#include "kernels.cuh"
#include "radix_sort.h"

using namespace psyd;

// Set once the push tables of the static-scene traversal are on the device;
// that traversal is launched only then.
static bool g_push_tables = false;

// ------------------------------------------------------------------ ray tracing
// STATIC: the static-scene traversal (trace_ray_static; the scene must have
// static_fast set, and the launch passes no counters); SPEC: its speculative
// form; H16: the static-scene traversal over the FP16 node copy.
template <int STACK, bool COUNT, int MINB, bool STATIC = false, bool SPEC = false, bool H16 = false>
__global__ void __launch_bounds__(128, MINB) k_trace_rays(GScene S, const PsyRay *__restrict__ rays, uint32_t n,
                                                    const uint32_t *__restrict__ order, PsyHit *__restrict__ hits,
                                                    PsySurfaceHit *__restrict__ full, int *err,
                                                    unsigned long long *counters) {
    __shared__ __align__(16) uint8_t table[8 * 48];  // push rows per octant and traversal code
    __shared__ __align__(16) uint16_t push_lut[PSY_PUSH_ROWS * 16];
    __shared__ float4 xfm[STATIC ? 1 : PSY_XFM_SLOT(MINB) * 128];  // per-thread slot of the general traversal
    __shared__ uint32_t sstack[STATIC && PSY_SSTACK > 0 ? PSY_SSTACK * PSY_TRACE_BLOCK : 1];  // stack tops (static)
    if (blockIdx.x * blockDim.x >= n) return;  // (whole block: before the table barrier)
    load_push_tables(table, push_lut);
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t i = q;
    TraceCount tc{0, 0};
    if (q < n) {
        if (order) i = order[q];  // binned order: thread q traces ray order[q]
        const float *r = reinterpret_cast<const float *>(rays + i);
        V3 o = v3(r[0], r[1], r[2]), d = v3(r[3], r[4], r[5]);
        float tmax = r[6], time = r[7];
        uint32_t flags = reinterpret_cast<const uint32_t *>(r)[9];
        HitRec h;
        bool oc = (flags & PSY_RAY_OCCLUSION) != 0;
        bool ok = STATIC ? trace_ray_static<STACK, SPEC, H16>(S, table, push_lut, sstack + threadIdx.x, o, d, tmax,
                                                              time, oc, h)
                         : trace_ray<STACK, COUNT, PSY_XFM_SLOT(MINB) == 6>(S, table, push_lut, xfm + PSY_XFM_SLOT(MINB) * threadIdx.x, o, d, tmax, time, oc, h, &tc);
        if (!ok) {
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
        unsigned long long a = tc.nodes, b = tc.tris, c = (q < n) ? 1ull : 0ull;
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

// Kernel variants: stack depth 64 or 192 entries (local memory only), and a
// register budget for 4 (the compiler's choice), 5, 6 or 8 resident blocks
// per SM.  Counting kernels (traversal statistics) exist for the default
// budget only: node and triangle counts do not depend on the launch shape.
cudaError_t launch_trace_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order, PsyHit *hits,
                              PsySurfaceHit *full, int stack, int minb, int *d_err, unsigned long long *counters,
                              cudaStream_t st, int fast) {
    if (n == 0) return cudaSuccess;
    dim3 b(128), g((n + 127) / 128);
    if (fast && S.static_fast && !counters) {
#define TF(SZ, MB, SP, H) \
    k_trace_rays<SZ, false, MB, true, SP, H><<<g, b, 0, st>>>(S, rays, n, order, hits, full, d_err, nullptr)
#define TFS(SZ, SP, H)                          \
    if (minb >= 12) TF(SZ, 12, SP, H);          \
    else if (minb >= 10) TF(SZ, 10, SP, H);     \
    else if (minb >= 8) TF(SZ, 8, SP, H);       \
    else TF(SZ, 6, SP, H)
        if (S.use_fp16) {  // FP16 nodes (the speculative form reads f32 nodes only)
            if (stack <= 64) { TFS(64, false, true); } else { TFS(192, false, true); }
        } else if (fast == 2) {
            if (stack <= 64) { TFS(64, true, false); } else { TFS(192, true, false); }
        } else {
            if (stack <= 64) { TFS(64, false, false); } else { TFS(192, false, false); }
        }
#undef TFS
#undef TF
        return cudaGetLastError();
    }
#define TR(SZ, C, MB) k_trace_rays<SZ, C, MB><<<g, b, 0, st>>>(S, rays, n, order, hits, full, d_err, counters)
#define TRS(SZ)                                                   \
    if (counters) TR(SZ, true, 4);                                \
    else if (minb >= 8) TR(SZ, false, 8);                         \
    else if (minb >= 6) TR(SZ, false, 6);                         \
    else if (minb == 5) TR(SZ, false, 5);                         \
    else TR(SZ, false, 4)
    if (stack <= 64) { TRS(64); } else { TRS(192); }
#undef TRS
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
    const uint32_t *order;  // optional: the q-th ray taken is order[q]
    __device__ __forceinline__ uint32_t n() const { return count; }
    __device__ __forceinline__ uint32_t load(uint32_t q, V3 &o, V3 &d, float &tmax, float &time, bool &oc) const {
        if (order) q = order[q];
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
        if (stack <= 64) TP(64, 8) else TP(192, 8)
    } else if (minb >= 6) {
        if (stack <= 64) TP(64, 6) else TP(192, 6)
    } else {
        if (stack <= 64) TP(64, 4) else TP(192, 4)
    }
#undef TP
    return cudaGetLastError();
}

// Static-scene traversal with lane refill (trace mode 5): the persistent
// loop of k_trace_persist over the static-scene traversal's steps
// (slane_step), so a lane whose ray finished -- a shadow ray that met an
// occluder early, a camera ray that left the scene -- takes the next ray
// while the others of its warp go on.  Hits are trace_ray_static's.
template <int STACK, int MINB, bool H16, class IO>
__global__ void __launch_bounds__(128, MINB) k_trace_static_refill(GScene S, IO io, uint32_t *work, int *err) {
    __shared__ __align__(16) uint8_t table[8 * 48];  // push rows per octant and traversal code
    __shared__ __align__(16) uint16_t push_lut[PSY_PUSH_ROWS * 16];
    load_push_tables(table, push_lut);
    const uint32_t n = io.n();
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint32_t stack[STACK + 4];  // 3 spare entries take the unconditional stores of the child push
    SLane L;
    HitRec hit;
    bool active = false, exhausted = false;
    uint32_t id = 0;
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
                    slane_init(S, L, o, d, tmax, time, oc);
                    active = true;
                }
            }
        }
        if (!__any_sync(FULL, active)) break;
        if (active) {
            int r = slane_step<STACK, H16>(S, table, push_lut, L, stack, hit);
            if (r != 0) {
                if (r < 0) {
                    atomicExch(err, PSY_E_OVERFLOW);
                    hit.kind = PSY_HIT_MISS_K;
                }
                io.store(S, id, hit);
                active = false;
            }
        }
    }
}

template <class IO, int STACK, bool H16>
static int refill_grid() {
    static int g = 0;
    if (g == 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trace_static_refill<STACK, 10, H16, IO>, 128, 0);
        g = sms * (per > 0 ? per : 1);
    }
    return g;
}

template <class IO>
static cudaError_t launch_static_refill(const GScene &S, const IO &io, uint32_t max_count, int stack, uint32_t *work,
                                        int *d_err, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(work, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
#define TS(SZ, H)                                                                                 \
    {                                                                                             \
        int g = refill_grid<IO, SZ, H>();                                                         \
        uint32_t need = (max_count + 127) / 128;                                                  \
        if ((uint32_t)g > need) g = (int)need;                                                    \
        if (g > 0) k_trace_static_refill<SZ, 10, H, IO><<<g, 128, 0, st>>>(S, io, work, d_err);  \
    }
    if (S.use_fp16) {
        if (stack <= 64) TS(64, true) else TS(192, true)
    } else {
        if (stack <= 64) TS(64, false) else TS(192, false)
    }
#undef TS
    return cudaGetLastError();
}

cudaError_t launch_trace_static_refill_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue,
                                             const uint32_t *count, uint32_t max_count, int stack, uint32_t *work,
                                             int *d_err, cudaStream_t st) {
    IOQueue io{queue, count, R.o, R.d, R.occl, H.ki, H.tb};
    return launch_static_refill(S, io, max_count, stack, work, d_err, st);
}
cudaError_t launch_trace_static_refill_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order,
                                            PsyHit *hits, int stack, uint32_t *work, int *d_err, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    IORays io{rays, n, hits, order};
    return launch_static_refill(S, io, n, stack, work, d_err, st);
}

cudaError_t launch_trace_persist_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue,
                                       const uint32_t *count, uint32_t max_count, int stack, int minb, uint32_t *work,
                                       int *d_err, unsigned long long *counters, cudaStream_t st) {
    IOQueue io{queue, count, R.o, R.d, R.occl, H.ki, H.tb};
    return launch_persist(S, io, max_count, stack, minb, work, d_err, counters, st);
}
cudaError_t launch_trace_persist_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order,
                                      PsyHit *hits, int stack, int minb, uint32_t *work, int *d_err,
                                      unsigned long long *counters, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    IORays io{rays, n, hits, order};
    return launch_persist(S, io, n, stack, minb, work, d_err, counters, st);
}

// ------------------------------------------------------------------ warp-packet traversal
// One warp traces 32 rays as a packet (dev_packet.cuh); the warp's stack
// lives in shared memory.  Grid-stride over the rays in warp-sized chunks.
template <int STACK>
struct PacketDepth {
    // every hit child is pushed (not count - 1 as per ray), plus octant
    // groups at the root and at instance entry
    static constexpr int value = 2 * STACK + 32;
};
template <int STACK, bool COUNT, class IO>
__global__ void __launch_bounds__(128) k_trace_packet(GScene S, IO io, int *err, unsigned long long *counters) {
    constexpr int DEPTH = PacketDepth<STACK>::value;
    __shared__ uint8_t table[8 * 48];
    __shared__ PacketEntry stk[4][DEPTH];
    load_traversal_table(table);
    PacketEntry *st = stk[threadIdx.x >> 5];
    const uint32_t n = io.n();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    TraceCount tc{0, 0};
    uint32_t nr = 0;
    for (uint32_t base = wid * 32; base < n; base += nw * 32) {
        uint32_t q = base + lane;
        bool active = q < n;
        V3 o = v3(0.0f, 0.0f, 0.0f), d = v3(0.0f, 0.0f, 1.0f);
        float tmax = 0.0f, time = 0.0f;
        bool oc = false;
        uint32_t p = 0;
        if (active) p = io.load(q, o, d, tmax, time, oc);
        HitRec h;
        bool ok = trace_packet<DEPTH, COUNT>(S, table, st, active, o, d, tmax, time, oc, h, &tc);
        if (active) {
            if (!ok) {
                atomicExch(err, PSY_E_OVERFLOW);
                h.kind = PSY_HIT_MISS_K;
            }
            io.store(S, p, h);
            nr++;
        }
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

template <class IO>
static cudaError_t launch_packet(const GScene &S, const IO &io, uint32_t max_count, int stack, int grid, int *d_err,
                                 unsigned long long *counters, cudaStream_t st) {
    if (grid <= 0) grid = (int)((max_count + 127) / 128);
    if (grid == 0) return cudaSuccess;
#define TK(SZ, C) k_trace_packet<SZ, C, IO><<<grid, 128, 0, st>>>(S, io, d_err, counters)
    if (stack <= 64) {
        if (counters) TK(64, true); else TK(64, false);
    } else {
        if (counters) TK(192, true); else TK(192, false);
    }
#undef TK
    return cudaGetLastError();
}
cudaError_t launch_trace_packet_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue,
                                      const uint32_t *count, uint32_t max_count, int stack, int grid, int *d_err,
                                      unsigned long long *counters, cudaStream_t st) {
    IOQueue io{queue, count, R.o, R.d, R.occl, H.ki, H.tb};
    return launch_packet(S, io, max_count, stack, grid, d_err, counters, st);
}
cudaError_t launch_trace_packet_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order,
                                     PsyHit *hits, int stack, int *d_err, unsigned long long *counters,
                                     cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    IORays io{rays, n, hits, order};
    return launch_packet(S, io, n, stack, 0, d_err, counters, st);
}

// Queue-driven trace for the render wavefront: a grid-stride loop over the
// live paths listed in queue[0 .. *count).  COUNT adds the work counters
// (node visits, triangle tests, rays) into counters[0..2].
template <int STACK, bool COUNT, int MINB, bool STATIC = false, bool SPEC = false, bool H16 = false>
__global__ void __launch_bounds__(128, MINB) k_trace_queue(GScene S, RayBuf R, HitBuf H, const uint32_t *__restrict__ queue,
                                                     const uint32_t *__restrict__ count, int *err,
                                                     unsigned long long *counters) {
    __shared__ __align__(16) uint8_t table[8 * 48];  // push rows per octant and traversal code
    __shared__ __align__(16) uint16_t push_lut[PSY_PUSH_ROWS * 16];
    __shared__ float4 xfm[STATIC ? 1 : PSY_XFM_SLOT(MINB) * 128];  // per-thread slot of the general traversal
    __shared__ uint32_t sstack[STATIC && PSY_SSTACK > 0 ? PSY_SSTACK * PSY_TRACE_BLOCK : 1];  // stack tops (static)
    uint32_t n = *count;
    // blocks past the queue's length (the grid covers the wave's capacity)
    // leave at once, before the table copy and its barrier
    if (blockIdx.x * blockDim.x >= n) return;
    load_push_tables(table, push_lut);
    TraceCount tc{0, 0};
    uint32_t nr = 0;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        uint32_t p = queue[q];
        float4 ro = R.o[p], rd = R.d[p];
        HitRec h;
        bool oc = R.occl[p] != 0;
        bool ok = STATIC ? trace_ray_static<STACK, SPEC, H16>(S, table, push_lut, sstack + threadIdx.x, v3(ro), v3(rd),
                                                              ro.w, rd.w, oc, h)
                         : trace_ray<STACK, COUNT, PSY_XFM_SLOT(MINB) == 6>(S, table, push_lut, xfm + PSY_XFM_SLOT(MINB) * threadIdx.x, v3(ro), v3(rd), ro.w, rd.w, oc,
                                                   h, &tc);
        if (!ok) {
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
                               uint32_t max_count, int stack, int minb, int grid, int *d_err,
                               unsigned long long *counters, cudaStream_t st, int fast) {
    if (max_count == 0) return cudaSuccess;
    if (fast && S.static_fast && !counters) {
#define TF(SZ, MB, SP, HH)                                                                         \
    {                                                                                              \
        int g = queue_grid((const void *)k_trace_queue<SZ, false, MB, true, SP, HH>, grid, max_count); \
        k_trace_queue<SZ, false, MB, true, SP, HH><<<g, 128, 0, st>>>(S, R, H, queue, count, d_err, nullptr); \
    }
#define TFS(SZ, SP, HH)                         \
    if (minb >= 12) TF(SZ, 12, SP, HH)          \
    else if (minb >= 10) TF(SZ, 10, SP, HH)     \
    else if (minb >= 8) TF(SZ, 8, SP, HH)       \
    else TF(SZ, 6, SP, HH)
        if (S.use_fp16) {  // FP16 nodes (the speculative form reads f32 nodes only)
            if (stack <= 64) { TFS(64, false, true); } else { TFS(192, false, true); }
        } else if (fast == 2) {
            if (stack <= 64) { TFS(64, true, false); } else { TFS(192, true, false); }
        } else {
            if (stack <= 64) { TFS(64, false, false); } else { TFS(192, false, false); }
        }
#undef TFS
#undef TF
        return cudaGetLastError();
    }
#define TQ(SZ, C, MB)                                                                              \
    {                                                                                              \
        int g = queue_grid((const void *)k_trace_queue<SZ, C, MB>, grid, max_count);               \
        k_trace_queue<SZ, C, MB><<<g, 128, 0, st>>>(S, R, H, queue, count, d_err, counters);       \
    }
#define TQS(SZ)                                                  \
    if (counters) TQ(SZ, true, 4)                                \
    else if (minb >= 8) TQ(SZ, false, 8)                         \
    else if (minb >= 6) TQ(SZ, false, 6)                         \
    else if (minb == 5) TQ(SZ, false, 5)                         \
    else TQ(SZ, false, 4)
    if (stack <= 64) { TQS(64); } else { TQS(192); }
#undef TQS
#undef TQ
    return cudaGetLastError();
}

// ------------------------------------------------------------------ ray order
// Before a large trace call, rays can be put in an order where a warp's rays
// start near each other and run in similar directions.  Key: 30-bit 6-D
// Morton code of the ray's origin and of the point at distance L along its
// unit direction, 5 bits per coordinate over the scene box grown by L on
// every side, L = 1/20 of the box diagonal (the "two-point" key of Meister,
// Boksansky, Guthe and Bittner, "On Ray Reordering Techniques for Faster GPU
// Ray Tracing", I3D 2020); then a stable radix sort of (key, ray index).
// Each ray's hit is still written at its own index, so results do not
// depend on the order.
__global__ void k_ray_keys(const PsyRay *__restrict__ rays, uint32_t n, float4 lo, float4 inv, float len,
                           uint32_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *r = reinterpret_cast<const float *>(rays + i);
    keys[i] = two_point_key(r[0], r[1], r[2], r[3], r[4], r[5], lo, inv, len, 5);
    vals[i] = i;
}

cudaError_t launch_ray_order(const GScene &S, const PsyRay *rays, uint32_t n, const RayOrderBufs &B,
                             const uint32_t **order, cudaStream_t st) {
    *order = nullptr;
    if (n == 0) return cudaSuccess;
    float4 glo, ginv;
    float len;
    two_point_box(S, glo, ginv, len);
    k_ray_keys<<<(n + 255) / 256, 256, 0, st>>>(rays, n, glo, ginv, len, B.keys, B.vals);
    uint32_t *ok = nullptr, *ov = nullptr;
    cudaError_t e = radix_sort_pairs(B.keys, B.vals, B.keys2, B.vals2, B.scratch, n, 30, &ok, &ov, st);
    *order = ov;
    return e;
}

// Push tables of the static-scene traversal from the device traversal table
// (positions past a node's child count already name its empty slots).
// Codes 0..26 order four children, 27..44 three, 45..47 two.
static bool push_tables_host(const uint8_t table[8][48], uint8_t rows[8][48], uint16_t lut[PSY_PUSH_ROWS][16]) {
    uint32_t keys[PSY_PUSH_ROWS];
    int nrows = 0;
    for (int oct = 0; oct < 8; oct++)
        for (int code = 0; code < 48; code++) {
            uint32_t count = code < 27 ? 4u : (code < 45 ? 3u : 2u);
            uint32_t key = table[oct][code] | (count << 8);
            int r = 0;
            while (r < nrows && keys[r] != key) r++;
            if (r == nrows) {
                if (nrows == PSY_PUSH_ROWS) return false;  // (8 + 8 + 8 + 2 distinct pairs are expected)
                keys[nrows++] = key;
                for (uint32_t m = 0; m < 16; m++) {
                    uint32_t me = m & ((1u << count) - 1u), list[4], k = 0;
                    for (int i = 0; i < 4; i++) {
                        uint32_t ci = (table[oct][code] >> (2 * i)) & 3u;
                        if ((me >> ci) & 1u) list[k++] = ci;
                    }
                    uint32_t e = 0;
                    if (k > 0) {
                        e = list[0] | ((k - 1) << 8) | 0x800u;
                        for (uint32_t j = 0; j + 1 < k; j++) e |= list[k - 1 - j] << (2 + 2 * j);
                    }
                    lut[r][m] = (uint16_t)e;
                }
            }
            rows[oct][code] = (uint8_t)r;
        }
    for (int r = nrows; r < PSY_PUSH_ROWS; r++)
        for (int m = 0; m < 16; m++) lut[r][m] = 0;
    return true;
}

bool psy_trace_tables_ready() { return g_push_tables; }

// The push tables as the device receives them (host-side only; for tests).
bool psy_push_tables_host(uint8_t rows[8][48], uint16_t lut[32][16]) {
    static_assert(PSY_PUSH_ROWS == 32, "table size of the debug export");
    uint8_t t[8][48];
    psy_traversal_table_device(t);
    return push_tables_host(t, rows, lut);
}

// Constants of this translation unit: the child-order table and the colour
// of unshaded instances (kernels.cu keeps its own copies).
void psy_upload_trace_constants(const uint8_t table[8][48], const float magenta[3]) {
    if (table) {
        cudaMemcpyToSymbol(c_traversal_table, table, 8 * 48);
        uint8_t rows[8][48];
        uint16_t lut[PSY_PUSH_ROWS][16];
        if (push_tables_host(table, rows, lut) && cudaMemcpyToSymbol(g_push_row, rows, sizeof(rows)) == cudaSuccess &&
            cudaMemcpyToSymbol(g_push_lut, lut, sizeof(lut)) == cudaSuccess)
            g_push_tables = true;
    }
    if (magenta) {
        GColor c{PSY_COLOR_XYZ_K, magenta[0], magenta[1], magenta[2]};
        cudaMemcpyToSymbol(c_magenta, &c, sizeof(c));
    }
}
