// C ABI of the GB300 tracing path (include/psy_gpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "kernels.cuh"
#include "psy_debug.h"
#include "scene_build.h"
#include "radix_sort.h"
#include "scene_handle.h"

void psy_set_magenta(const float xyz[3]);

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PSY_E_NOMEM : PSY_E_CUDA;
}
#define CK(call, what)                                \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

std::once_flag g_const_once;
int g_device_init = 0;
// Sobol directions, traversal tables and the unassigned-shader colour to the
// device's constant banks (once per process).
void upload_device_constants() {
    std::call_once(g_const_once, []() {
        psy_upload_constants();
        float m[3];
        unassigned_magenta_xyz(m);
        psy_set_magenta(m);
        g_device_init = 1;
    });
}

}  // namespace

int psy_fail(int code, const std::string &msg) { return fail(code, msg); }
int psy_cuda_fail(cudaError_t e, const char *what) { return cuda_fail(e, what); }


template <class T>
static int upload(PsyScene *s, const std::vector<T> &v, const T **out) {
    size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
    void *p = nullptr;
    CK(cudaMalloc(&p, bytes), "cudaMalloc scene");
    s->allocs.push_back(p);
    s->device_bytes += bytes;
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s->stream), "upload");
    *out = reinterpret_cast<const T *>(p);
    return PSY_OK;
}

static void free_render(PsyScene *s) {
    s->graph.reset();
    void *ptrs[] = {s->P.color, s->P.latt, s->P.pending, s->P.nafac, s->P.nb_o, s->P.nb_d, s->P.tw, s->P.seed, s->P.flags,
                    s->R.o, s->R.d, s->R.occl, s->H.ki, s->H.tb, s->queue[0], s->queue[1], s->counts, s->d_raycount,
                    s->d_stage, s->d_stage_key, s->d_bins, s->d_qradix, s->d_waves};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    s->P = PathState{};
    s->R = RayBuf{};
    s->H = HitBuf{};
    s->queue[0] = s->queue[1] = nullptr;
    s->counts = nullptr;
    s->d_raycount = nullptr;
    s->d_stage = nullptr;
    s->d_stage_key = nullptr;
    s->d_bins = nullptr;
    s->d_qradix = nullptr;
    s->d_waves = nullptr;
    s->cap_waves = 0;
    s->cap_paths = 0;
}

static int ensure_render(PsyScene *s, uint32_t n) {
    if (n <= s->cap_paths) return PSY_OK;
    free_render(s);
    size_t N = n;
#define AL(ptr, bytes) CK(cudaMalloc((void **)&(ptr), (bytes)), "cudaMalloc render state")
    AL(s->P.color, N * 16); AL(s->P.latt, N * 16); AL(s->P.pending, N * 16); AL(s->P.nafac, N * 16);
    AL(s->P.nb_o, N * 16); AL(s->P.nb_d, N * 16); AL(s->P.tw, N * 8); AL(s->P.seed, N * 4); AL(s->P.flags, N * 4);
    AL(s->R.o, N * 16); AL(s->R.d, N * 16); AL(s->R.occl, N);
    AL(s->H.ki, N * 16); AL(s->H.tb, N * 16);
    AL(s->queue[0], N * 4); AL(s->queue[1], N * 4);
    AL(s->counts, 16);
    AL(s->d_raycount, 8);
    AL(s->d_stage, N * 4); AL(s->d_stage_key, N * 2); AL(s->d_bins, 65536 * 4);
    AL(s->d_qradix, queue_radix_words(n) * 4);
#undef AL
    s->cap_paths = n;
    return PSY_OK;
}

static int ensure_trace(PsyScene *s, size_t n, bool full) {
    if (n <= s->cap_rays && (!full || s->d_full)) return PSY_OK;
    if (s->d_rays) cudaFree(s->d_rays);
    if (s->d_hits) cudaFree(s->d_hits);
    if (s->d_full) cudaFree(s->d_full);
    s->d_rays = nullptr; s->d_hits = nullptr; s->d_full = nullptr;
    size_t cap = std::max(n, s->cap_rays);
    CK(cudaMalloc((void **)&s->d_rays, cap * sizeof(PsyRay)), "cudaMalloc rays");
    CK(cudaMalloc((void **)&s->d_hits, cap * sizeof(PsyHit)), "cudaMalloc hits");
    if (full) CK(cudaMalloc((void **)&s->d_full, cap * sizeof(PsySurfaceHit)), "cudaMalloc full hits");
    s->cap_rays = cap;
    return PSY_OK;
}

// Trace calls below this many rays are not binned (the three binning
// kernels cost more than they save).
constexpr uint32_t kBinMinRays = 1u << 16;

static int ensure_counters(PsyScene *s) {
    if (s->d_counters) return PSY_OK;
    CK(cudaMalloc((void **)&s->d_counters, 3 * sizeof(unsigned long long)), "cudaMalloc counters");
    CK(cudaMemsetAsync(s->d_counters, 0, 3 * sizeof(unsigned long long), s->stream), "memset counters");
    return PSY_OK;
}

static int check_err(PsyScene *s) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "read error word");
    CK(cudaStreamSynchronize(s->stream), "stream sync");
    if (h != 0) {
        int z = 0;
        cudaMemcpy(s->d_err, &z, sizeof(int), cudaMemcpyHostToDevice);
        return fail(h, "device reported error (traversal stack overflow)");
    }
    return PSY_OK;
}

extern "C" {

const char *psy_last_error(void) { return g_last_error.c_str(); }
const char *psy_version(void) { return "psychopath_gb300 0.1 (sm_103a)"; }

int psy_scene_create(const PsySceneDesc *desc, const PsySceneOptions *opts, PsyScene **out) {
    if (!out) return fail(PSY_E_INVALID, "out is null");
    *out = nullptr;
    HostScene hs;
    std::string err;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    bool have_gpu = ce == cudaSuccess && ndev > 0;
    GpuMeshBuild gpu_build = [](const LbvhInput &in, LbvhOutput &out, std::string &e) -> int {
        cudaStream_t bs = nullptr;
        cudaError_t c = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
        if (c == cudaSuccess) c = lbvh_build_mesh(in, out, bs);
        if (bs) cudaStreamDestroy(bs);
        if (c != cudaSuccess) {
            e = std::string("GPU BVH build: ") + cudaGetErrorString(c);
            return c == cudaErrorMemoryAllocation ? PSY_E_NOMEM : PSY_E_CUDA;
        }
        return PSY_OK;
    };
    int rc = build_host_scene(desc, opts, hs, err, have_gpu ? &gpu_build : nullptr);
    if (rc != PSY_OK) return fail(rc, err);
    if (!have_gpu) return fail(PSY_E_CUDA, "no CUDA device available");
    upload_device_constants();
    if (!psy_trace_tables_ready()) return fail(PSY_E_CUDA, "traversal push tables were not uploaded");
    PsyScene *s = new PsyScene();
    if (cudaGetDevice(&s->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return fail(PSY_E_CUDA, "cudaStreamCreate failed");
    }
    GScene &g = s->g;
    int r = PSY_OK;
#define UP(field, vec) if (r == PSY_OK) r = upload(s, hs.vec, &g.field)
    UP(nodes, nodes); UP(bounds_ext, bounds_ext);
    if (!hs.nodes_h.empty()) { UP(nodes_h, nodes_h); }
    UP(tri_idx, tri_idx); UP(tris, tris); UP(verts, verts); UP(normals, normals); UP(meshes, meshes);
    UP(instances, instances); UP(xforms, xforms); UP(xforms_inv, xforms_inv); UP(shaders, shaders);
    UP(lights, lights); UP(light_dims, light_dims); UP(light_colors, light_colors);
    UP(lt_nodes, lt_nodes); UP(lt_bounds, lt_bounds); UP(light_instances, light_instances);
    UP(distant, distant); UP(distant_radii, distant_radii); UP(distant_dirs, distant_dirs);
    UP(distant_colors, distant_colors); UP(cam_xf, cam_xf); UP(cam_tfov, cam_tfov); UP(cam_ap, cam_ap);
    UP(cam_fd, cam_fd);
#undef UP
    // the spectrum tables of the scene's constant XYZ colours, built on the
    // device from their XYZ values
    if (r == PSY_OK) {
        const float4 *d_sxyz = nullptr;
        std::vector<float4> sx = hs.spec_xyz;
        r = upload(s, sx, &d_sxyz);
        void *p = nullptr;
        size_t bytes = std::max<size_t>(1, hs.spec_xyz.size()) * PSY_SPEC_TABLE * sizeof(float);
        if (r == PSY_OK) {
            cudaError_t e = cudaMalloc(&p, bytes);
            if (e == cudaSuccess) {
                s->allocs.push_back(p);
                s->device_bytes += bytes;
                e = launch_spectrum_tables(d_sxyz, (uint32_t)hs.spec_xyz.size(), (float *)p, s->stream);
            }
            if (e != cudaSuccess) r = cuda_fail(e, "spectrum tables");
        }
        g.spec_tables = (const float *)p;
        s->d_spec_xyz = d_sxyz;
        s->n_spec = (uint32_t)hs.spec_xyz.size();
    }
    if (r == PSY_OK) {
        cudaError_t e = cudaMalloc((void **)&s->d_err, sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_work, 64 * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "scene upload");
    }
    if (r != PSY_OK) {
        psy_scene_destroy(s);
        return r;
    }
    g.top_root = hs.top_root;
    g.n_instances = (uint32_t)hs.instances.size();
    g.n_light_instances = (uint32_t)hs.light_instances.size();
    g.n_distant = desc->num_distant_lights;
    g.lt_empty = hs.lt_empty ? 1u : 0u;
    g.n_cam_xf = (uint32_t)hs.cam_xf.size() / 3;
    g.n_cam_tfov = (uint32_t)hs.cam_tfov.size();
    g.n_cam_ap = (uint32_t)hs.cam_ap.size();
    g.n_cam_fd = (uint32_t)hs.cam_fd.size();
    g.background = hs.background;
    g.width = hs.width; g.height = hs.height; g.spp = hs.spp; g.seed = hs.seed; g.max_bounces = hs.max_bounces;
    g.use_fp16 = hs.nodes_h.empty() ? 0u : 1u;
    // boxes with lo <= hi on every axis let the traversal pick each axis's
    // near and far plane from the ray direction's sign alone
    g.ordered_slabs = 1u;
    for (const GNode &n : hs.nodes) {
        uint32_t cnt = n.meta.z >> 8;
        for (uint32_t k = 0; k < std::max(1u, n.meta.y); k++) {  // every time key of the node
            const GBounds4 &b = k == 0 ? *reinterpret_cast<const GBounds4 *>(&n) : hs.bounds_ext[n.meta.x + k - 1];
            const float *lo[3] = {&b.xlo.x, &b.ylo.x, &b.zlo.x}, *hi[3] = {&b.xhi.x, &b.yhi.x, &b.zhi.x};
            for (uint32_t c = 0; c < cnt && c < 4; c++)
                for (int a = 0; a < 3; a++)
                    if (!(lo[a][c] <= hi[a][c])) g.ordered_slabs = 0u;
        }
    }
    // the static-scene traversal: nodes without motion keys (FP32 or FP16),
    // ordered boxes, static meshes, untransformed mesh instances
    g.static_fast = g.ordered_slabs == 1u ? 1u : 0u;
    for (const GNode &n : hs.nodes)
        if (n.meta.y > 1) g.static_fast = 0u;
    for (const GMesh &m : hs.meshes)
        if (m.ts != 1) g.static_fast = 0u;
    for (const GInstance &in : hs.instances)
        if (in.kind == PSY_INST_MESH && in.xc != 0) g.static_fast = 0u;
    g.distant_energy_total = hs.distant_energy_total;
    g.lt_root_energy = hs.lt_root_energy;
    for (int a = 0; a < 3; a++) {
        float ext = hs.scene_max[a] - hs.scene_min[a];
        (&g.bounds_min.x)[a] = hs.scene_min[a];
        (&g.bounds_inv_extent.x)[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    s->max_stack = hs.max_stack;
    s->prec = (opts && opts->shading_precision == PSY_SHADING_F32) ? 1 : 0;
    s->ray_order = (opts && opts->ray_order == PSY_RAY_ORDER_BINNED) ? 1 : 0;
    s->stack = hs.max_stack <= 64 ? 64 : 192;
    if (hs.max_stack > 192) {
        psy_scene_destroy(s);
        return fail(PSY_E_OVERFLOW, "scene needs a traversal stack deeper than 192 entries");
    }
    s->mesh_tri_order = std::move(hs.mesh_tri_order);
    s->mesh_node_count = std::move(hs.mesh_node_count);
    s->object_to_mesh = std::move(hs.object_to_mesh);
    s->node_count = (uint32_t)hs.nodes.size();
    if (const char *wp = std::getenv("PSY_WAVE_PATHS")) {
        long v = std::atol(wp);
        if (v > 1024) s->wave_paths = (uint32_t)v;
    }
    *out = s;
    return PSY_OK;
}

int psy_scene_destroy(PsyScene *s) {
    if (!s) return PSY_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->graph.reset();
    for (void *p : s->allocs) cudaFree(p);
    free_render(s);
    if (s->d_rays) cudaFree(s->d_rays);
    if (s->d_hits) cudaFree(s->d_hits);
    if (s->d_full) cudaFree(s->d_full);
    if (s->d_xyz) cudaFree(s->d_xyz);
    if (s->d_err) cudaFree(s->d_err);
    if (s->d_counters) cudaFree(s->d_counters);
    if (s->d_work) cudaFree(s->d_work);
    if (s->d_border) cudaFree(s->d_border);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return PSY_OK;
}

int psy_scene_device_bytes(const PsyScene *s, uint64_t *bytes) {
    if (!s || !bytes) return fail(PSY_E_INVALID, "null argument");
    *bytes = s->device_bytes;
    return PSY_OK;
}

// Ray order scratch for trace calls of n rays (allocated on first use):
// 4n words of keys / values plus the radix sort's scratch.
static int ensure_binning(PsyScene *s, size_t n) {
    if (n <= s->cap_bin) return PSY_OK;
    if (s->d_border) cudaFree(s->d_border);
    s->d_border = nullptr; s->cap_bin = 0;
    size_t words = 4 * n + radix_sort_scratch_words((uint32_t)n);
    CK(cudaMalloc((void **)&s->d_border, words * sizeof(uint32_t)), "cudaMalloc ray order");
    s->cap_bin = n;
    return PSY_OK;
}

// Traces n device-resident rays; with the scene's ray_order option, large
// batches are first binned by direction octant and origin cell.
static int trace_device_core(PsyScene *s, const PsyRay *d_rays, uint32_t n, PsyHit *d_hits, PsySurfaceHit *d_full,
                             cudaStream_t st) {
    unsigned long long *ctr = nullptr;
    if (s->counting) {
        int r = ensure_counters(s);
        if (r != PSY_OK) return r;
        ctr = s->d_counters;
    }
    const uint32_t *order = nullptr;
    if (s->ray_order && n >= kBinMinRays) {
        int r = ensure_binning(s, n);
        if (r != PSY_OK) return r;
        uint32_t *b = s->d_border;
        RayOrderBufs rb{b, b + n, b + 2 * (size_t)n, b + 3 * (size_t)n, b + 4 * (size_t)n};
        CK(launch_ray_order(s->g, d_rays, n, rb, &order, st), "ray order");
    }
    if (s->trace_mode == 5 && s->g.static_fast && !d_full && !ctr)
        CK(launch_trace_static_refill_rays(s->g, d_rays, n, order, d_hits, s->stack, s->d_work, s->d_err, st),
           "trace launch");
    else if (d_full || s->trace_mode == 0 || s->trace_mode >= 3)
        CK(launch_trace_rays(s->g, d_rays, n, order, d_hits, d_full, s->stack, s->minb, s->d_err, ctr, st,
                             s->trace_mode >= 3 ? s->trace_mode - 2 : 0),
           "trace launch");
    else if (s->trace_mode == 2)
        CK(launch_trace_packet_rays(s->g, d_rays, n, order, d_hits, s->stack, s->d_err, ctr, st), "trace launch");
    else
        CK(launch_trace_persist_rays(s->g, d_rays, n, order, d_hits, s->stack, s->minb, s->d_work, s->d_err, ctr, st),
           "trace launch");
    s->rays_traced += n;
    return PSY_OK;
}

int psy_trace_device(PsyScene *s, const PsyRay *d_rays, uint32_t n, PsyHit *d_hits, void *stream) {
    if (!s || (n && (!d_rays || !d_hits))) return fail(PSY_E_INVALID, "null argument");
    if (n == 0) return PSY_OK;
    std::lock_guard<std::mutex> lk(s->mu);  // binning scratch and counters belong to the scene
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    return trace_device_core(s, d_rays, n, d_hits, nullptr, st);
}

int psy_trace(PsyScene *s, const PsyRay *rays, uint32_t n, PsyHit *hits, PsySurfaceHit *full_out, void *stream) {
    if (!s || (n && (!rays || !hits))) return fail(PSY_E_INVALID, "null argument");
    if (n == 0) return PSY_OK;
    std::lock_guard<std::mutex> lk(s->mu);
    int r = ensure_trace(s, n, full_out != nullptr);
    if (r != PSY_OK) return r;
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    CK(cudaMemcpyAsync(s->d_rays, rays, (size_t)n * sizeof(PsyRay), cudaMemcpyHostToDevice, st), "copy rays");
    r = trace_device_core(s, s->d_rays, n, s->d_hits, full_out ? s->d_full : nullptr, st);
    if (r != PSY_OK) return r;
    CK(cudaMemcpyAsync(hits, s->d_hits, (size_t)n * sizeof(PsyHit), cudaMemcpyDeviceToHost, st), "copy hits");
    if (full_out)
        CK(cudaMemcpyAsync(full_out, s->d_full, (size_t)n * sizeof(PsySurfaceHit), cudaMemcpyDeviceToHost, st),
           "copy full hits");
    CK(cudaStreamSynchronize(st), "trace sync");
    return check_err(s);
}

int psy_rays_traced(const PsyScene *s, uint64_t *count) {
    if (!s || !count) return fail(PSY_E_INVALID, "null argument");
    *count = s->rays_traced;
    return PSY_OK;
}

}  // extern "C"

// The launch sequence of one wave on stream st: camera rays, then the fixed
// 2 * max_bounces + 3 trace/shade iterations over the live-path queues, then
// accumulation.  Grids cover max_paths / max_pix (the wave's capacity); the
// kernels read the actual sizes from the descriptor, so the sequence does not
// depend on the wave's contents.  ev (optional) receives 3 + 3 * iters
// timing events.
int launch_wave(PsyScene *s, const WaveBufs &B, const WaveDesc *d_wave, uint32_t max_paths, uint32_t max_pix,
                cudaStream_t st, unsigned long long *ctr, const cudaEvent_t *ev) {
    uint32_t iters = 2 * s->g.max_bounces + 3;
    uint32_t n = max_paths;
    bool binning = s->sort_bits > 0 && B.stage && (s->sort_bits <= 16 || B.qradix);
    if (ev) cudaEventRecord(ev[0], st);
    CK(launch_camera(s->g, d_wave, n, B.P, B.R, B.queue[0], B.counts, s->prec, st), "camera launch");
    if (ev) cudaEventRecord(ev[1], st);
    // queue rotation: without binning the live paths alternate between
    // queue[0] and queue[1]; with binning shade writes queue[1] (after the
    // first iteration its input is the stage buffer) and the binning pass
    // writes the grouped queue back into the stage buffer
    uint32_t *qin = B.queue[0], *cin = B.counts;
    for (uint32_t it = 0; it < iters; it++) {
        if (ev) cudaEventRecord(ev[2 + 3 * it], st);
        // the last resident_tail iterations, whose queues hold few paths,
        // launch each kernel on its resident blocks (every kernel strides
        // over its queue, so any grid covers any count); the traversal gets
        // four rounds of them, so the block scheduler still balances the
        // rays' uneven cost while the tail's first queues are large
        const bool tail = (int)it + s->resident_tail >= (int)iters;
        const int grid = tail ? PSY_GRID_RESIDENT : s->grid;
        const int tgrid = tail ? 4 * PSY_GRID_RESIDENT : s->grid;
        if (s->trace_mode == 5 && s->g.static_fast && !ctr)
            CK(launch_trace_static_refill_queue(s->g, B.R, B.H, qin, cin, n, s->stack, B.work, B.err, st),
               "trace launch");
        else if (s->trace_mode == 1)
            CK(launch_trace_persist_queue(s->g, B.R, B.H, qin, cin, n, s->stack, s->minb, B.work, B.err, ctr, st),
               "trace launch");
        else if (s->trace_mode == 2)
            CK(launch_trace_packet_queue(s->g, B.R, B.H, qin, cin, n, s->stack, tgrid, B.err, ctr, st),
               "trace launch");
        else
            CK(launch_trace_queue(s->g, B.R, B.H, qin, cin, n, s->stack, s->minb, tgrid, B.err, ctr, st,
                                  s->trace_mode >= 3 ? s->trace_mode - 2 : 0),
               "trace launch");
        if (ev) cudaEventRecord(ev[3 + 3 * it], st);
        // the live paths go to the queue and the count this iteration did not
        // read (the input may be a compacted queue, the binning stage or the
        // radix sort's second buffer)
        uint32_t *qout = qin == B.queue[1] ? B.queue[0] : B.queue[1];
        uint32_t *cout = cin == B.counts + 1 ? B.counts : B.counts + 1;
        const bool bin_next = binning && it + 1 < iters;
        // radix-sorted ordering: the shading kernels write each live path's
        // two-point key beside it (QueueOut), and the sort runs on those
        QueueOut qo{qout, cout, nullptr, make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f),
                    0.0f, 0};
        QueueSortBufs Q{B.stage_key, B.bins, nullptr, nullptr, nullptr, nullptr};
        if (B.qradix) {
            Q.keys = B.qradix; Q.keys2 = B.qradix + B.cap; Q.vals2 = B.qradix + 2 * (size_t)B.cap;
            Q.scratch = B.qradix + 3 * (size_t)B.cap;
        }
        const bool radix = bin_next && s->sort_bits > 16;
        if (radix) {
            qo.keys = Q.keys;
            two_point_box(s->g, qo.lo, qo.inv, qo.len);
            qo.p = (s->sort_bits - 1) / 6;
        }
        CK(cudaMemsetAsync(cout, 0, 4, st), "memset count");
        CK(launch_shade(s->g, d_wave, B.P, B.R, B.H, qin, cin, n, qo, s->shade_minb, grid, s->prec, st),
           "shade launch");
        if (radix) {
            uint32_t *sorted = nullptr;
            CK(launch_queue_radix(Q, qout, cout, n, s->sort_bits, &sorted, st), "queue ordering");
            qin = sorted;
            cin = cout;
        } else if (bin_next) {
            CK(launch_queue_binning(s->g, B.R, qout, cout, n, s->sort_bits, Q, B.stage, B.counts + 2, st),
               "queue binning");
            qin = B.stage;
            cin = B.counts + 2;
        } else {
            qin = qout;
            cin = cout;
        }
        if (ev) cudaEventRecord(ev[4 + 3 * it], st);
    }
    CK(launch_accumulate(s->g, d_wave, max_pix, B.P, st), "accumulate launch");
    if (ev) cudaEventRecord(ev[2 + 3 * iters], st);
    return PSY_OK;
}

// Captures launch_wave on a private stream (thread-local capture mode, so
// other threads' CUDA calls are unaffected) and replays it on st.  The graph
// is re-captured when the launch configuration or the buffers change.
int launch_wave_graph(PsyScene *s, const WaveBufs &B, WaveGraph &G, const WaveDesc *d_wave, uint32_t max_paths,
                      uint32_t max_pix, cudaStream_t st) {
    WaveLaunchKey k{s->trace_mode, s->minb, s->sort_bits, s->prec, s->stack, s->grid, s->shade_minb,
                    s->resident_tail, max_paths, max_pix, d_wave, B.P.color};
    if (!G.valid || !(G.key == k)) {
        G.reset();
        cudaStream_t cs = nullptr;
        CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cs);
            return cuda_fail(e, "begin wave capture");
        }
        int r = launch_wave(s, B, d_wave, max_paths, max_pix, cs, nullptr, nullptr);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(cs, &graph);
        cudaStreamDestroy(cs);
        if (r != PSY_OK || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return r != PSY_OK ? r : cuda_fail(e, "end wave capture");
        }
        e = cudaGraphInstantiate(&G.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            G.exec = nullptr;
            return cuda_fail(e, "instantiate wave graph");
        }
        G.key = k;
        G.valid = true;
    }
    CK(cudaGraphLaunch(G.exec, st), "wave graph launch");
    return PSY_OK;
}

int alloc_wave_bufs(WaveBufs &B, uint32_t cap, uint32_t cap_waves, bool sorting, std::vector<void *> &allocs,
                    uint64_t &bytes) {
    B = WaveBufs{};
    size_t N = cap;
    cudaError_t e = cudaSuccess;
    auto al = [&](auto **p, size_t b) {
        if (e != cudaSuccess) return;
        void *q = nullptr;
        e = cudaMalloc(&q, b);
        if (e == cudaSuccess) {
            allocs.push_back(q);
            bytes += b;
            *p = reinterpret_cast<std::remove_pointer_t<decltype(p)>>(q);
        }
    };
    al(&B.P.color, N * 16); al(&B.P.latt, N * 16); al(&B.P.pending, N * 16); al(&B.P.nafac, N * 16);
    al(&B.P.nb_o, N * 16); al(&B.P.nb_d, N * 16); al(&B.P.tw, N * 8); al(&B.P.seed, N * 4); al(&B.P.flags, N * 4);
    al(&B.R.o, N * 16); al(&B.R.d, N * 16); al(&B.R.occl, N);
    al(&B.H.ki, N * 16); al(&B.H.tb, N * 16);
    al(&B.queue[0], N * 4); al(&B.queue[1], N * 4);
    unsigned char *ctrl = nullptr;
    al(&ctrl, 1024);
    if (sorting) {
        al(&B.stage, N * 4); al(&B.stage_key, N * 2); al(&B.bins, 65536 * 4);
        al(&B.qradix, queue_radix_words(cap) * 4);
    }
    al(&B.waves, (size_t)cap_waves * sizeof(WaveDesc));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc wave buffers");
    B.counts = reinterpret_cast<uint32_t *>(ctrl);
    B.work = reinterpret_cast<uint32_t *>(ctrl + 256);
    B.err = reinterpret_cast<int *>(ctrl + 512);
    CK(cudaMemset(ctrl, 0, 1024), "clear wave control block");
    B.cap = cap;
    B.cap_waves = cap_waves;
    return PSY_OK;
}

// Render h rows of w pixels from (x0, y0) of a cam_w x cam_h image -- image
// rows y0, y0 + ystep, ..., y0 + (h - 1) * ystep -- into d_xyz (row stride
// img_w): region row k, column x lands in out row orow + k, column x - ox.
// Waves of `rows` region rows each.
int render_region_core(PsyScene *s, const WaveBufs &B, uint32_t rows, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h,
                       uint32_t spp, uint32_t seed, float *d_xyz, uint32_t img_w, uint32_t ox, uint32_t orow,
                       uint32_t cam_w, uint32_t cam_h, cudaStream_t st, PsyRenderStats *stats, uint32_t ystep) {
    if (spp == 0 || w == 0 || h == 0) return PSY_OK;
    uint32_t iters = 2 * s->g.max_bounces + 3;
    bool timing = stats != nullptr;
    // one single-segment descriptor per wave, uploaded with one copy
    std::vector<WaveDesc> waves;
    for (uint32_t k = 0; k < h; k += rows) {
        WaveDesc d{};
        WaveSeg &g = d.seg[0];
        g.x0 = x0; g.y0 = y0 + k * ystep; g.w = w; g.h = std::min(rows, h - k);
        g.ystep = ystep;
        g.spp = spp; g.seed = seed;
        g.img_w = cam_w; g.img_h = cam_h;
        g.out = d_xyz; g.out_stride = img_w;
        g.out_x0 = ox; g.orow0 = orow + k;
        d.nseg = 1; d.npix = g.w * g.h; d.npaths = d.npix * spp;
        waves.push_back(d);
    }
    if (waves.size() > B.cap_waves) return fail(PSY_E_OVERFLOW, "too many waves for the descriptor buffer");
    CK(cudaMemcpyAsync(B.waves, waves.data(), waves.size() * sizeof(WaveDesc), cudaMemcpyHostToDevice, st),
       "upload wave descriptors");
    uint32_t max_paths = std::min<uint32_t>(rows, h) * w * spp;
    uint32_t max_pix = std::min<uint32_t>(rows, h) * w;
    // events: camera start/end, per iteration trace start/end + shade end, accumulate end
    std::vector<cudaEvent_t> ev;
    if (timing) {
        ev.resize(3 + 3 * iters);
        for (auto &e : ev) cudaEventCreate(&e);
        CK(cudaMemsetAsync(s->d_raycount, 0, 8, st), "memset");
    }
    unsigned long long *ctr = (s->counting && stats) ? s->d_counters : nullptr;
    double t_gen = 0, t_trace = 0, t_shade = 0, t_acc = 0;
    auto t0 = std::chrono::steady_clock::now();
    // CUDA graph replay needs a spare descriptor slot (the graph reads a fixed
    // address; each wave's descriptor is copied there first).  The
    // no-allocation entry point has none, so it never instantiates a graph.
    bool graph = s->use_graph && !timing && B.cap_waves > waves.size();
    WaveDesc *slot = B.waves + (B.cap_waves - 1);
    for (size_t i = 0; i < waves.size(); i++) {
        int r;
        if (graph) {
            CK(cudaMemcpyAsync(slot, B.waves + i, sizeof(WaveDesc), cudaMemcpyDeviceToDevice, st), "wave slot copy");
            r = launch_wave_graph(s, B, s->graph, slot, max_paths, max_pix, st);
        } else {
            r = launch_wave(s, B, B.waves + i, max_paths, max_pix, st, ctr, timing ? ev.data() : nullptr);
        }
        if (r != PSY_OK) return r;
        if (timing) {
            CK(launch_count_rays(B.P, waves[i].npaths, s->d_raycount, st), "count launch");
            CK(cudaEventSynchronize(ev[2 + 3 * iters]), "event sync");
            float ms;
            cudaEventElapsedTime(&ms, ev[0], ev[1]);
            t_gen += ms * 1e-3;
            for (uint32_t it = 0; it < iters; it++) {
                cudaEventElapsedTime(&ms, ev[2 + 3 * it], ev[3 + 3 * it]);
                t_trace += ms * 1e-3;
                cudaEventElapsedTime(&ms, ev[3 + 3 * it], ev[4 + 3 * it]);
                t_shade += ms * 1e-3;
            }
            cudaEventElapsedTime(&ms, ev[1 + 3 * iters], ev[2 + 3 * iters]);
            t_acc += ms * 1e-3;
            stats->samples += waves[i].npaths;
        }
    }
    if (timing) {
        unsigned long long rc = 0;
        CK(cudaMemcpyAsync(&rc, s->d_raycount, 8, cudaMemcpyDeviceToHost, st), "copy ray count");
        CK(cudaStreamSynchronize(st), "sync");
        stats->ray_count += rc;
        stats->initial_ray_generation_time += t_gen;
        stats->trace_time += t_trace;
        stats->ray_generation_time += t_shade;
        stats->sample_writing_time += t_acc;
        stats->total_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (auto &e : ev) cudaEventDestroy(e);
        s->rays_traced += rc;
    }
    return PSY_OK;
}


// Render with the scene's own wavefront buffers (allocated on first use,
// sized for waves of whole pixel rows up to wave_paths paths).
// Region (x0, y0, w, h) into d_xyz with row stride img_w, where image pixel
// (ox, oy) is d_xyz[0]; with ystep > 1 the region is the h rows y0,
// y0 + ystep, ... and out row k holds region row k (oy unused).
static int render_region(PsyScene *s, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h, uint32_t spp, uint32_t seed,
                         float *d_xyz, uint32_t img_w, uint32_t ox, uint32_t oy, cudaStream_t st,
                         PsyRenderStats *stats, uint32_t cam_w = 0, uint32_t cam_h = 0, uint32_t ystep = 1) {
    if (cam_w == 0) { cam_w = s->g.width; cam_h = s->g.height; }
    if (spp == 0 || w == 0 || h == 0) return PSY_OK;
    uint64_t row_paths = (uint64_t)w * spp;
    uint32_t rows = (uint32_t)std::max<uint64_t>(1, s->wave_paths / row_paths);
    rows = std::min(rows, h);
    uint64_t max_paths = (uint64_t)rows * row_paths;
    if (max_paths > 0xFFFFFFFFull) return fail(PSY_E_UNSUPPORTED, "wave too large");
    int r = ensure_render(s, (uint32_t)max_paths);
    if (r != PSY_OK) return r;
    if (s->counting && stats) {
        r = ensure_counters(s);
        if (r != PSY_OK) return r;
    }
    WaveBufs B;
    B.P = s->P; B.R = s->R; B.H = s->H;
    B.queue[0] = s->queue[0]; B.queue[1] = s->queue[1];
    B.counts = s->counts;
    B.work = s->d_work;
    B.err = s->d_err;
    B.stage = s->d_stage; B.stage_key = s->d_stage_key; B.bins = s->d_bins; B.qradix = s->d_qradix;
    B.cap = s->cap_paths;
    uint32_t nwaves = (h + rows - 1) / rows + 1;  // + the graph's descriptor slot
    if (nwaves > s->cap_waves) {
        s->graph.reset();
        if (s->d_waves) cudaFree(s->d_waves);
        s->d_waves = nullptr;
        s->cap_waves = 0;
        CK(cudaMalloc((void **)&s->d_waves, (size_t)nwaves * sizeof(WaveDesc)), "cudaMalloc wave descriptors");
        s->cap_waves = nwaves;
    }
    B.waves = s->d_waves;
    B.cap_waves = s->cap_waves;
    return render_region_core(s, B, rows, x0, y0, w, h, spp, seed, d_xyz, img_w, ox, ystep > 1 ? 0 : y0 - oy, cam_w,
                              cam_h, st, stats, ystep);
}


// ---------------------------------------------------------------- no-allocation bucket render
// Scratch of psy_render_bucket_noalloc: one file-scope device array, resident
// on every GPU that loads this library until the process exits.  Host code
// must not pass the symbol itself to a kernel (on the host it is only a
// stand-in); its device address comes from cudaGetSymbolAddress, taken once
// per device with that device current.
namespace {
constexpr size_t kNoallocAlign = 256;
constexpr size_t na_round(size_t b) { return (b + kNoallocAlign - 1) / kNoallocAlign * kNoallocAlign; }
constexpr size_t kNoallocPaths = PSY_NOALLOC_MAX_SAMPLES;
// path state (9 arrays), ray (3), hit (2), two queues, control block, wave descriptor
constexpr size_t kNoallocBytes = 6 * na_round(kNoallocPaths * 16) + na_round(kNoallocPaths * 8) +
                                 2 * na_round(kNoallocPaths * 4) + 2 * na_round(kNoallocPaths * 16) +
                                 na_round(kNoallocPaths) + 2 * na_round(kNoallocPaths * 16) +
                                 2 * na_round(kNoallocPaths * 4) + na_round(1024) + na_round(sizeof(WaveDesc));
}  // namespace
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

namespace {
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {nullptr};

// Device address of the scratch array on device `dev`, which must be the
// current device (set up on the first call per device).
int noalloc_base(int dev, unsigned char **out) {
    int cur = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (cur != dev) return fail(PSY_E_INVALID, "the scene's device is not the current device");
    if (dev < 0 || dev >= 64) return fail(PSY_E_UNSUPPORTED, "device index beyond 63");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_noalloc_ptr[dev]);
    return PSY_OK;
}
}  // namespace

extern "C" int psy_render_bucket_noalloc(PsyScene *s, const PsyBucket *b, uint32_t spp, uint32_t seed,
                                         float *d_xyz_out, void *stream) {
    if (!s || !b || !d_xyz_out) return fail(PSY_E_INVALID, "null argument");
    if (b->w == 0 || b->h == 0 || spp == 0) return fail(PSY_E_INVALID, "empty bucket or zero spp");
    if ((uint64_t)b->x + b->w > s->g.width || (uint64_t)b->y + b->h > s->g.height)
        return fail(PSY_E_INVALID, "bucket outside the image");
    uint64_t n = (uint64_t)b->w * b->h * spp;
    if (n > PSY_NOALLOC_MAX_SAMPLES)
        return fail(PSY_E_INVALID, "bucket too large for the no-allocation scratch: w*h*spp must be <= " +
                                       std::to_string(PSY_NOALLOC_MAX_SAMPLES));
    unsigned char *base = nullptr;
    int r = noalloc_base(s->device, &base);
    if (r != PSY_OK) return r;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += na_round(bytes);
        return p;
    };
    const size_t C = kNoallocPaths;
    WaveBufs B;
    B.P.color = (float4 *)take(C * 16); B.P.latt = (float4 *)take(C * 16); B.P.pending = (float4 *)take(C * 16);
    B.P.nafac = (float4 *)take(C * 16); B.P.nb_o = (float4 *)take(C * 16); B.P.nb_d = (float4 *)take(C * 16);
    B.P.tw = (float2 *)take(C * 8); B.P.seed = (uint32_t *)take(C * 4); B.P.flags = (uint32_t *)take(C * 4);
    B.R.o = (float4 *)take(C * 16); B.R.d = (float4 *)take(C * 16); B.R.occl = (uint8_t *)take(C);
    B.H.ki = (uint4 *)take(C * 16); B.H.tb = (float4 *)take(C * 16);
    B.queue[0] = (uint32_t *)take(C * 4); B.queue[1] = (uint32_t *)take(C * 4);
    unsigned char *ctrl = take(1024);
    B.counts = (uint32_t *)ctrl;            // [2]
    B.work = (uint32_t *)(ctrl + 256);      // persistent-kernel work counter
    B.err = (int *)(ctrl + 512);            // device error word
    B.stage = nullptr; B.stage_key = nullptr; B.bins = nullptr; B.qradix = nullptr;
    B.cap = (uint32_t)C;
    B.waves = (WaveDesc *)take(sizeof(WaveDesc));  // the bucket is one wave
    B.cap_waves = 1;
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    std::lock_guard<std::mutex> lk(s->mu);
    // every call shares the scratch: clear the control block (queue lengths,
    // work counter, error word); the camera kernel writes all path state
    CK(cudaMemsetAsync(ctrl, 0, 1024, st), "clear scratch control block");
    // the bucket's pixels land at (x - b.x, y - b.y) of the bucket-sized output
    int sort = s->sort_bits;
    s->sort_bits = 0;
    r = render_region_core(s, B, b->h, b->x, b->y, b->w, b->h, spp, seed, d_xyz_out, b->w, b->x, 0, s->g.width,
                           s->g.height, st, nullptr, 1);
    s->sort_bits = sort;
    if (r != PSY_OK) return r;
    int h = 0;
    CK(cudaMemcpyAsync(&h, B.err, sizeof(int), cudaMemcpyDeviceToHost, st), "read error word");
    CK(cudaStreamSynchronize(st), "stream sync");
    if (h != 0) return fail(h, "device reported error (traversal stack overflow)");
    return PSY_OK;
}

extern "C" {

int psy_render_image_device(PsyScene *s, const uint32_t *crop, float *d_xyz, void *stream, PsyRenderStats *stats) {
    if (!s || !d_xyz) return fail(PSY_E_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t W = s->g.width, H = s->g.height;
    uint32_t x0 = 0, y0 = 0, w = W, h = H;
    if (crop) {
        uint32_t x1 = std::min(crop[0], W - 1), y1 = std::min(crop[1], H - 1);
        uint32_t x2 = std::min(crop[2], W - 1), y2 = std::min(crop[3], H - 1);
        if (x2 < x1 || y2 < y1) return fail(PSY_E_INVALID, "empty crop");
        x0 = x1; y0 = y1; w = x2 - x1 + 1; h = y2 - y1 + 1;
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    int r = render_region(s, x0, y0, w, h, s->g.spp, s->g.seed, d_xyz, W, 0, 0, st, stats);
    if (r != PSY_OK) return r;
    if (stats) return check_err(s);
    return PSY_OK;
}

int psy_render_rows_device(PsyScene *s, uint32_t first_row, uint32_t row_step, float *d_xyz, void *stream,
                           PsyRenderStats *stats) {
    if (!s || !d_xyz || row_step == 0) return fail(PSY_E_INVALID, "null argument or zero row step");
    std::lock_guard<std::mutex> lk(s->mu);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    uint32_t W = s->g.width, H = s->g.height;
    if (first_row >= H) return PSY_OK;
    uint32_t n = (H - first_row + row_step - 1) / row_step;
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    int r = render_region(s, 0, first_row, W, n, s->g.spp, s->g.seed, d_xyz, W, 0, 0, st, stats, 0, 0, row_step);
    if (r != PSY_OK) return r;
    if (stats) return check_err(s);
    return PSY_OK;
}

int psy_render_image(PsyScene *s, const uint32_t *crop, float *xyz_out, PsyRenderStats *stats) {
    if (!s || !xyz_out) return fail(PSY_E_INVALID, "null argument");
    size_t bytes = (size_t)s->g.width * s->g.height * 3 * sizeof(float);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->cap_xyz < bytes) {
            if (s->d_xyz) cudaFree(s->d_xyz);
            s->d_xyz = nullptr;
            CK(cudaMalloc((void **)&s->d_xyz, bytes), "cudaMalloc image");
            s->cap_xyz = bytes;
        }
        CK(cudaMemsetAsync(s->d_xyz, 0, bytes, s->stream), "memset image");
    }
    int r = psy_render_image_device(s, crop, s->d_xyz, s->stream, stats);
    if (r != PSY_OK) return r;
    CK(cudaMemcpyAsync(xyz_out, s->d_xyz, bytes, cudaMemcpyDeviceToHost, s->stream), "copy image");
    CK(cudaStreamSynchronize(s->stream), "sync");
    return check_err(s);
}

int psy_render_bucket(PsyScene *s, const PsyBucket *b, uint32_t spp, uint32_t seed, float *xyz_out,
                      PsyRenderStats *stats) {
    if (!s || !b || !xyz_out) return fail(PSY_E_INVALID, "null argument");
    if (b->w == 0 || b->h == 0 || spp == 0) return fail(PSY_E_INVALID, "empty bucket or zero spp");
    if ((uint64_t)b->x + b->w > s->g.width || (uint64_t)b->y + b->h > s->g.height)
        return fail(PSY_E_INVALID, "bucket outside the image");
    std::lock_guard<std::mutex> lk(s->mu);
    size_t bytes = (size_t)b->w * b->h * 3 * sizeof(float);
    if (s->cap_xyz < bytes) {
        if (s->d_xyz) cudaFree(s->d_xyz);
        s->d_xyz = nullptr;
        CK(cudaMalloc((void **)&s->d_xyz, bytes), "cudaMalloc bucket");
        s->cap_xyz = bytes;
    }
    if (stats) std::memset(stats, 0, sizeof(*stats));
    // the bucket's pixels land at (x - b.x, y - b.y) of a bucket-sized buffer
    int r = render_region(s, b->x, b->y, b->w, b->h, spp, seed, s->d_xyz, b->w, b->x, b->y, s->stream, stats);
    if (r != PSY_OK) return r;
    CK(cudaMemcpyAsync(xyz_out, s->d_xyz, bytes, cudaMemcpyDeviceToHost, s->stream), "copy bucket");
    CK(cudaStreamSynchronize(s->stream), "sync");
    return check_err(s);
}

}  // extern "C"

// ---------------------------------------------------------------- autotuning
namespace {
struct TuneCfg {
    int trace_mode, minb, stack, grid, sort_bits;
    uint32_t wave_paths;
    bool graph;
    int shade_minb;
    int tail;
};
TuneCfg get_cfg(const PsyScene *s) {
    return {s->trace_mode, s->minb, s->stack, s->grid, s->sort_bits, s->wave_paths, s->use_graph, s->shade_minb,
            s->resident_tail};
}
void set_cfg(PsyScene *s, const TuneCfg &c) {
    s->trace_mode = c.trace_mode; s->minb = c.minb; s->stack = c.stack; s->grid = c.grid;
    s->shade_minb = c.shade_minb; s->resident_tail = c.tail;
    s->sort_bits = c.sort_bits; s->wave_paths = c.wave_paths;
    if (s->use_graph != c.graph) s->graph.reset();
    s->use_graph = c.graph;
}
}  // namespace

extern "C" int psy_autotune(PsyScene *s, const PsyTuneOptions *opts, PsyTuneResult *res) {
    if (!s || !res) return fail(PSY_E_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t probe = (opts && opts->probe_paths) ? opts->probe_paths : (1u << 24);
    uint32_t reps = (opts && opts->repeats) ? opts->repeats : 3;
    uint32_t W = s->g.width, H = s->g.height, spp = s->g.spp;
    if (W == 0 || H == 0 || spp == 0) return fail(PSY_E_INVALID, "scene has an empty image");
    uint64_t row = (uint64_t)W * spp;
    uint32_t rows = (uint32_t)std::min<uint64_t>(H, std::max<uint64_t>(1, probe / row));
    uint32_t y0 = (H - rows) / 2;
    float *d_img = nullptr;
    CK(cudaMalloc((void **)&d_img, (size_t)W * rows * 12), "cudaMalloc probe image");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaStream_t st = s->stream;
    uint32_t ncand = 0;
    int err = PSY_OK;
    // time one configuration: one untimed render, then the best of reps
    auto measure = [&](const TuneCfg &c, double &out) -> int {
        set_cfg(s, c);
        int r = render_region(s, 0, y0, W, rows, spp, s->g.seed, d_img, W, 0, y0, st, nullptr);
        if (r != PSY_OK) return r;
        double best = 1e30;
        for (uint32_t k = 0; k < reps; k++) {
            cudaEventRecord(e0, st);
            r = render_region(s, 0, y0, W, rows, spp, s->g.seed, d_img, W, 0, y0, st, nullptr);
            if (r != PSY_OK) return r;
            cudaEventRecord(e1, st);
            CK(cudaEventSynchronize(e1), "probe sync");
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            best = std::min(best, (double)ms * 1e-3);
        }
        ncand++;
        out = best;
        return check_err(s);
    };
    TuneCfg start = get_cfg(s), cur = start;
    double best = 0, t = 0;
    err = measure(cur, best);
    double default_s = best;
    // the fastest candidate of a set replaces the current choice when it
    // beats it by 2%: differences inside the run-to-run noise keep the
    // earlier (simpler) choice, and the order of the set does not matter
    auto try_set = [&](std::vector<TuneCfg> cands) {
        double set_best = best;
        TuneCfg set_cfg_best = cur;
        for (const TuneCfg &c : cands) {
            if (err != PSY_OK) return;
            err = measure(c, t);
            if (err == PSY_OK && t < set_best) {
                set_best = t;
                set_cfg_best = c;
            }
        }
        if (err == PSY_OK && set_best < 0.98 * best) {
            best = set_best;
            cur = set_cfg_best;
        }
    };
    // 1. trace kernel and register budget
    {
        std::vector<TuneCfg> v;
        for (int m : {4, 5, 6, 8}) { TuneCfg c = cur; c.trace_mode = 0; c.minb = m; v.push_back(c); }
        for (int m : {4, 6, 8}) { TuneCfg c = cur; c.trace_mode = 1; c.minb = m; v.push_back(c); }
        if (s->g.static_fast) {  // the static-scene traversal, and its lane-refill form
            for (int m : {8, 10, 12}) { TuneCfg c = cur; c.trace_mode = 3; c.minb = m; v.push_back(c); }
            TuneCfg c = cur; c.trace_mode = 5; c.minb = 10; v.push_back(c);
        }
        // warp packets (trace mode 2) are not tried: 2-7x slower on every
        // measured workload, as one-thread-per-ray keeps more rays in flight
        try_set(v);
    }
    // 1b. shading kernel register budget
    {
        std::vector<TuneCfg> v;
        for (int m : {6, 8}) { TuneCfg c = cur; c.shade_minb = m; v.push_back(c); }
        try_set(v);
    }
    // 2. stack depth: the fitting variant and the larger ones
    {
        std::vector<TuneCfg> v;
        for (int k : {64, 192})
            if ((uint32_t)k >= s->max_stack && k != cur.stack) { TuneCfg c = cur; c.stack = k; v.push_back(c); }
        try_set(v);
    }
    // 3. queue tile: grid of the wavefront kernels
    {
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        std::vector<TuneCfg> v;
        for (int k : {0, 8, 16, 32}) { TuneCfg c = cur; c.grid = k * sms; if (c.grid != cur.grid) v.push_back(c); }
        if (cur.grid != PSY_GRID_RESIDENT) { TuneCfg c = cur; c.grid = PSY_GRID_RESIDENT; v.push_back(c); }
        try_set(v);
    }
    // 3b. resident grids for the last iterations of a wave only (their
    //     queues hold few paths; a grid sized by the wave spends ~0.5 ms per
    //     launch scheduling blocks that find nothing to do)
    {
        const int iters = 2 * (int)s->g.max_bounces + 3;
        std::vector<TuneCfg> v;
        for (int k : {4, 6, 8, 10})
            if (k < iters && k != cur.tail && cur.grid != PSY_GRID_RESIDENT) { TuneCfg c = cur; c.tail = k; v.push_back(c); }
        try_set(v);
    }
    // 4. ray-sort key width
    {
        std::vector<TuneCfg> v;
        for (int b : {0, 4, 10, 13, 16, 19, 25}) { TuneCfg c = cur; c.sort_bits = b; if (b != cur.sort_bits) v.push_back(c); }
        try_set(v);
    }
    // 5. wave size
    {
        std::vector<TuneCfg> v;
        for (uint32_t w : {1u << 21, 1u << 22, 1u << 23, 1u << 24}) {
            TuneCfg c = cur; c.wave_paths = w;
            if (w != cur.wave_paths) v.push_back(c);
        }
        try_set(v);
    }
    // 6. CUDA graph replay of each wave
    {
        TuneCfg c = cur; c.graph = !cur.graph;
        try_set({c});
    }
    // 7. waves beyond the probe band, timed on the whole image: a larger
    //    wave pays the late, sparsely filled iterations once for more paths
    //    (mesh-stress frame: 16M -> 128M paths per wave, 447 -> 483 M
    //    samples/s).  Sizes whose wave buffers fit in the buffers already
    //    held plus a quarter of the free device memory (or the caller's
    //    max_wave_mib); a candidate that cannot allocate ends the step.
    if (err == PSY_OK) {
        const uint64_t kBytesPerPath = 224;  // ensure_render's buffers per path (185-207 bytes), rounded up
        uint64_t img = (uint64_t)W * H * spp;
        size_t fb = 0, tb = 0;
        cudaMemGetInfo(&fb, &tb);
        uint64_t budget = (uint64_t)s->cap_paths * kBytesPerPath + fb / 4;
        if (opts && opts->max_wave_mib) budget = std::min<uint64_t>(budget, (uint64_t)opts->max_wave_mib << 20);
        std::vector<uint64_t> sizes;
        for (uint64_t w : {(uint64_t)cur.wave_paths * 2, (uint64_t)cur.wave_paths * 4, img})
            if (w > cur.wave_paths && w <= img && w * kBytesPerPath <= budget && w <= 0xFFFFFFFFull &&
                (sizes.empty() || w > sizes.back()))
                sizes.push_back(w);
        float *d_full = nullptr;
        if (!sizes.empty() && cudaMalloc((void **)&d_full, (size_t)W * H * 12) == cudaSuccess) {
            auto measure_full = [&](const TuneCfg &c, double &out) -> int {
                set_cfg(s, c);
                int r = render_region(s, 0, 0, W, H, spp, s->g.seed, d_full, W, 0, 0, st, nullptr);
                if (r != PSY_OK) return r;
                double best_t = 1e30;
                for (uint32_t k = 0; k < 2; k++) {
                    cudaEventRecord(e0, st);
                    r = render_region(s, 0, 0, W, H, spp, s->g.seed, d_full, W, 0, 0, st, nullptr);
                    if (r != PSY_OK) return r;
                    cudaEventRecord(e1, st);
                    CK(cudaEventSynchronize(e1), "probe sync");
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    best_t = std::min(best_t, (double)ms * 1e-3);
                }
                out = best_t;
                return PSY_OK;
            };
            double base_t = 0.0;
            if (measure_full(cur, base_t) == PSY_OK) {
                ncand++;
                // the fastest candidate, if it beats the starting point by 2%
                TuneCfg best_c = cur, fastest_c = cur;
                double best_t = base_t, fastest_t = base_t;
                for (uint64_t w : sizes) {
                    TuneCfg c = cur;
                    c.wave_paths = (uint32_t)w;
                    double t = 0.0;
                    int r = measure_full(c, t);
                    ncand++;
                    if (r != PSY_OK) {  // did not fit after all: keep what was measured
                        cudaGetLastError();
                        break;
                    }
                    if (t < fastest_t) {
                        fastest_t = t;
                        fastest_c = c;
                    }
                }
                if (fastest_t < 0.98 * base_t) {
                    best_t = fastest_t;
                    best_c = fastest_c;
                }
                // with a larger wave, the grid of the wavefront kernels and
                // the queue-ordering key again, on the whole image: a grid
                // sized by a huge wave spends ~0.5 ms per launch scheduling
                // blocks that find the late queues empty, and a wave of the
                // whole frame repays a wider key (mesh stress, one wave:
                // 13 bits 484, 19 bits 495 M samples/s)
                if (best_c.wave_paths != cur.wave_paths) {
                    int dev = 0, sms = 152;
                    cudaGetDevice(&dev);
                    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                    auto recheck = [&](const std::vector<TuneCfg> &cands) {
                        TuneCfg set_c = best_c;
                        double set_t = best_t;
                        for (const TuneCfg &c : cands) {
                            double t = 0.0;
                            int r = measure_full(c, t);
                            ncand++;
                            if (r != PSY_OK) {
                                cudaGetLastError();
                                break;
                            }
                            if (t < set_t) {
                                set_t = t;
                                set_c = c;
                            }
                        }
                        if (set_t < 0.98 * best_t) {
                            best_t = set_t;
                            best_c = set_c;
                        }
                    };
                    std::vector<TuneCfg> grids, keys;
                    for (int k : {-1, 0, 16, 32, 64}) {
                        TuneCfg c = best_c;
                        c.grid = k < 0 ? PSY_GRID_RESIDENT : k * sms;
                        if (c.grid != best_c.grid) grids.push_back(c);
                    }
                    recheck(grids);
                    std::vector<TuneCfg> tails;
                    for (int k : {0, 4, 6, 8, 10}) {
                        TuneCfg c = best_c;
                        c.tail = k;
                        if (k < 2 * (int)s->g.max_bounces + 3 && k != best_c.tail && c.grid != PSY_GRID_RESIDENT)
                            tails.push_back(c);
                    }
                    recheck(tails);
                    for (int b : {10, 13, 16, 19, 25}) {
                        TuneCfg c = best_c;
                        c.sort_bits = b;
                        if (b != best_c.sort_bits) keys.push_back(c);
                    }
                    recheck(keys);
                }
                cur = best_c;
            } else {
                cudaGetLastError();
            }
            cudaFree(d_full);
            set_cfg(s, cur);
            // release wave buffers larger than the chosen waves need
            uint64_t need = std::min<uint64_t>(img, (uint64_t)std::max<uint64_t>(1, cur.wave_paths / ((uint64_t)W * spp)) *
                                                        (uint64_t)W * spp);
            if ((uint64_t)s->cap_paths > need) free_render(s);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_img);
    if (err != PSY_OK) {
        set_cfg(s, start);
        return err;
    }
    set_cfg(s, cur);
    res->trace_mode = (uint32_t)cur.trace_mode;
    res->minb = (uint32_t)cur.minb;
    res->stack = (uint32_t)cur.stack;
    res->grid = (uint32_t)cur.grid;
    res->sort_bits = (uint32_t)cur.sort_bits;
    res->wave_paths = cur.wave_paths;
    res->use_graph = cur.graph ? 1u : 0u;
    res->shade_minb = (uint32_t)cur.shade_minb;
    res->resident_tail = (uint32_t)cur.tail;
    res->candidates = ncand;
    res->default_s = default_s;
    res->best_s = best;
    return PSY_OK;
}

extern "C" {

// ---------------------------------------------------------------- image output
// XYZ image -> sRGB RGBA8 as Image::write_png converts it (src/image.rs:138-164).
int psy_xyz_to_srgb8(const float *d_xyz, uint32_t width, uint32_t height, uint8_t *d_rgba, void *stream) {
    if (!d_xyz || !d_rgba) return fail(PSY_E_INVALID, "null argument");
    if ((uint64_t)width * height > 0xFFFFFFFFull) return fail(PSY_E_INVALID, "image too large");
    static Mat3f m = [] {
        Mat3f r;
        xyz_to_rec709_e_matrix(r.m);
        return r;
    }();
    CK(launch_xyz_to_srgb8(d_xyz, width, height, m, d_rgba, (cudaStream_t)stream), "srgb conversion");
    return PSY_OK;
}

// ---------------------------------------------------------------- inspection
// Not part of the reference-facing interface: facts of the build for tests.
int psy_debug_mesh_bvh_info(PsyScene *s, uint32_t object, uint32_t *tri_order, uint32_t *node_count) {
    if (!s || object >= s->object_to_mesh.size() || s->object_to_mesh[object] < 0) return fail(PSY_E_INVALID, "not a mesh");
    int m = s->object_to_mesh[object];
    if (tri_order) std::memcpy(tri_order, s->mesh_tri_order[m].data(), s->mesh_tri_order[m].size() * 4);
    if (node_count) *node_count = s->mesh_node_count[m];
    return PSY_OK;
}
// Host-side only (no device): the traversal table as the device holds it and
// the push tables of the static-scene traversal.
int psy_debug_push_tables(uint8_t *table, uint8_t *rows, uint16_t *lut) {
    if (!table || !rows || !lut) return fail(PSY_E_INVALID, "null argument");
    psy_traversal_table_device(reinterpret_cast<uint8_t(*)[48]>(table));
    if (!psy_push_tables_host(reinterpret_cast<uint8_t(*)[48]>(rows), reinterpret_cast<uint16_t(*)[16]>(lut)))
        return fail(PSY_E_INVALID, "push tables need more rows");
    return PSY_OK;
}
// Host-side build only (no device): BVH facts of a mesh object.
int psy_debug_host_build(const PsySceneDesc *desc, const PsySceneOptions *opts, uint32_t object, uint32_t *tri_order,
                         uint32_t *node_count, uint32_t *max_stack) {
    HostScene hs;
    std::string err;
    int rc = build_host_scene(desc, opts, hs, err);
    if (rc != PSY_OK) return fail(rc, err);
    if (max_stack) *max_stack = hs.max_stack;
    if (object >= hs.object_to_mesh.size() || hs.object_to_mesh[object] < 0) return PSY_OK;
    int m = hs.object_to_mesh[object];
    if (tri_order) std::memcpy(tri_order, hs.mesh_tri_order[m].data(), hs.mesh_tri_order[m].size() * 4);
    if (node_count) *node_count = hs.mesh_node_count[m];
    return PSY_OK;
}
// Host-side build only (no device): the whole scene's BVH4 nodes (128 bytes
// each) and motion bounds (96 bytes per key), built with worker threads or
// on one thread.  With null arrays only the counts are returned.
int psy_debug_host_nodes(const PsySceneDesc *desc, const PsySceneOptions *opts, int serial, void *nodes,
                         uint32_t *node_count, void *bounds_ext, uint32_t *ext_count) {
    HostScene hs;
    std::string err;
    int rc = build_host_scene(desc, opts, hs, err, nullptr, serial != 0);
    if (rc != PSY_OK) return fail(rc, err);
    if (node_count) *node_count = (uint32_t)hs.nodes.size();
    if (ext_count) *ext_count = (uint32_t)hs.bounds_ext.size();
    if (nodes) std::memcpy(nodes, hs.nodes.data(), hs.nodes.size() * sizeof(GNode));
    if (bounds_ext) std::memcpy(bounds_ext, hs.bounds_ext.data(), hs.bounds_ext.size() * sizeof(GBounds4));
    return PSY_OK;
}
int psy_debug_host_nodes_h(const PsySceneDesc *desc, const PsySceneOptions *opts, void *nodes_h,
                           uint32_t *node_count) {
    HostScene hs;
    std::string err;
    int rc = build_host_scene(desc, opts, hs, err, nullptr, false);
    if (rc != PSY_OK) return fail(rc, err);
    if (node_count) *node_count = (uint32_t)hs.nodes_h.size();
    if (nodes_h) std::memcpy(nodes_h, hs.nodes_h.data(), hs.nodes_h.size() * sizeof(GNodeH));
    return PSY_OK;
}
int psy_debug_scene_info(PsyScene *s, uint32_t *max_stack, uint32_t *nodes, uint32_t *stack_variant) {
    if (!s) return fail(PSY_E_INVALID, "null");
    if (max_stack) *max_stack = s->max_stack;
    if (nodes) *nodes = s->node_count;
    if (stack_variant) *stack_variant = (uint32_t)s->stack;
    return PSY_OK;
}
// Scene facts the kernel choice depends on: bit 0 = the static-scene
// traversal applies, bit 1 = ordered child boxes, bit 2 = FP16 bounds.
int psy_debug_scene_flags(PsyScene *s, uint32_t *flags) {
    if (!s || !flags) return fail(PSY_E_INVALID, "null");
    *flags = (s->g.static_fast ? 1u : 0u) | (s->g.ordered_slabs ? 2u : 0u) | (s->g.use_fp16 ? 4u : 0u);
    return PSY_OK;
}
// Traversal counters of renders: enable (and zero) or read them.
int psy_debug_counters(PsyScene *s, int enable, uint64_t *nodes, uint64_t *tris, uint64_t *rays) {
    if (!s) return fail(PSY_E_INVALID, "null");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->d_counters) {
        unsigned long long h[3] = {0, 0, 0};
        CK(cudaMemcpyAsync(h, s->d_counters, sizeof(h), cudaMemcpyDeviceToHost, s->stream), "copy counters");
        CK(cudaStreamSynchronize(s->stream), "sync");
        if (nodes) *nodes = h[0];
        if (tris) *tris = h[1];
        if (rays) *rays = h[2];
        CK(cudaMemsetAsync(s->d_counters, 0, sizeof(h), s->stream), "memset counters");
    } else {
        if (nodes) *nodes = 0;
        if (tris) *tris = 0;
        if (rays) *rays = 0;
    }
    s->counting = enable != 0;
    return PSY_OK;
}
// Traversal kernel choice: mode 0 = one thread per ray, 1 = persistent with
// lane refill, 2 = warp packets, 3 = the static-scene traversal (one thread
// per ray; scenes without it fall back to mode 0's kernels), 4 = its
// speculative form; minb = resident blocks per SM the register budget
// targets.
int psy_debug_set_trace(PsyScene *s, int mode, int minb) {
    if (!s || mode < 0 || mode > 5) return fail(PSY_E_INVALID, "bad trace mode");
    s->trace_mode = mode;
    // persistent kernel: 4, 6 or 8 blocks per SM; one thread per ray: 4, 5,
    // 6 or 8; static-scene traversal: 6, 8, 10 or 12 (its lane-refill form,
    // mode 5, always 10)
    if (mode == 1) s->minb = minb >= 8 ? 8 : (minb >= 6 ? 6 : 4);
    else if (mode >= 3) s->minb = minb >= 12 ? 12 : (minb >= 10 ? 10 : (minb >= 8 ? 8 : 6));
    else s->minb = minb >= 8 ? 8 : (minb >= 6 ? 6 : (minb == 5 ? 5 : 4));
    return PSY_OK;
}
// Shading kernel register budget: 4 (f32 form: 128 registers; f64 form: the
// compiler's choice), 6 or 8 blocks per SM.
int psy_debug_set_shade(PsyScene *s, int minb) {
    if (!s || !(minb == 4 || minb == 6 || minb == 8)) return fail(PSY_E_INVALID, "bad shade budget");
    s->shade_minb = minb;
    return PSY_OK;
}
// Queue binning key width between wavefront iterations: 0 (off), 4, 10, 13, 16
// (counting sort), 19, 25, 31 (two-point keys, radix sort).
int psy_debug_set_sort(PsyScene *s, int bits) {
    if (!s || !(bits == 0 || bits == 4 || bits == 10 || bits == 13 || bits == 16 || bits == 19 || bits == 25 ||
                bits == 31))
        return fail(PSY_E_INVALID, "bad sort bits");
    s->sort_bits = bits;
    return PSY_OK;
}
int psy_debug_set_launch(PsyScene *s, int grid, uint32_t wave_paths) {
    if (!s) return fail(PSY_E_INVALID, "null");
    s->grid = grid;
    if (wave_paths >= 1024) s->wave_paths = wave_paths;
    return PSY_OK;
}
int psy_debug_color_spectra(PsyScene *s, uint32_t n, const float *d_hero, float *d_exact, float *d_table,
                            uint32_t *n_colors) {
    if (!s || !n_colors) return fail(PSY_E_INVALID, "null");
    *n_colors = s->n_spec;
    if (n == 0 || s->n_spec == 0) return PSY_OK;
    if (!d_hero || !d_exact || !d_table) return fail(PSY_E_INVALID, "null");
    std::lock_guard<std::mutex> lk(s->mu);
    CK(launch_debug_color_spectra(s->g, s->d_spec_xyz, s->n_spec, d_hero, n, d_exact, d_table, s->stream),
       "color spectra launch");
    CK(cudaStreamSynchronize(s->stream), "sync");
    return PSY_OK;
}
int psy_debug_set_resident_tail(PsyScene *s, int iterations) {
    if (!s || iterations < 0) return fail(PSY_E_INVALID, "invalid argument");
    s->resident_tail = iterations;
    return PSY_OK;
}
// Render a whole width x height image with spp samples and seed through the
// scene's camera (a resolution other than the scene's own) into the device
// buffer d_xyz; returns when done.  The one-request-at-a-time form of what
// the render server does.
int psy_debug_render_sized(PsyScene *s, uint32_t width, uint32_t height, uint32_t spp, uint32_t seed, float *d_xyz,
                           void *stream) {
    if (!s || !d_xyz || width == 0 || height == 0 || spp == 0) return fail(PSY_E_INVALID, "invalid argument");
    std::lock_guard<std::mutex> lk(s->mu);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    int r = render_region(s, 0, 0, width, height, spp, seed, d_xyz, width, 0, 0, st, nullptr, width, height);
    if (r != PSY_OK) return r;
    CK(cudaStreamSynchronize(st), "sync");
    return check_err(s);
}
// Ray order of trace calls: 0 = as given, 1 = binned (PsySceneOptions.ray_order).
int psy_debug_set_ray_order(PsyScene *s, int order) {
    if (!s || order < 0 || order > 1) return fail(PSY_E_INVALID, "bad ray order");
    s->ray_order = order;
    return PSY_OK;
}
// The ray order of a trace call of n device rays: d_keys receives the
// sorted two-point keys, d_order the ray index at each position.
int psy_debug_ray_order(PsyScene *s, const PsyRay *d_rays, uint32_t n, uint32_t *d_keys, uint32_t *d_order,
                        void *stream) {
    if (!s || (n && (!d_rays || !d_keys || !d_order))) return fail(PSY_E_INVALID, "null argument");
    if (n == 0) return PSY_OK;
    std::lock_guard<std::mutex> lk(s->mu);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    int r = ensure_binning(s, n);
    if (r != PSY_OK) return r;
    uint32_t *b = s->d_border;
    RayOrderBufs rb{b, b + n, b + 2 * (size_t)n, b + 3 * (size_t)n, b + 4 * (size_t)n};
    const uint32_t *order = nullptr;
    CK(launch_ray_order(s->g, d_rays, n, rb, &order, st), "ray order");
    const uint32_t *keys = order == rb.vals ? rb.keys : rb.keys2;
    CK(cudaMemcpyAsync(d_keys, keys, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st), "copy keys");
    CK(cudaMemcpyAsync(d_order, order, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st), "copy order");
    CK(cudaStreamSynchronize(st), "ray order");
    return PSY_OK;
}
// Replay each wave from a CUDA graph (1) or launch it kernel by kernel (0).
int psy_debug_set_graph(PsyScene *s, int on) {
    if (!s) return fail(PSY_E_INVALID, "null");
    std::lock_guard<std::mutex> lk(s->mu);
    s->use_graph = on != 0;
    if (!s->use_graph) s->graph.reset();
    return PSY_OK;
}
// One bucket as one wave; every path's final colour and hero wavelength.
int psy_debug_render_paths(PsyScene *s, const PsyBucket *b, uint32_t spp, uint32_t seed, float *color4,
                           float *wavelength) {
    if (!s || !b || !color4) return fail(PSY_E_INVALID, "null argument");
    if (b->w == 0 || b->h == 0 || spp == 0) return fail(PSY_E_INVALID, "empty bucket or zero spp");
    if ((uint64_t)b->x + b->w > s->g.width || (uint64_t)b->y + b->h > s->g.height)
        return fail(PSY_E_INVALID, "bucket outside the image");
    uint64_t n = (uint64_t)b->w * b->h * spp;
    if (n > (1u << 20)) return fail(PSY_E_INVALID, "at most 1,048,576 samples");
    std::lock_guard<std::mutex> lk(s->mu);
    size_t bytes = (size_t)b->w * b->h * 3 * sizeof(float);
    if (s->cap_xyz < bytes) {
        if (s->d_xyz) cudaFree(s->d_xyz);
        s->d_xyz = nullptr;
        CK(cudaMalloc((void **)&s->d_xyz, bytes), "cudaMalloc bucket");
        s->cap_xyz = bytes;
    }
    uint32_t wave = s->wave_paths;
    s->wave_paths = std::max<uint32_t>(wave, (uint32_t)n);  // the whole bucket in one wave
    int r = render_region(s, b->x, b->y, b->w, b->h, spp, seed, s->d_xyz, b->w, b->x, b->y, s->stream, nullptr);
    s->wave_paths = wave;
    if (r != PSY_OK) return r;
    std::vector<float2> tw(n);
    CK(cudaMemcpyAsync(color4, s->P.color, n * sizeof(float4), cudaMemcpyDeviceToHost, s->stream), "copy colours");
    CK(cudaMemcpyAsync(tw.data(), s->P.tw, n * sizeof(float2), cudaMemcpyDeviceToHost, s->stream), "copy wavelengths");
    CK(cudaStreamSynchronize(s->stream), "sync");
    if (wavelength)
        for (size_t i = 0; i < n; i++) wavelength[i] = tw[i].y;
    return check_err(s);
}
// Sampler values on the device (ops in psy_debug.h).
int psy_debug_samplers(int op, const uint32_t *d_args, uint32_t n, uint32_t *d_out, void *stream) {
    if (op < 0 || op > 4) return fail(PSY_E_INVALID, "bad sampler op");
    if (n && (!d_args || !d_out)) return fail(PSY_E_INVALID, "null argument");
    upload_device_constants();  // the Sobol direction numbers
    cudaStream_t st = (cudaStream_t)stream;
    CK(launch_debug_samplers(op, d_args, n, d_out, st), "sampler kernel");
    CK(cudaStreamSynchronize(st), "sync");
    return PSY_OK;
}

}  // extern "C"
