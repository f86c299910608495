// Internal definitions shared by the C ABI translation units (capi.cu,
// server.cu): the scene handle, error reporting and the wave launcher.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"

// Sets the calling thread's last error message and returns code.
int psy_fail(int code, const std::string &msg);
// Same for a CUDA error (PSY_E_NOMEM for allocation failures, else PSY_E_CUDA).
int psy_cuda_fail(cudaError_t e, const char *what);

// Launch configuration of the wave sequence; the fields a captured CUDA graph
// depends on.
struct WaveLaunchKey {
    int trace_mode, minb, sort_bits, prec, stack, grid, shade_minb, tail;
    uint32_t max_paths, max_pix;
    const WaveDesc *d_wave;
    const void *bufs;  // identity of the WaveBufs (its path-state base)
    bool operator==(const WaveLaunchKey &o) const {
        return trace_mode == o.trace_mode && minb == o.minb && sort_bits == o.sort_bits && prec == o.prec &&
               shade_minb == o.shade_minb && tail == o.tail &&
               stack == o.stack && grid == o.grid && max_paths == o.max_paths && max_pix == o.max_pix &&
               d_wave == o.d_wave && bufs == o.bufs;
    }
};
// One wave's launch sequence captured as a CUDA graph (re-captured when the
// scene's launch configuration or the buffers change).
struct WaveGraph {
    cudaGraphExec_t exec = nullptr;
    WaveLaunchKey key{};
    bool valid = false;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        valid = false;
    }
};

struct PsyScene {
    GScene g{};
    int device = 0;                      // the device current at psy_scene_create (holds all scene memory)
    std::vector<void *> allocs;
    uint64_t device_bytes = 0;
    cudaStream_t stream = nullptr;
    int *d_err = nullptr;
    uint64_t rays_traced = 0;
    int stack = 64;
    // per-scene facts kept for debugging / tree checks
    std::vector<std::vector<uint32_t>> mesh_tri_order;
    std::vector<uint32_t> mesh_node_count;
    std::vector<int32_t> object_to_mesh;
    uint32_t max_stack = 0;
    uint32_t node_count = 0;
    // trace scratch (host-buffer calls)
    PsyRay *d_rays = nullptr;
    PsyHit *d_hits = nullptr;
    PsySurfaceHit *d_full = nullptr;
    size_t cap_rays = 0;
    // render scratch
    uint32_t cap_paths = 0;
    PathState P{};
    RayBuf R{};
    HitBuf H{};
    uint32_t *queue[2] = {nullptr, nullptr};
    uint32_t *counts = nullptr;          // [2]
    unsigned long long *d_raycount = nullptr;
    float *d_xyz = nullptr;
    size_t cap_xyz = 0;
    uint32_t wave_paths = 1u << 24;      // paths per wave
    int grid = 0;                        // grid of the queue kernels (0: size by queue, -1: resident)
    int resident_tail = 0;               // the last n iterations of a wave launch on resident grids
    const float4 *d_spec_xyz = nullptr;  // XYZ of each colour with a spectrum table
    uint32_t n_spec = 0;
    bool counting = false;               // accumulate traversal counters during renders
    int trace_mode = 0;                  // 0: one thread per ray, 1: persistent with lane refill, 2: warp packets
    int prec = 0;                        // shading arithmetic: 0 f64 (reference), 1 f32
    int sort_bits = 0;                   // ray binning key width between iterations (0: off)
    uint32_t *d_stage = nullptr;         // binning staging queue
    uint16_t *d_stage_key = nullptr;
    uint32_t *d_bins = nullptr;
    uint32_t *d_qradix = nullptr;        // radix queue ordering scratch (queue_radix_words)
    WaveDesc *d_waves = nullptr;         // wave descriptors of one render call
    uint32_t cap_waves = 0;
    int minb = 4;                        // trace kernel register budget (target resident blocks per SM)
    int shade_minb = 4;                  // shading kernel register budget
    uint32_t *d_work = nullptr;          // work counter of the persistent kernels
    unsigned long long *d_counters = nullptr;  // node visits, triangle tests, rays
    bool use_graph = false;              // replay each wave's launch sequence from a CUDA graph
    int ray_order = 0;                   // trace calls: 1 = bin rays by octant and origin cell first
    uint32_t *d_border = nullptr;  // ray order scratch of trace calls: keys, order, second buffers, sort scratch
    size_t cap_bin = 0;
    WaveGraph graph;                     // graph of the scene's own render buffers
    std::mutex mu;
};

// The launch sequence of one wave on stream st (see capi.cu).
int launch_wave(PsyScene *s, const WaveBufs &B, const WaveDesc *d_wave, uint32_t max_paths, uint32_t max_pix,
                cudaStream_t st, unsigned long long *ctr, const cudaEvent_t *ev);
// Same through a CUDA graph of the sequence (captured on first use).
int launch_wave_graph(PsyScene *s, const WaveBufs &B, WaveGraph &G, const WaveDesc *d_wave, uint32_t max_paths,
                      uint32_t max_pix, cudaStream_t st);
// Allocates wave buffers for cap paths and cap_waves descriptors; adds the
// allocations to `allocs` and their size to `bytes`.
int alloc_wave_bufs(WaveBufs &B, uint32_t cap, uint32_t cap_waves, bool sorting, std::vector<void *> &allocs,
                    uint64_t &bytes);
