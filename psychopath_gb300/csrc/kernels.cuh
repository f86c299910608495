// Kernel interfaces of the tracing path (host-visible launch helpers).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/psy_gpu.h"
#include "psy_layout.h"

// Wavefront path state, structure of arrays (one entry per path = one
// (pixel, sample) of the wave).  Mirrors LightPath (src/renderer.rs:370-388).
struct PathState {
    float4 *color;    // accumulated path colour (4 hero wavelengths)
    float4 *latt;     // light_attenuation (times next_attenuation_fac once a bounce is set up)
    float4 *pending;  // pending_color_addition
    float4 *nafac;    // next_attenuation_fac of the last bounce sample that succeeded
    float4 *nb_o;     // next bounce ray origin, w = closure_sample_pdf
    float4 *nb_d;     // next bounce ray direction, w unused
    float2 *tw;       // (time, wavelength)
    uint32_t *seed;   // sampling_seed
    uint32_t *flags;  // event (bits 0-1) | bounce_count << 2 (8 bits) | has_next_bounce << 10 | rays << 16
};
struct RayBuf {
    float4 *o;        // origin xyz, max_t
    float4 *d;        // direction xyz, time
    uint8_t *occl;    // occlusion flag
};
struct HitBuf {
    uint4 *ki;        // kind, prim, slot, 0
    float4 *tb;       // t, b0, b1, b2
};
// One wave of the wavefront renderer: up to PSY_WAVE_MAX_SEGS segments, each
// a rectangle of pixels of some image rendered with all its spp samples.
// Segments may belong to different requests (different resolution, spp and
// seed) that share the wave's queues.  Paths of a segment are numbered
// pixel-major (all samples of a pixel are consecutive).
#define PSY_WAVE_MAX_SEGS 16
struct WaveSeg {
    uint32_t x0, y0, w, h;  // pixel rectangle in the segment's image
    uint32_t spp, seed;
    uint32_t img_w, img_h;  // resolution the camera maps (the request's image)
    float *out;             // XYZ buffer of the segment's pixels
    uint32_t out_stride;    // row stride of `out` in pixels
    uint32_t path_begin;    // first path of the segment in the wave
    uint32_t pix_begin;     // first pixel of the segment in the wave
    uint32_t out_x0;        // out column of image column x: x - out_x0
    uint32_t orow0;         // out row of the segment's first row
    uint32_t ystep;         // image rows of the segment: y0, y0 + ystep, ... (h rows)
};
struct WaveDesc {
    uint32_t nseg, npaths, npix, pad;
    WaveSeg seg[PSY_WAVE_MAX_SEGS];
};

void psy_upload_constants();  // Sobol nibble tables, traversal and push tables
// The traversal table as the device holds it (positions past a node's child
// count name its empty slots).
void psy_traversal_table_device(uint8_t t[8][48]);
// Push tables of the static-scene traversal built from that table (false:
// more distinct rows than the device table holds).
bool psy_push_tables_host(uint8_t rows[8][48], uint16_t lut[32][16]);
// True once the traversal kernels' push tables are on the device.
bool psy_trace_tables_ready();
// The traversal translation unit's own copies of its constants (null: skip).
void psy_upload_trace_constants(const uint8_t table[8][48], const float magenta[3]);

// Trace n PsyRay records (device) into PsyHit records (device).
// minb: resident blocks of 128 threads per SM the register budget targets
// (4 = the compiler's choice, 5 or 6 = fewer registers, some spills).
// order (optional): thread q traces ray order[q] (hits still land at the
// ray's own index).  fast: as for launch_trace_queue.
cudaError_t launch_trace_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order, PsyHit *hits,
                              PsySurfaceHit *full, int stack, int minb, int *d_err, unsigned long long *counters,
                              cudaStream_t st, int fast = 0);
// Box of the two-point sort keys: the scene box grown on every side by the
// key length len = 1/20 of the scene box diagonal.
inline void two_point_box(const GScene &S, float4 &lo, float4 &inv, float &len) {
    float ext[3], d2 = 0.0f;
    for (int a = 0; a < 3; a++) {
        float iv = (&S.bounds_inv_extent.x)[a];
        ext[a] = iv > 0.0f ? 1.0f / iv : 0.0f;
        d2 += ext[a] * ext[a];
    }
    len = d2 > 0.0f ? sqrtf(d2) / 20.0f : 1.0f;
    lo = make_float4(S.bounds_min.x - len, S.bounds_min.y - len, S.bounds_min.z - len, 0.0f);
    inv = make_float4(1.0f / (ext[0] + 2.0f * len), 1.0f / (ext[1] + 2.0f * len), 1.0f / (ext[2] + 2.0f * len), 0.0f);
}
// Ray order of trace calls (two-point keys, stable radix sort): n words each.
struct RayOrderBufs {
    uint32_t *keys, *vals, *keys2, *vals2;
    uint32_t *scratch;  // radix_sort_scratch_words(n)
};
cudaError_t launch_ray_order(const GScene &S, const PsyRay *rays, uint32_t n, const RayOrderBufs &B,
                             const uint32_t **order, cudaStream_t st);
// Persistent traversal kernels with per-lane ray refill.  `minb` selects the
// register budget (4 or 8 resident blocks of 128 threads per SM); `work` is a
// device counter the launch zeroes first.
// The static-scene traversal with lane refill (trace mode 5; the scene must
// have static_fast set): persistent blocks, work counter `work`.
cudaError_t launch_trace_static_refill_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue,
                                             const uint32_t *count, uint32_t max_count, int stack, uint32_t *work,
                                             int *d_err, cudaStream_t st);
cudaError_t launch_trace_static_refill_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order,
                                            PsyHit *hits, int stack, uint32_t *work, int *d_err, cudaStream_t st);
cudaError_t launch_trace_persist_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue,
                                       const uint32_t *count, uint32_t max_count, int stack, int minb, uint32_t *work,
                                       int *d_err, unsigned long long *counters, cudaStream_t st);
cudaError_t launch_trace_persist_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order,
                                      PsyHit *hits, int stack, int minb, uint32_t *work, int *d_err,
                                      unsigned long long *counters, cudaStream_t st);
// Camera rays for the wave described by d_wave (device memory; the grid
// covers max_paths); fills queue with 0..n-1 and *count = n.
// prec: 0 = f64 sampling arithmetic as the reference, 1 = f32.
cudaError_t launch_camera(const GScene &S, const WaveDesc *d_wave, uint32_t max_paths, PathState P, RayBuf R,
                          uint32_t *queue, uint32_t *count, int prec, cudaStream_t st);
// Warp-packet traversal (trace mode 2): the same hits as the per-ray kernels.
cudaError_t launch_trace_packet_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue,
                                      const uint32_t *count, uint32_t max_count, int stack, int grid, int *d_err,
                                      unsigned long long *counters, cudaStream_t st);
cudaError_t launch_trace_packet_rays(const GScene &S, const PsyRay *rays, uint32_t n, const uint32_t *order,
                                     PsyHit *hits, int stack, int *d_err, unsigned long long *counters,
                                     cudaStream_t st);
// Where the shading kernels put the live paths: the queue and its count,
// and -- when the next queue is ordered by two-point key (the radix-sorted
// binning) -- each entry's sort key beside it (keys != nullptr): the key of
// the path's next ray with the occlusion flag above it, computed where the
// ray is written instead of by a pass that reads every queued ray again.
// lo, inv, len: the key box (two_point_box); p: bits per coordinate.
struct QueueOut {
    uint32_t *queue, *count;
    uint32_t *keys;
    float4 lo, inv;
    float len;
    int p;
};
// The f32 (optimized form) camera and hit-shading kernels, in their own
// translation unit (wave_f32.cu) compiled with FMA contraction; its copies
// of the Sobol nibble tables and the unshaded-instance colour are set by
// psy_upload_wave_f32_constants (null arguments are left alone).
cudaError_t launch_camera_f32(const GScene &S, const WaveDesc *d_wave, uint32_t max_paths, PathState P, RayBuf R,
                              uint32_t *queue, uint32_t *count, cudaStream_t st);
cudaError_t launch_shade_hit_f32(const GScene &S, const WaveDesc *d_wave, PathState P, RayBuf R, HitBuf H,
                                 const uint32_t *queue, const uint32_t *count, uint32_t max_count,
                                 const QueueOut &out, int minb, int grid, cudaStream_t st);
void psy_upload_wave_f32_constants(const uint32_t sobol_nib[8][8][16], const float magenta[3]);
// Grid of a wavefront kernel `fn` (128 threads per block) over a device-side
// queue of at most max_count entries: `grid` > 0 as given, 0 one thread per
// queue slot, PSY_GRID_RESIDENT (-1) the blocks of `fn` that are resident
// on the device at once, -k k rounds of them.  The kernels stride over the
// queue, so any grid covers any count; in the late iterations of a large
// wave, whose queues hold few paths, a resident grid launches a few
// thousand blocks instead of one per slot of the wave (about a million
// empty blocks on a 132M-path wave).
#define PSY_GRID_RESIDENT (-1)
int queue_grid(const void *fn, int grid, uint32_t max_count);
// Trace the queued rays of a wave.  fast: the static-scene traversal (1) or
// its speculative form (2) when the scene allows it (GScene::static_fast)
// and no counters are requested; minb 6, 8, 10 or 12 there.
cudaError_t launch_trace_queue(const GScene &S, RayBuf R, HitBuf H, const uint32_t *queue, const uint32_t *count,
                               uint32_t max_count, int stack, int minb, int grid, int *d_err,
                               unsigned long long *counters, cudaStream_t st, int fast = 0);
// LightPath::next for the queued paths; live paths go to next_queue.
// minb: register budget for 4 (f32 form: at most 128 registers; f64 form: the
// compiler's choice), 6 or 8 resident blocks.
cudaError_t launch_shade(const GScene &S, const WaveDesc *d_wave, PathState P, RayBuf R, HitBuf H, const uint32_t *queue,
                         const uint32_t *count, uint32_t max_count, const QueueOut &out, int minb, int grid, int prec,
                         cudaStream_t st);
// Scratch of the queue ordering: u16 keys and 2^16 counters (bins) for the
// counting sort, u32 keys / second buffers / radix scratch for the radix
// sort (null when absent).
struct QueueSortBufs {
    uint16_t *keys16;
    uint32_t *bins;
    uint32_t *keys, *keys2, *vals2, *scratch;
};
// Groups the live paths of queue[0 .. *count) by their next ray into
// out[0 .. n) and sets *out_count = n: a counting sort by occlusion flag,
// direction octant and origin cell, bits 4, 10, 13 or 16 (= 4 + 3k).  Wider
// keys (19, 25, 31: the occlusion flag above a two-point key of
// (bits - 1) / 6 bits per coordinate) are written by the shading kernels
// and radix-sorted by launch_queue_radix.
cudaError_t launch_queue_binning(const GScene &S, RayBuf R, const uint32_t *queue, const uint32_t *count,
                                 uint32_t max_count, int bits, const QueueSortBufs &Q, uint32_t *out,
                                 uint32_t *out_count, cudaStream_t st);
// The radix-sorted binning of a queue whose keys the shading kernels wrote
// (QueueOut::keys = Q.keys, QueueOut::queue = vals, count = the queue's
// count): a stable radix sort of (Q.keys, vals) by `bits` bits; *sorted is
// the buffer holding the sorted paths (vals or Q.vals2, by the number of
// passes).
cudaError_t launch_queue_radix(const QueueSortBufs &Q, uint32_t *vals, const uint32_t *count, uint32_t max_count,
                               int bits, uint32_t **sorted, cudaStream_t st);
// Words of QueueSortBufs' radix part (keys, keys2, vals2, scratch) for n paths.
size_t queue_radix_words(uint32_t n);
// All device buffers one render wave needs (owned by a scene, or carved from
// a static scratch array by the no-allocation entry point).
struct WaveBufs {
    PathState P;
    RayBuf R;
    HitBuf H;
    uint32_t *queue[2];
    uint32_t *counts;      // [3] lengths of queue[0], queue[1] and stage
    uint32_t *work;        // persistent-kernel work counter
    int *err;              // device error word
    uint32_t *stage;       // binned queue (may be null: no binning)
    uint16_t *stage_key;   // binning keys
    uint32_t *bins;        // 2^16 bin counters
    uint32_t *qradix;      // radix ordering scratch, queue_radix_words(cap) (may be null)
    uint32_t cap;          // paths per wave
    WaveDesc *waves;       // wave descriptors (device)
    uint32_t cap_waves;
};
// Per-pixel XYZ (sum over samples in sample order / spp) into each segment's
// image: local row r (image row y0 + r * ystep) and column x land at
// out[((orow0 + r) * out_stride + x - out_x0) * 3].  The grid covers max_pix
// pixels.
cudaError_t launch_accumulate(const GScene &S, const WaveDesc *d_wave, uint32_t max_pix, PathState P, cudaStream_t st);
// The spectrum table of each indexed colour (PSY_SPEC_TABLE floats each)
// from its XYZ value.
cudaError_t launch_spectrum_tables(const float4 *d_xyz, uint32_t n, float *d_tables, cudaStream_t st);
cudaError_t launch_debug_color_spectra(const GScene &S, const float4 *d_xyz, uint32_t n_colors, const float *d_hero,
                                       uint32_t n, float *d_exact, float *d_table, cudaStream_t st);
// Sampler values for tests (op 0-4 as psy_debug_samplers documents):
// d_args holds n rows of 5 words, d_out n rows of 4 words.
cudaError_t launch_debug_samplers(int op, const uint32_t *d_args, uint32_t n, uint32_t *d_out, cudaStream_t st);
// 3x3 matrix passed by value to a kernel.
struct Mat3f {
    float m[9];
};
// XYZ image (w*h*3 floats, row 0 first) -> RGBA8 sRGB, rows flipped, as the
// reference writes PNGs; m = the XYZ -> rec709 matrix.
cudaError_t launch_xyz_to_srgb8(const float *xyz, uint32_t w, uint32_t h, const Mat3f &m, uint8_t *rgba,
                                cudaStream_t st);
// Sum of per-path ray counts of a wave into *out (u64).
cudaError_t launch_count_rays(PathState P, uint32_t n, unsigned long long *out, cudaStream_t st);
