/* Internal test and tuning hooks of libpsy_gpu.so.
 *
 * These entry points are exported for the library's own tests and benchmark
 * (bound in psychopath_gb300/gpu.py).  They are not part of the
 * reference-facing interface of include/psy_gpu.h: a host that replaces
 * Psychopath's Tracer and bucket renderer needs none of them.  They follow
 * the same conventions (PSY_OK or a negative PSY_E_* code; psy_last_error()
 * for the message; `stream` is a cudaStream_t passed as void*, NULL = the
 * scene's stream or the legacy default stream where no scene is given).
 */
#ifndef PSY_DEBUG_H
#define PSY_DEBUG_H

#include "../../include/psy_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- build facts (host side, no device work) */
/* The triangle order of mesh object `object` as the scene's BVH stores it
 * (original triangle index per position) and its BVH4 node count. */
int psy_debug_mesh_bvh_info(PsyScene *scene, uint32_t object, uint32_t *tri_order, uint32_t *node_count);
/* The traversal table as the device holds it (8 x 48 bytes), the push rows
 * (8 x 48) and the push lookup table (32 x 16 entries) of the static-scene
 * traversal. */
int psy_debug_push_tables(uint8_t *table, uint8_t *rows, uint16_t *lut);
/* Host build only: the triangle order and node count of one mesh object, and
 * the worst-case traversal stack depth of the scene. */
int psy_debug_host_build(const PsySceneDesc *desc, const PsySceneOptions *opts, uint32_t object,
                         uint32_t *tri_order, uint32_t *node_count, uint32_t *max_stack);
/* Host build only: all BVH4 nodes (128 bytes each) and motion bounds (96
 * bytes per key) of the scene, built with worker threads or (serial != 0) on
 * one thread.  Null arrays return the counts only. */
int psy_debug_host_nodes(const PsySceneDesc *desc, const PsySceneOptions *opts, int serial, void *nodes,
                         uint32_t *node_count, void *bounds_ext, uint32_t *ext_count);
/* Host build only: the FP16 node copies (96 bytes each, same indices as the
 * BVH4 nodes; none unless opts asks for FP16 bounds).  Null nodes_h returns
 * the count only. */
int psy_debug_host_nodes_h(const PsySceneDesc *desc, const PsySceneOptions *opts, void *nodes_h,
                           uint32_t *node_count);
/* Worst-case stack depth, node count and the stack variant (64 or 192). */
int psy_debug_scene_info(PsyScene *scene, uint32_t *max_stack, uint32_t *nodes, uint32_t *stack_variant);
/* bit 0: the static-scene traversal applies; bit 1: ordered child boxes;
 * bit 2: FP16 child bounds. */
int psy_debug_scene_flags(PsyScene *scene, uint32_t *flags);

/* ---- launch configuration (what psy_autotune chooses) */
/* Enable (and zero) or read the traversal counters of renders. */
int psy_debug_counters(PsyScene *scene, int enable, uint64_t *nodes, uint64_t *tris, uint64_t *rays);
/* Trace kernel: 0 one thread per ray, 1 persistent with lane refill, 2 warp
 * packets, 3 static-scene traversal, 4 its speculative form, 5 the
 * static-scene traversal with lane refill; minb = target resident blocks
 * per SM of the register budget. */
int psy_debug_set_trace(PsyScene *scene, int mode, int minb);
/* Shading kernel register budget: 4, 6 or 8 resident blocks per SM. */
int psy_debug_set_shade(PsyScene *scene, int minb);
/* Queue binning key width between wavefront iterations: 0, 4, 10, 13, 16,
 * 19, 25 or 31 bits. */
int psy_debug_set_sort(PsyScene *scene, int bits);
/* Grid of the wavefront kernels (0: sized by the queue, > 0: that many
 * blocks striding over the queue, -1: each kernel's resident blocks) and
 * the paths per wave (>= 1024 to change it). */
int psy_debug_set_launch(PsyScene *scene, int grid, uint32_t wave_paths);
/* The spectrum of each of the scene's tabulated colours (constant XYZ
 * colours) at n hero wavelengths (device arrays), by the upsampling
 * (d_exact) and from the colour's table (d_table): n_colors x n x 4 floats
 * each.  *n_colors is set even when n == 0. */
int psy_debug_color_spectra(PsyScene *scene, uint32_t n, const float *d_hero, float *d_exact, float *d_table,
                            uint32_t *n_colors);
/* The last `iterations` wavefront iterations of a wave launch each kernel on
 * its resident blocks (0: none). */
int psy_debug_set_resident_tail(PsyScene *scene, int iterations);
/* Replay each wave from a CUDA graph (1) or launch kernel by kernel (0). */
int psy_debug_set_graph(PsyScene *scene, int on);
/* Ray order of trace calls: 0 as given, 1 binned. */
int psy_debug_set_ray_order(PsyScene *scene, int order);
/* The binned order of n device rays: sorted keys and ray index per position
 * (device buffers of n words each). */
int psy_debug_ray_order(PsyScene *scene, const PsyRay *d_rays, uint32_t n, uint32_t *d_keys, uint32_t *d_order,
                        void *stream);

/* ---- renders for tests */
/* A whole width x height image with spp samples and `seed` through the
 * scene's camera into the device buffer d_xyz (width*height*3 floats);
 * returns when done.  The one-request-at-a-time form of what the render
 * server does. */
int psy_debug_render_sized(PsyScene *scene, uint32_t width, uint32_t height, uint32_t spp, uint32_t seed,
                           float *d_xyz, void *stream);
/* Render one bucket as one wave and return every path's final colour (4
 * floats per sample, the 4 hero wavelengths' values) and hero wavelength,
 * in the oracle's order: sample s of bucket pixel (x, y) at index
 * ((y - bucket.y) * bucket.w + (x - bucket.x)) * spp + s.  Host buffers of
 * w*h*spp*4 and w*h*spp floats; at most 1,048,576 samples. */
int psy_debug_render_paths(PsyScene *scene, const PsyBucket *bucket, uint32_t spp, uint32_t seed, float *color4,
                           float *wavelength);
/* The samplers of the render path evaluated on the device, for bit-for-bit
 * comparison: d_args holds n rows of 5 words (a, b, c, d, e), d_out
 * receives n rows of 4 words.
 *   op 0: hash_u32(a, b)                                   (src/hash.rs:1-10)
 *   op 1: hash_u32_to_f32(a, b) as f32 bits                (src/hash.rs:26-29)
 *   op 2: golden_ratio_sample(a, b) as f32 bits            (src/renderer.rs:728-737)
 *   op 3: get_sample_4d(i = a, set = b, px = c, py = d, seed = e), 4 f32
 *         (src/renderer.rs:698-725)
 *   op 4: the 4 wavelengths of sample a of pixel (c, d) with seed e
 *         (src/renderer.rs:261-265, src/color.rs:20-43)
 * Unused words are 0.  Runs on `stream`; returns after it finishes. */
int psy_debug_samplers(int op, const uint32_t *d_args, uint32_t n, uint32_t *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PSY_DEBUG_H */
