/*
 * Oracle (test infrastructure only).  A CPU restatement of Psychopath's
 * tracing path -- scene build, BVH4 packet traversal, lights, closures,
 * spectral upsampling and the bucket renderer -- used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU baseline as the checker.  The
 * product (psychopath_gb300) never links or calls it.
 *
 * It consumes the same PsySceneDesc as the GPU library (include/psy_gpu.h).
 */
#ifndef PSY_ORACLE_H
#define PSY_ORACLE_H

#include "../include/psy_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct PsyoScene PsyoScene;

PsyoScene *psyo_scene_create(const PsySceneDesc *desc);
void psyo_scene_destroy(PsyoScene *s);

/* Trace rays with the reference's packet traversal (Tracer::trace), in
 * batches of at most 65536 rays (the reference's u16 ray index), spread over
 * nthreads host threads.  full may be NULL.  node_tests / tri_tests receive
 * the ray x BVH4-node and ray x triangle test counts (may be NULL). */
int psyo_trace(PsyoScene *s, const PsyRay *rays, uint32_t n, PsyHit *hits, PsySurfaceHit *full,
               uint64_t *node_tests, uint64_t *tri_tests, uint32_t nthreads);

/* Render the image (or crop x0,y0,x1,y1) with the reference's bucket
 * scheduler: buckets of side sqrt(spb/spp) in Hilbert order, nthreads
 * workers.  xyz: width*height*3 floats.  When `max_buckets` > 0 only the
 * first max_buckets buckets of the Hilbert order are rendered (a bounded
 * sample for timing). */
int psyo_render(PsyoScene *s, uint32_t spb, uint32_t nthreads, const uint32_t *crop,
                uint32_t max_buckets, float *xyz, PsyRenderStats *stats);

/* As psyo_render, keeping only every bucket_stride-th bucket of the Hilbert
 * order (a sample spread over the whole image). */
int psyo_render_sampled(PsyoScene *s, uint32_t spb, uint32_t nthreads, const uint32_t *crop, uint32_t bucket_stride,
                        uint32_t max_buckets, float *xyz, PsyRenderStats *stats);

/* Render one bucket and return every sample's final path colour (4 floats)
 * and hero wavelength, indexed ((y - b.y) * b.w + (x - b.x)) * spp + si,
 * plus the number of rays each sample traced. */
int psyo_render_paths(PsyoScene *s, const PsyBucket *b, float *color4, float *wavelength,
                      uint32_t *rays_per_sample);

/* Known-answer helpers. */
uint32_t psyo_hash_u32(uint32_t n, uint32_t seed);
uint64_t psyo_hash_u64(uint64_t n, uint64_t seed);
float psyo_hash_u32_to_f32(uint32_t n, uint32_t seed);
void psyo_get_sample_4d(uint32_t i, uint32_t set, uint32_t px, uint32_t py, uint32_t seed, float *out4);
float psyo_golden_ratio_sample(uint32_t i, uint32_t scramble);
void psyo_wavelengths(uint32_t sample, uint32_t x, uint32_t y, uint32_t seed, float *out4);
float psyo_probit(float n, float width);
float psyo_fast_exp(float p);
void psyo_hilbert_d2xy(uint32_t d, uint32_t *x, uint32_t *y);
uint32_t psyo_hilbert_xy2d(uint32_t x, uint32_t y);
void psyo_traversal_table(uint8_t *out8x48);
void psyo_xf_mul(const float *a, const float *b, float *out);
void psyo_xf_inverse(const float *a, float *out);
void psyo_xf_lerp(const float *a, const float *b, float alpha, float *out);
void psyo_xf_point(const float *m, const float *p, float *out);
void psyo_xf_normal(const float *m, const float *n, float *out);
void psyo_xf_vector(const float *m, const float *v, float *out);
void psyo_lerp3(const float *a, const float *b, float alpha, float *out);
float psyo_lerp(float a, float b, float alpha);
float psyo_lerp_slice(const float *s, uint32_t n, float alpha);
void psyo_xyz_to_spectrum(const float *xyz, float hero_wavelength, float *out4);
void psyo_spectrum_to_xyz(const float *e4, float hero_wavelength, float *xyz_out);
void psyo_rec709_e_to_xyz(const float *rgb, float *xyz);
void psyo_rec709_to_xyz(const float *rgb, float *xyz);
void psyo_xyz_to_srgb8(const float *xyz, uint32_t w, uint32_t h, uint8_t *rgba);
int psyo_intersect_triangle(const float *orig, const float *dir, float max_t, const float *p0, const float *p1,
                            const float *p2, float *out_tb);
uint32_t psyo_quick_select_ints(int32_t *list, uint32_t n, uint32_t place);
int psyo_increment_ulp_check(void);

/* BVH dump for tree-identity checks: the mesh object's triangle order after
 * the build (original triangle indices) and the number of BVH4 nodes. */
int psyo_mesh_bvh_info(PsyoScene *s, uint32_t object, uint32_t *tri_order, uint32_t *node_count);
/* Light tree shape: node count, leaf count, depth (levels root to deepest
 * leaf). */
int psyo_light_tree_info(PsyoScene *s, uint32_t *nodes, uint32_t *leaves, uint32_t *depth);

/* halton::sample(index, dimension) (sub_crates/halton), restated in
 * oracle_halton.cpp; -1 for dimension >= 128. */
int psyo_halton_sample(uint32_t index, uint32_t dimension, float *out);

/* The `compact` crate's encodings and the colour / closure byte formats
 * (oracle_compact.cpp), with the GPU library's batch signatures; -1 for an
 * unknown format or a stride below 6.  *invalid receives the number of
 * elements outside the format's domain. */
int psyo_compact_encode(uint32_t format, const float *xyz, uint32_t n, uint8_t *out, uint32_t *invalid);
int psyo_compact_decode(uint32_t format, const uint8_t *in, uint32_t n, float *xyz);
void psyo_signed48_decode_u64(uint64_t t, float *out);
void psyo_fluv32_decode_yuv(const uint32_t *in, uint32_t n, PsyYuv *out);
uint32_t psyo_f16_from_f32(float f);
float psyo_f16_to_f32(uint32_t h);
int psyo_color_compress(const PsyColor *c, uint32_t n, uint8_t *out, uint32_t *invalid);
int psyo_color_decompress(const uint8_t *in, uint32_t n, PsyColor *c, uint32_t *invalid);
int psyo_closure_compress(const PsyShaderDesc *s, uint32_t n, uint32_t stride, uint8_t *out, uint32_t *invalid);
int psyo_closure_decompress(const uint8_t *in, uint32_t n, uint32_t stride, PsyShaderDesc *s, uint32_t *invalid);

#ifdef __cplusplus
}
#endif

#endif
