/*
 * psy_gpu.h -- C ABI of the GB300 tracing path for the Psychopath renderer.
 *
 * This library replaces two things in Psychopath's Rust renderer:
 *
 *   1. `Tracer::trace` (src/tracer.rs:34-37): trace a batch of rays against
 *      the scene and return one surface intersection per ray.  Here:
 *      psy_trace().
 *   2. The body of `Renderer::render_job` for one bucket
 *      (src/renderer.rs:239-310): per-sample camera rays, the light-path
 *      state machine (LightPath::next, src/renderer.rs:449-691) and the XYZ
 *      accumulation.  Here: psy_render_bucket() / psy_render_image().
 *
 * The Rust host keeps the .psy parser, the scene/assembly builders and the
 * bucket scheduler.  It flattens its `Scene` into a PsySceneDesc (plain
 * pointers and sizes, no Rust or torch types) and calls psy_scene_create()
 * once; the library builds the same BVH4 trees the reference builds
 * (src/accel/bvh_base.rs, src/accel/bvh4.rs), uploads everything to HBM and
 * keeps it resident until psy_scene_destroy().
 *
 * Conventions:
 *   - Every call returns PSY_OK (0) or a negative PSY_E_* code; no call
 *     aborts the process.  psy_last_error() returns a short message for the
 *     calling thread's last failure.
 *   - Handles are opaque and owned by the caller (create/destroy pairs).
 *   - Calls on different handles may run on different host threads; calls
 *     on one handle must be serialised by the caller.
 *   - `stream` arguments are cudaStream_t passed as void* (NULL = the
 *     library's own stream for that handle).  Calls that take host buffers
 *     synchronise with that stream before returning.
 *   - Transforms are 3x4 row-major affine matrices [a b c d; e f g h;
 *     i j k l] (the reference's Transform::new_from_values order); a point p
 *     maps to (a*px + b*py + c*pz + d, ...).
 */
#ifndef PSY_GPU_H
#define PSY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- errors */
#define PSY_OK 0
#define PSY_E_INVALID (-1)     /* bad argument or malformed scene description */
#define PSY_E_CUDA (-2)        /* a CUDA call failed (message in psy_last_error) */
#define PSY_E_NOMEM (-3)       /* device or host allocation failed */
#define PSY_E_UNSUPPORTED (-4) /* feature outside what this build implements */
#define PSY_E_TIMEOUT (-5)     /* a bounded device wait ran out */
#define PSY_E_BUSY (-6)        /* admission refused: over the memory budget */
#define PSY_E_NOTFOUND (-7)    /* unknown request id */
#define PSY_E_CANCELLED (-8)   /* request was cancelled */
#define PSY_E_OVERFLOW (-9)    /* traversal stack overflow (scene deeper than supported) */

/* ---------------------------------------------------------------- scene */

/* Colour, as the reference's `Color` enum (src/color.rs:47-60).  XYZ values
 * are already converted from the scene's RGB by the host
 * (rec709_e_to_xyz, as parse_color does in src/parse/psy.rs:582-615). */
#define PSY_COLOR_XYZ 0
#define PSY_COLOR_BLACKBODY 1   /* v = (temperature K, factor, unused) */
#define PSY_COLOR_TEMPERATURE 2 /* v = (temperature K, factor, unused) */
typedef struct PsyColor {
    uint32_t kind;
    float v[3];
} PsyColor;

/* Surface shader, as `SimpleSurfaceShader` (src/shading/mod.rs:27-40). */
#define PSY_SHADER_EMIT 0
#define PSY_SHADER_LAMBERT 1
#define PSY_SHADER_GGX 2
typedef struct PsyShaderDesc {
    uint32_t kind;
    PsyColor color;
    float roughness; /* GGX only */
    float fresnel;   /* GGX only */
} PsyShaderDesc;

/* Objects of an assembly (src/scene/assembly.rs:398-402). */
#define PSY_OBJ_MESH 0         /* TriangleMesh (src/surface/triangle_mesh.rs) */
#define PSY_OBJ_RECT_LIGHT 1   /* RectangleLight (src/light/rectangle_light.rs) */
#define PSY_OBJ_SPHERE_LIGHT 2 /* SphereLight (src/light/sphere_light.rs) */
typedef struct PsyObjectDesc {
    uint32_t kind;
    uint32_t time_samples; /* motion keys: vertex keys (mesh) or light keys */
    /* PSY_OBJ_MESH */
    uint32_t num_verts;
    uint32_t num_tris;
    const float *verts;       /* [time_samples][num_verts][3] */
    const float *normals;     /* [time_samples][num_verts][3] or NULL */
    const uint32_t *indices;  /* [num_tris][3], as written in the scene */
    /* PSY_OBJ_RECT_LIGHT: dims = [time_samples][2] (width, height)
     * PSY_OBJ_SPHERE_LIGHT: dims = [time_samples] (radius) */
    const float *dims;
    const PsyColor *colors;   /* [time_samples] */
} PsyObjectDesc;

/* An instance in the root assembly (src/scene/assembly.rs:404-411).
 * xform_count motion keys of world-to-object transforms start at
 * xforms[xform_start]; xform_count == 0 means no transform. */
typedef struct PsyInstanceDesc {
    uint32_t object;
    int32_t shader; /* index into shaders, or -1 (unassigned: magenta Emit) */
    uint32_t xform_start;
    uint32_t xform_count;
} PsyInstanceDesc;

typedef struct PsyTransform {
    float m[12];
} PsyTransform;

/* Camera (src/camera.rs:12-72): camera-to-world transforms, field of view
 * in radians, aperture radius and focus distance, each with its own keys. */
typedef struct PsyCameraDesc {
    uint32_t num_transforms;
    const PsyTransform *transforms;
    uint32_t num_fovs;
    const float *fovs;
    uint32_t num_aperture_radii; /* 0: pinhole */
    const float *aperture_radii;
    uint32_t num_focus_distances;
    const float *focus_distances;
} PsyCameraDesc;

/* DistantDiskLight (src/light/distant_disk_light.rs:17-35): angular radius
 * (radians), direction the light travels, colour; num_keys keys each. */
typedef struct PsyDistantLightDesc {
    uint32_t num_keys;
    const float *radii;       /* [num_keys] */
    const float *directions;  /* [num_keys][3] */
    const PsyColor *colors;   /* [num_keys] */
} PsyDistantLightDesc;

typedef struct PsySceneDesc {
    uint32_t num_objects;
    const PsyObjectDesc *objects;
    uint32_t num_shaders;
    const PsyShaderDesc *shaders;
    uint32_t num_instances;
    const PsyInstanceDesc *instances;
    uint32_t num_xforms;
    const PsyTransform *xforms;
    PsyCameraDesc camera;
    PsyColor background; /* World background colour (src/scene/world.rs) */
    uint32_t num_distant_lights;
    const PsyDistantLightDesc *distant_lights;
    /* RenderSettings (src/parse/psy.rs:260-351) */
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint32_t seed;
    /* Bounce limit of LightPath::next; the reference hard-codes 2
     * (src/renderer.rs:599). */
    uint32_t max_bounces;
} PsySceneDesc;

/* Options of a scene build. */
#define PSY_BOUNDS_FP32 0 /* BVH4 child bounds as f32, bit-identical to the reference */
#define PSY_BOUNDS_FP16 1 /* child bounds as f16 rounded outward (conservative) */
/* Arithmetic of the light / cone / spherical-triangle sampling and the pixel
 * filter, which the reference evaluates in f64. */
#define PSY_SHADING_F64 0 /* as the reference (f64 where it uses f64) */
#define PSY_SHADING_F32 1 /* f32 throughout: no FP64 outside the watertight triangle retest */
/* Order in which psy_trace / psy_trace_device traverse the rays of a call.
 * Hits always land at each ray's own index, so results do not change. */
#define PSY_RAY_ORDER_AS_GIVEN 0
#define PSY_RAY_ORDER_BINNED 1 /* calls of >= 65,536 rays: sort by origin and a point along the ray first */
/* How mesh BVHs are built.  PSY_BVH_SAH is the reference's builder
 * (src/accel/bvh_base.rs, objects_split.rs, bvh4.rs) on the host: the same
 * tree, so the same hits including exact ties and the same node-visit
 * counts.  PSY_BVH_GPU builds static meshes' BVHs on the GPU (Morton codes,
 * radix sort, binary radix tree, BVH4 collapse): a different tree, so hits
 * agree except where two primitives tie exactly, in a fraction of the scene
 * creation time.  Motion-blurred meshes always use the SAH build. */
#define PSY_BVH_SAH 0
#define PSY_BVH_GPU 1
typedef struct PsySceneOptions {
    uint32_t bounds_precision;  /* PSY_BOUNDS_* */
    uint32_t shading_precision; /* PSY_SHADING_* */
    uint32_t ray_order;         /* PSY_RAY_ORDER_* */
    uint32_t bvh_build;         /* PSY_BVH_* */
    uint32_t reserved[4];
} PsySceneOptions;

typedef struct PsyScene PsyScene; /* opaque */

/* Build a scene.  Replaces the reference's scene/accel construction:
 * TriangleMesh::from_verts_and_indices (src/surface/triangle_mesh.rs:29-115),
 * AssemblyBuilder::build (src/scene/assembly.rs:288-350) and
 * Camera::new (src/camera.rs:22-72).  opts may be NULL (FP32 bounds). */
int psy_scene_create(const PsySceneDesc *desc, const PsySceneOptions *opts,
                     PsyScene **out);
/* Free everything psy_scene_create allocated. */
int psy_scene_destroy(PsyScene *scene);
/* Device bytes the scene holds resident (BVHs, geometry, lights). */
int psy_scene_device_bytes(const PsyScene *scene, uint64_t *bytes);

/* ---------------------------------------------------------------- trace */

/* One ray of a batch; the fields of the reference's `Ray` (src/ray.rs:15-21)
 * plus the occlusion flag of RayBatch::push (src/ray.rs:65-78). */
#define PSY_RAY_OCCLUSION 1u
typedef struct PsyRay {
    float orig[3];
    float dir[3];
    float max_t;
    float time;
    float wavelength;
    uint32_t flags; /* PSY_RAY_OCCLUSION */
} PsyRay;

/* Result for one ray: the discriminant and intersection data of the
 * reference's `SurfaceIntersection` (src/surface/mod.rs:72-92). */
#define PSY_HIT_MISS 0
#define PSY_HIT_OCCLUDE 1
#define PSY_HIT_SURFACE 2 /* triangle of a mesh */
#define PSY_HIT_LIGHT 3   /* surface of a rectangle or sphere light (Emit closure) */
typedef struct PsyHit {
    uint32_t kind;
    uint32_t prim; /* original triangle index in the mesh (rect light: 0/1) */
    uint32_t inst; /* instance index in PsySceneDesc.instances */
    float t;
    float b0, b1, b2; /* barycentrics (triangles) */
    float pad;
} PsyHit;

/* Full intersection data (SurfaceIntersectionData, src/surface/mod.rs:76-88)
 * for callers that keep shading on the host. */
typedef struct PsySurfaceHit {
    PsyHit hit;
    float pos[3];
    float pos_err;
    float nor[3];     /* shading normal */
    float sample_pdf; /* lights only */
    float nor_g[3];   /* geometric normal */
    int32_t shader;   /* instance's shader index, -1 if none */
} PsySurfaceHit;

/* Trace n rays (host buffers) and write one PsyHit per ray.  Replaces
 * Tracer::trace (src/tracer.rs:34-37).  Like the reference, a hit shrinks
 * the ray's max_t; this call does not write the rays back.
 * full_out may be NULL; when given, it receives PsySurfaceHit records. */
int psy_trace(PsyScene *scene, const PsyRay *rays, uint32_t n, PsyHit *hits,
              PsySurfaceHit *full_out, void *stream);

/* Device-resident form: rays/hits are device pointers (PsyRay / PsyHit
 * arrays).  Asynchronous on `stream`. */
int psy_trace_device(PsyScene *scene, const PsyRay *d_rays, uint32_t n,
                     PsyHit *d_hits, void *stream);

/* Total rays traced through this scene handle (Tracer::rays_traced,
 * src/tracer.rs:39-41). */
int psy_rays_traced(const PsyScene *scene, uint64_t *count);

/* ---------------------------------------------------------------- render */

typedef struct PsyBucket {
    uint32_t x, y, w, h; /* BucketJob (src/renderer.rs:739-745) */
} PsyBucket;

/* Stage timers of RenderStats (src/renderer.rs:40-73), in seconds of device
 * time, plus counters. */
typedef struct PsyRenderStats {
    double trace_time;
    double initial_ray_generation_time;
    double ray_generation_time;
    double sample_writing_time;
    double total_time;
    uint64_t ray_count;
    uint64_t accel_node_visits;
    uint64_t samples;
} PsyRenderStats;

/* Render one bucket: spp samples per pixel with the scene's seed.
 * xyz_out (host) receives bucket.w*bucket.h*3 floats, row-major, the XYZ
 * value each pixel would hold after the reference's accumulation
 * (src/renderer.rs:299-310).  stats may be NULL.  An empty bucket, spp == 0
 * or a bucket reaching past the image returns PSY_E_INVALID. */
int psy_render_bucket(PsyScene *scene, const PsyBucket *bucket, uint32_t spp,
                      uint32_t seed, float *xyz_out, PsyRenderStats *stats);

/* Render the whole image (or the crop x0,y0,x1,y1 inclusive when crop is not
 * NULL) into d_xyz, a DEVICE buffer of width*height*3 floats.  Asynchronous
 * on `stream`; stats (if not NULL) are filled after an internal sync. */
int psy_render_image_device(PsyScene *scene, const uint32_t *crop,
                            float *d_xyz, void *stream, PsyRenderStats *stats);

/* Same, into a HOST buffer (synchronous). */
int psy_render_image(PsyScene *scene, const uint32_t *crop, float *xyz_out,
                     PsyRenderStats *stats);

/* One share of a frame rendered on several GPUs: the image rows first_row,
 * first_row + row_step, first_row + 2 * row_step, ... (all columns), into
 * d_xyz, a DEVICE buffer of n * width * 3 floats holding those rows in order
 * (n = ceil((height - first_row) / row_step)).  Each pixel is the one a
 * whole-image render gives.  With row_step = N and first_row = rank, N GPUs
 * split a frame into interleaved rows, which balances their work as the
 * reference's bucket queue balances its threads (Renderer::render hands
 * Hilbert-ordered buckets to whichever thread is free,
 * src/renderer.rs:150-180).  Asynchronous on `stream` (NULL: the scene's
 * stream); stats (if not NULL) are filled after an internal sync.
 * row_step = 0 returns PSY_E_INVALID. */
int psy_render_rows_device(PsyScene *scene, uint32_t first_row, uint32_t row_step,
                           float *d_xyz, void *stream, PsyRenderStats *stats);

/* Image output as the reference writes PNGs (Image::write_png,
 * src/image.rs:138-164): the XYZ image d_xyz (width*height*3 floats, row 0
 * first, as the render calls produce) becomes RGBA8 in d_rgba
 * (width*height*4 bytes): XYZ -> rec709 (equal-energy white), sRGB gamma,
 * clamp to [0, 1], x 255 truncated; rows flipped (d_rgba row 0 = the
 * image's last row), alpha 255.  Runs on `stream` (NULL: the legacy default
 * stream); both buffers are device memory. */
int psy_xyz_to_srgb8(const float *d_xyz, uint32_t width, uint32_t height, uint8_t *d_rgba, void *stream);

/* Halton sample generation, replacing halton::sample(index, dimension) of
 * sub_crates/halton (src/lib.rs includes the code build.rs:101-225
 * generates): Halton points with Faure digit permutations in the first 128
 * prime bases, bit-exact.  d_out[i] = sample(d_indices[i], dimension) for
 * i < n (both device buffers), on `stream` (NULL: the legacy default
 * stream).  dimension >= 128 returns PSY_E_INVALID (the reference panics).
 * The first call on a device uploads the permutation tables (~80 KB of
 * device memory, kept until exit). */
int psy_halton_samples(uint32_t dimension, const uint32_t *d_indices, uint32_t n, float *d_out, void *stream);

/* ------------------------------------------------------- compact codecs */

/* Batch forms of the `compact` crate's encodings (sub_crates/compact), bit
 * for bit.  Encoders read n (x, y, z) f32 triples (12 bytes each) and write
 * n codes of psy_compact_element_size() bytes, packed; decoders do the
 * reverse.  Multi-byte codes are little-endian, as the crate's
 * to_ne_bytes / u64_to_bytes give on little-endian hosts. */
#define PSY_COMPACT_FLUV32 0        /* fluv::fluv32 (fluv/fluv32.rs:76-170): XYZ colour, u32 */
#define PSY_COMPACT_OCT32 1         /* unit_vec::oct32 encode/decode (unit_vec/oct32.rs:15-70), u32 */
#define PSY_COMPACT_OCT32_PRECISE 2 /* oct32::encode_precise (:24-61); decodes as PSY_COMPACT_OCT32 */
#define PSY_COMPACT_UNSIGNED32 3    /* shared_exp::unsigned32 (shared_exp/unsigned32.rs:36-85), u32 */
#define PSY_COMPACT_UNSIGNED40 4    /* shared_exp::unsigned40 (shared_exp/unsigned40.rs:36-120), 5 bytes */
#define PSY_COMPACT_SIGNED48 5      /* shared_exp::signed48 (shared_exp/signed48.rs:48-144), 6 bytes */

/* Bytes per code of `format`; PSY_E_INVALID for an unknown format. */
int psy_compact_element_size(uint32_t format, uint32_t *bytes);

/* Encode n triples of d_xyz (device, 3*n floats) into d_out (device, n codes).
 * The crate's encoders assert their domain in debug builds (fluv32,
 * unsigned32, unsigned40: no negative or NaN component; signed48: no NaN;
 * oct32: none) and write the release build's code otherwise; here every
 * element gets the release build's code and, when d_invalid (a device u32)
 * is not NULL, the number of elements outside the domain is added to it.
 * Asynchronous on `stream` (NULL: the legacy default stream).  Buffers may
 * have any alignment (16-byte aligned ones take the vector path); d_invalid
 * must be 4-byte aligned (else PSY_E_INVALID). */
int psy_compact_encode(uint32_t format, const float *d_xyz, uint32_t n, void *d_out, uint32_t *d_invalid,
                       void *stream);

/* Decode n codes of d_in (device) into d_xyz (device, 3*n floats).  Every
 * bit pattern decodes (the crate's decoders cannot fail). */
int psy_compact_decode(uint32_t format, const void *d_in, uint32_t n, float *d_xyz, void *stream);

/* fluv32::decode_yuv (fluv/fluv32.rs:160-170): Y and the raw u', v' bytes. */
typedef struct PsyYuv {
    float y;
    uint8_t u, v;
    uint8_t pad[2]; /* written as 0 */
} PsyYuv;
int psy_fluv32_decode_yuv(const uint32_t *d_in, uint32_t n, PsyYuv *d_yuv, void *stream);

/* Colour compression as Color::write_compressed / Color::from_compressed
 * (src/color.rs:144-249): 5 bytes per colour, a discriminant byte (0 XYZ,
 * 1 blackbody, 2 temperature) then the fluv32 code of the XYZ triple, or
 * the temperature as a saturating u16 and the factor as an IEEE half (round
 * to nearest even), both little-endian.  d_out / d_in hold 5*n bytes.
 * d_invalid (optional device u32) counts XYZ colours outside fluv32's domain
 * and unknown kinds on compression, and unknown discriminants on
 * decompression (the reference's unreachable!()); such records are
 * written as zeros. */
int psy_color_compress(const PsyColor *d_colors, uint32_t n, uint8_t *d_out, uint32_t *d_invalid, void *stream);
int psy_color_decompress(const uint8_t *d_in, uint32_t n, PsyColor *d_colors, uint32_t *d_invalid, void *stream);

/* Closure compression as SurfaceClosure::write_compressed / from_compressed
 * (src/shading/surface_closure.rs:157-253), for closures given as shader
 * descriptions (kind, colour, roughness, fresnel): a discriminant byte
 * (Lambert 0, GGX 1, Emit 2); a GGX closure then carries roughness and
 * fresnel, each clamped to [0, 1] and stored as a truncated u16 fraction of
 * 65535, little-endian; the compressed colour follows (6 bytes in all, 10
 * for GGX).  Record i starts at byte i*stride, as MicropolyBatch packs them
 * (src/surface/micropoly_batch.rs:322-332); bytes past a record's end are
 * left alone.  stride < 6, or PsyShaderDesc arrays or d_invalid that are
 * not 4-byte aligned, return PSY_E_INVALID.  d_invalid (optional)
 * counts records that do not fit the stride (the reference panics) -- left
 * unwritten on compression, decoded as a black Emit closure on
 * decompression -- and the colour errors of psy_color_compress. */
int psy_closure_compress(const PsyShaderDesc *d_closures, uint32_t n, uint32_t stride, uint8_t *d_out,
                         uint32_t *d_invalid, void *stream);
int psy_closure_decompress(const uint8_t *d_in, uint32_t n, uint32_t stride, PsyShaderDesc *d_closures,
                           uint32_t *d_invalid, void *stream);

/* Render one bucket without allocating device memory.  This call has no
 * counterpart in the reference: it exists for hosts that cannot call
 * cudaMalloc once they are running -- for example a process whose device
 * memory is reserved up front by another framework's allocator, or a render
 * worker that must keep a fixed memory footprint after start-up.  The caller
 * passes d_xyz_out, a DEVICE buffer of bucket->w * bucket->h * 3 floats
 * (row-major within the bucket), and receives the same values
 * psy_render_bucket writes.  All scratch lives in one static device array of
 * the library (46.25 MiB, held on every GPU that loads the library until the
 * process exits), so a bucket may hold at most PSY_NOALLOC_MAX_SAMPLES
 * samples (w * h * spp); larger buckets are rejected with PSY_E_INVALID.
 * Nothing has to start at zero: every value of d_xyz_out is overwritten, and
 * the call clears its own queue counters and error word inside the array at
 * the start of each call.  The scene itself must have been created (its
 * geometry upload is the one allocation, made at psy_scene_create).
 * The first call on a device looks up that array's device address, so make
 * the first call before any stream capture.  The scene's device (the one
 * current at psy_scene_create) must be the current device; otherwise the
 * call returns PSY_E_INVALID.  Every call shares the array:
 * calls that overlap on the GPU (other threads, other streams) race and must
 * be serialised by the caller.  The call runs on `stream` (NULL: the scene's
 * stream) and returns after that stream has finished the bucket. */
#define PSY_NOALLOC_MAX_SAMPLES 262144u
int psy_render_bucket_noalloc(PsyScene *scene, const PsyBucket *bucket, uint32_t spp, uint32_t seed,
                              float *d_xyz_out, void *stream);

/* ---------------------------------------------------------------- autotuning */

/* Picks the scene's launch configuration by timing a probe render: a band of
 * full-width rows in the middle of the scene's image with about probe_paths
 * paths (all samples of each pixel).  Coordinate descent over, in order: the
 * trace kernel (one thread per ray with a register budget of 4, 5, 6 or 8
 * resident blocks per SM, persistent with lane refill at 4, 6 or 8, or --
 * on scenes without motion or mesh instance transforms -- the static-scene
 * traversal at 8, 10 or 12 and its lane-refill form), the shading kernel's
 * register budget (4, 6 or
 * 8 blocks per SM), the traversal stack depth (64 or 192 entries, if the
 * scene fits), the queue tile (grid of the wavefront kernels: sized by the
 * queue, a grid-stride grid of 8, 16 or 32 blocks per SM, or each kernel's
 * resident blocks striding over the queue; then resident blocks for the
 * last 4, 6, 8 or 10 iterations of a wave only), the key width
 * of the queue binning between wavefront iterations (0 = off, 4 = occlusion
 * flag and direction octant, 10 / 13 / 16 = also 2 / 3 / 4 bits per axis of
 * the origin's cell, 19 / 25 = occlusion flag above a two-point key, radix
 * sorted), the wave size (paths per wave) and CUDA graph replay; the
 * fastest candidate of each set replaces the current choice when its probe
 * time is at least 2% lower.  A last step times the whole image with larger
 * waves (twice, four times the chosen one, the whole image), bounded by
 * max_wave_mib or by the buffers already held plus a quarter of the free
 * device memory; when the wave grows, the grid and the key width are timed
 * again on the whole image.  Every candidate renders the same image bit for
 * bit (only scheduling changes), so tuning never changes results.  The
 * chosen configuration stays on the scene.  No counterpart in the reference
 * (its renderer has no GPU launch parameters). */
typedef struct PsyTuneOptions {
    uint32_t probe_paths;  /* 0: 16,777,216 (capped at the whole image) */
    uint32_t repeats;      /* timed probe renders per candidate, best taken (0: 3) */
    uint32_t max_wave_mib; /* cap on the wave buffers the last (whole-image, larger
                              waves) step may choose, MiB; 0: the buffers already
                              held plus a quarter of the free device memory */
    uint32_t reserved[5];
} PsyTuneOptions;

#define PSY_TUNE_GRID_RESIDENT 0xFFFFFFFFu

typedef struct PsyTuneResult {
    uint32_t trace_mode;   /* 0: one thread per ray, 1: persistent, 2: warp packets,
                              3: static-scene traversal (scenes without motion or mesh
                              instance transforms), 4: its speculative form, 5: the
                              static-scene traversal with lane refill */
    uint32_t minb;         /* register budget (resident blocks per SM) */
    uint32_t stack;        /* traversal stack entries */
    uint32_t grid;         /* wavefront kernel grid (0: sized by the queue,
                              PSY_TUNE_GRID_RESIDENT: each kernel's resident blocks) */
    uint32_t sort_bits;
    uint32_t wave_paths;
    uint32_t use_graph;
    uint32_t shade_minb;   /* shading kernel register budget (resident blocks per SM) */
    uint32_t candidates;   /* configurations timed */
    double default_s;      /* probe time of the configuration before tuning */
    double best_s;         /* probe time of the chosen configuration */
    uint32_t resident_tail; /* the last n wavefront iterations of a wave launch each
                               kernel on its resident blocks (0: none) */
    uint32_t reserved;
} PsyTuneResult;

int psy_autotune(PsyScene *scene, const PsyTuneOptions *opts, PsyTuneResult *result);

/* ---------------------------------------------------------------- serving */

/* A render server: a persistent request loop over resident scenes.  The
 * reference renders one scene per process invocation (src/main.rs:150-330,
 * Renderer::render src/renderer.rs:76-191) and has no request API; these
 * calls are the serving surface of the GPU path.  Each added scene gets a
 * lane (its own stream and wavefront buffers).  Requests of a scene -- each
 * with its own resolution, spp and seed -- are admitted while the HBM budget
 * and the active-request limit allow, split into rows of pixels, and packed
 * together into the lane's waves, so the paths of several requests share
 * one set of wavefront queues.  Requests that arrive while waves are on the
 * GPU join the next wave (continuous batching).  A request's image is the
 * same whether it ran alone or among others: every path depends only on
 * (scene, resolution, pixel, sample index, seed). */
typedef struct PsyServer PsyServer;

typedef struct PsyServerOptions {
    uint64_t hbm_budget_bytes; /* resident scenes + lane buffers + request images (0: 120 GB) */
    uint32_t wave_paths;       /* paths per wave of each lane (0: 4,194,304) */
    uint32_t max_active;       /* requests admitted at once (0: 64) */
    uint32_t use_graphs;       /* 1: replay each wave's launch sequence from a CUDA graph */
    uint32_t waves_in_flight;  /* queued waves per lane, 1..4 (0: 2) */
    uint32_t policy;           /* PSY_SCHED_*: order of admission and of rows in a wave (0: FIFO) */
    uint32_t aging_ms;         /* PSY_SCHED_SHORTEST: a request waiting longer than this goes first
                                  (0: 1000 ms) */
    uint32_t reserved[2];
} PsyServerOptions;

/* Scheduling policies.  FIFO: requests are admitted and their rows packed
 * into waves in arrival order.  SHORTEST: the request with the fewest
 * samples left goes first (small requests finish in one wave instead of
 * waiting behind large ones), except that requests older than aging_ms go
 * first in arrival order, which bounds how long a large request waits. */
#define PSY_SCHED_FIFO 0u
#define PSY_SCHED_SHORTEST 1u

typedef struct PsyRequest {
    uint32_t scene;            /* lane index from psy_server_add_scene */
    uint32_t width, height;    /* resolution, through the scene's camera */
    uint32_t spp, seed;
    uint32_t reserved;
    float *xyz_out;            /* HOST result, width*height*3 floats (row-major XYZ), or NULL */
    float *d_xyz_out;          /* DEVICE result buffer instead (no image allocation, no copy), or NULL */
} PsyRequest;

#define PSY_REQ_QUEUED 0u
#define PSY_REQ_RUNNING 1u
#define PSY_REQ_DONE 2u
#define PSY_REQ_CANCELLED 3u
#define PSY_REQ_FAILED 4u

typedef struct PsyRequestStatus {
    uint32_t state;            /* PSY_REQ_* */
    int32_t error;             /* PSY_E_* of a failed request */
    uint64_t samples;          /* width * height * spp */
    double queued_s;           /* submit -> admission */
    double latency_s;          /* submit -> result in place (DONE / CANCELLED / FAILED) */
    uint32_t waves;            /* waves that carried some of its paths */
    uint32_t shared_waves;     /* of those, waves that also carried other requests */
} PsyRequestStatus;

typedef struct PsyServerStats {
    uint64_t requests_done, samples_done, waves;
    uint64_t kernel_launches;  /* kernels launched for those waves */
    uint64_t hbm_used_bytes, hbm_peak_bytes, hbm_budget_bytes;
    uint32_t queued, active;
} PsyServerStats;

/* Creates the server (its scheduling thread starts at once) on the current
 * CUDA device. */
int psy_server_create(const PsyServerOptions *opts, PsyServer **out);
/* Makes `scene` resident for serving and returns its lane index.  The scene
 * is borrowed: it must outlive the server.  PSY_E_NOMEM when the scene's
 * bytes plus the lane's buffers exceed the budget. */
int psy_server_add_scene(PsyServer *srv, PsyScene *scene, uint32_t *lane);
/* Queues a request; returns at once with its id.  The result buffer must
 * stay valid until the request is finished.  PSY_E_INVALID when one row of
 * the request (width * spp paths) does not fit a wave or no output is given. */
int psy_submit(PsyServer *srv, const PsyRequest *req, uint64_t *id);
/* Current status of a request (PSY_E_NOTFOUND for an unknown id). */
int psy_poll(PsyServer *srv, uint64_t id, PsyRequestStatus *status);
/* Waits until the request is finished or timeout_s passes (PSY_E_TIMEOUT). */
int psy_wait(PsyServer *srv, uint64_t id, double timeout_s, PsyRequestStatus *status);
/* Cancels a queued or running request: it schedules no further rows and
 * ends CANCELLED once its waves in flight are done (its result buffer is
 * then partly written).  PSY_E_INVALID if it has already finished. */
int psy_cancel(PsyServer *srv, uint64_t id);
int psy_server_stats(PsyServer *srv, PsyServerStats *stats);
/* Cancels what is queued or running, waits for the GPU, frees the lanes. */
int psy_server_destroy(PsyServer *srv);

/* ---------------------------------------------------------------- misc */

/* Short description of the calling thread's last error. */
const char *psy_last_error(void);
/* Library version string. */
const char *psy_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PSY_GPU_H */
