// Device-resident scene layout of the GB300 tracing path.
//
// Everything a kernel touches lives in HBM in these flat arrays, built once
// by psy_scene_create and kept resident.  One BVH4 node is one 128-byte
// record (a full L2 line): the bounds of its four children for time key 0
// as six float4 slabs (x/y/z min/max across the 4 lanes), the four child
// references, and the node meta.  Nodes of motion-blurred BVHs keep keys
// 1..n-1 in a separate bounds array (96 bytes per key).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define PSY_HD __host__ __device__
#else
#define PSY_HD
#include <vector_types.h>
#endif

// Child reference: bit 31 set = leaf.  Mesh BVH leaves hold up to three
// triangles: bits 29..30 = count - 1, bits 0..28 = first triangle (global
// index into the triangle arrays).  Instance BVH leaves hold one instance
// slot in bits 0..28.  Otherwise the value is a node index.
#define PSY_LEAF_BIT 0x80000000u
#define PSY_LEAF_FIRST_MASK 0x1FFFFFFFu
#define PSY_REF_NONE 0xFFFFFFFFu      // also the "leave instance" stack marker
static inline PSY_HD bool psy_is_leaf(uint32_t r) { return (r & PSY_LEAF_BIT) != 0; }
static inline PSY_HD uint32_t psy_leaf_first(uint32_t r) { return r & PSY_LEAF_FIRST_MASK; }
static inline PSY_HD uint32_t psy_leaf_count(uint32_t r) { return ((r >> 29) & 3u) + 1u; }
static inline PSY_HD uint32_t psy_make_leaf(uint32_t first, uint32_t count) {
    return PSY_LEAF_BIT | ((count - 1u) << 29) | first;
}

struct __align__(16) GNode {
    float4 xlo, xhi, ylo, yhi, zlo, zhi;  // key-0 bounds of children 0..3
    uint4 child;                          // child references
    uint4 meta;  // x: first extra key in bounds_ext, y: key count, z: traversal code | child count << 8, w: 0
};
struct __align__(16) GBounds4 {
    float4 xlo, xhi, ylo, yhi, zlo, zhi;
};
// Half-precision variant: child bounds as signed f16 offsets, lower bounds
// from an anchor (per axis the min corner of the children's union, or the
// plane of a child that is flat on that axis), upper bounds from a top
// corner decoded as fl32(anchor + ext), each chosen so the decoded f32 bound
// fl32(corner + offset) lies outside the f32 bound (the decoded box contains
// the f32 box; a flat child decodes exactly flat).  96 bytes per node.
struct __align__(16) GNodeH {
    float4 anchor;  // xyz: per axis the children's min corner or a flat child's plane, w: meta bits
                    // (traversal code | child count << 8 | PSY_NODEH_F32 flags)
    uint4 child;
    uint2 ext;      // f16 extents x | y << 16 and z: the top corner is fl32(anchor + ext)
    uint2 xlo, xhi, ylo, yhi, zlo, zhi;  // 4 x f16 per slab (48 bytes)
    uint2 pad;
};
// Meta bits of GNodeH: the node has motion keys (bit 16) or an offset that
// does not fit an f16 (bit 17); the traversal then reads the f32 node.
#define PSY_NODEH_F32 0x30000u

#define PSY_COLOR_XYZ_K 0u
#define PSY_COLOR_BLACKBODY_K 1u
#define PSY_COLOR_TEMPERATURE_K 2u
// Bits 0-15 of GColor::kind are the colour kind; bits 16-31 are 1 + the
// index of the colour's precomputed spectrum table (GScene::spec_tables)
// for the constant XYZ colours the scene stores, 0 for none.
#define PSY_COLOR_KIND_MASK 0xFFFFu
// Floats per spectrum table: the 95 samples of the Meng point spectra,
// combined with the colour's weights, and a pad.
#define PSY_SPEC_TABLE 96
// Colour (PsyColor): kind, three values.
struct __align__(16) GColor {
    uint32_t kind;
    float a, b, c;
};
struct __align__(16) GShader {
    uint32_t kind;
    float roughness, fresnel, pad;
    GColor color;
};
#define PSY_INST_MESH 0u
#define PSY_INST_RECT 1u
#define PSY_INST_SPHERE 2u
struct __align__(16) GInstance {
    uint32_t kind;
    uint32_t obj;     // mesh / rect / sphere index
    int32_t shader;   // -1: unassigned
    uint32_t id;      // index in the caller's instance list
    uint32_t xs, xc;  // world->object keys in xforms (xc == 0: none)
    uint32_t xinv;    // index of the precomputed inverse of key 0 in xforms_inv (xc == 1)
    uint32_t pad;
};
struct __align__(16) GMesh {
    uint32_t root;       // child reference of the root
    uint32_t tri_base;   // first triangle (global) of this mesh
    uint32_t ntris;
    uint32_t ts;         // vertex time samples
    uint32_t vert_base;  // vertex v, key k at verts[vert_base + v * ts + k]
    uint32_t has_normals;
    uint32_t normal_base;
    uint32_t pad;
};
struct __align__(16) GLight {  // rectangle or sphere light
    uint32_t key_base;  // dims (float2 rect / float radius in .x) and colors at key_base + k
    uint32_t nkeys;
    float energy;       // approximate_energy
    uint32_t pad;
};
struct __align__(16) GLightTreeNode {
    uint32_t leaf;
    uint32_t index;     // leaf: light instance slot; inner: first child node
    uint32_t nchild;
    uint32_t bounds_base;
    uint32_t nbounds;
    float energy;
    uint32_t pad[2];
};
struct __align__(16) GDistant {
    uint32_t key_base, nkeys;
    float energy;
    uint32_t is_static;  // one key: the cone constants below are valid
    double ctm;          // cos(radius), evaluated by the host in f64
    float sai;           // (float)(1 / (2 pi (1 - cos(radius)))) = solid-angle inverse = cone pdf
    float pad;
};

// Everything the kernels need, passed by value as a kernel argument.
struct GScene {
    const GNode *nodes;
    const GBounds4 *bounds_ext;
    const GNodeH *nodes_h;         // FP16 variant (same indices as nodes)
    const uint4 *tri_idx;          // (v0, v2, v1, original index) per triangle, BVH order
    const float4 *tris;            // 3 x float4 per static triangle (w of the first = original index bits)
    const float4 *verts;           // xyz per vertex key
    const float4 *normals;
    const GMesh *meshes;
    const GInstance *instances;    // instance-BVH order (slot)
    const float4 *xforms;          // 3 float4 rows per transform
    const float4 *xforms_inv;      // precomputed inverses of single-key instance transforms
    const GShader *shaders;
    const GLight *lights;          // rect + sphere lights
    const float2 *light_dims;      // per key: rect (w, h); sphere (r, 0)
    const GColor *light_colors;
    const GLightTreeNode *lt_nodes;
    const float4 *lt_bounds;       // 2 float4 per bbox (min, max)
    const GInstance *light_instances;  // by light-tree leaf index
    const GDistant *distant;
    const float *distant_radii;
    const float4 *distant_dirs;
    const GColor *distant_colors;
    const float *spec_tables;      // PSY_SPEC_TABLE floats per indexed colour (see PSY_COLOR_KIND_MASK)
    const float4 *cam_xf;          // 3 float4 per key
    const float *cam_tfov, *cam_ap, *cam_fd;
    uint32_t top_root;             // child reference of the instance BVH root (PSY_REF_NONE: empty)
    uint32_t n_instances, n_light_instances, n_distant;
    uint32_t lt_empty;
    uint32_t n_cam_xf, n_cam_tfov, n_cam_ap, n_cam_fd;
    GColor background;
    uint32_t width, height, spp, seed, max_bounces;
    uint32_t use_fp16;
    uint32_t ordered_slabs;      // every child box of every node has lo <= hi on each axis (host-checked)
    uint32_t static_fast;        // nodes without motion keys (FP32 or FP16), ordered boxes, every mesh static
                                 // and every mesh instance untransformed: the static-scene traversal applies
    float distant_energy_total;  // sum of distant light energies
    float lt_root_energy;
    float4 bounds_min, bounds_inv_extent;  // scene box, for the ray sort key's origin cell
};
