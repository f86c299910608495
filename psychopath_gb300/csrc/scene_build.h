// Host-side scene build: PsySceneDesc -> flat device layout (psy_layout.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/psy_gpu.h"
#include "psy_layout.h"

// Host copy of everything that goes to the device, plus build facts.
struct HostScene {
    std::vector<GNode> nodes;
    std::vector<GBounds4> bounds_ext;
    std::vector<GNodeH> nodes_h;
    std::vector<uint4> tri_idx;
    std::vector<float4> tris;
    std::vector<float4> verts, normals;
    std::vector<GMesh> meshes;
    std::vector<GInstance> instances;
    std::vector<float4> xforms, xforms_inv;
    std::vector<GShader> shaders;
    std::vector<GLight> lights;
    std::vector<float2> light_dims;
    std::vector<GColor> light_colors;
    std::vector<GLightTreeNode> lt_nodes;
    std::vector<float4> lt_bounds;
    std::vector<GInstance> light_instances;
    std::vector<GDistant> distant;
    std::vector<float> distant_radii;
    std::vector<float4> distant_dirs;
    std::vector<GColor> distant_colors;
    std::vector<float4> cam_xf;
    std::vector<float> cam_tfov, cam_ap, cam_fd;
    uint32_t top_root = PSY_REF_NONE;
    uint32_t max_stack = 0;   // worst-case traversal stack entries
    float distant_energy_total = 0.0f;
    float lt_root_energy = 0.0f;
    bool lt_empty = true;
    float scene_min[3] = {0, 0, 0}, scene_max[3] = {0, 0, 0};  // union of instance bounds
    GColor background{};
    std::vector<float4> spec_xyz;  // the XYZ value of each indexed colour (spectrum tables)
    uint32_t width = 0, height = 0, spp = 0, seed = 0, max_bounces = 2;
    // per mesh object (desc order): BVH-order original triangle indices and BVH4 node count
    std::vector<std::vector<uint32_t>> mesh_tri_order;
    std::vector<uint32_t> mesh_node_count;
    std::vector<int32_t> object_to_mesh;
};

#include <functional>

#include "bvh_build.h"

// Builds one static mesh's BVH4 on the GPU (PSY_BVH_GPU); returns PSY_OK or
// a PSY_E_* code with a message in `err`.
using GpuMeshBuild = std::function<int(const LbvhInput &, LbvhOutput &, std::string &)>;

// Validates the description and builds the host scene.  Returns PSY_OK or a
// PSY_E_* code with a message in `err`.  gpu_build is needed when the
// options ask for GPU-built mesh BVHs (a host-only build then fails with
// PSY_E_UNSUPPORTED).
// serial: build every BVH on the calling thread (large subtrees otherwise go
// to worker threads; the result is the same).
int build_host_scene(const PsySceneDesc *d, const PsySceneOptions *opts, HostScene &hs, std::string &err,
                     const GpuMeshBuild *gpu_build = nullptr, bool serial = false);

// rec709_to_xyz((1, 0, 1)) in the reference's f32 arithmetic (the colour of
// the tracer's shader for instances that have none).
void unassigned_magenta_xyz(float out[3]);

// The XYZ -> rec709 (equal-energy white) matrix of the reference's image
// output, row-major, as f32 constants.
void xyz_to_rec709_e_matrix(float out[9]);
