// GPU build of a static mesh's BVH4 (bvh_build.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "psy_layout.h"

struct LbvhInput {
    const float *verts;      // host, num_verts * 3 (one time sample)
    uint32_t num_verts;
    const uint32_t *indices; // host, ntris * 3
    uint32_t ntris;
    uint32_t node_base;      // global node index the mesh's first BVH4 node will get
    uint32_t tri_base;       // global index of the mesh's first triangle
};
struct LbvhOutput {
    uint32_t root = 0;            // child reference of the mesh root (node or leaf)
    uint32_t node_count = 0;
    uint32_t depth = 0;           // BVH4 levels
    bool ordered = true;          // every child box has lo <= hi
    std::vector<GNode> nodes;     // node_count nodes, the root first
    std::vector<uint32_t> order;  // original triangle index at each position of the tree order
};

// Builds on the current device, on stream st, and returns when done.
cudaError_t lbvh_build_mesh(const LbvhInput &in, LbvhOutput &out, cudaStream_t st);
