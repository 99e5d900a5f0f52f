// lt_bvh_gpu.h -- the GPU BVH builder (lt_bvh_gpu.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lt_scene.h"

namespace lt {

struct GpuBvh {
    void *nodes;        // BvhNode array (device), num_nodes entries
    void *leaf_tris;    // leaf-ordered triangles (device), 3 float4 each
    uint32_t num_nodes;
    uint32_t max_depth; // deepest leaf
    float build_ms;     // device time of the build
};

// Builds the BVH of n > 4 triangles given as 9 floats each (v0, v0 - v1,
// v2 - v0) on the device. The caller owns out->nodes and out->leaf_tris.
cudaError_t build_bvh_gpu(const float *d_tri, uint32_t n, GpuBvh *out, cudaStream_t st);

}  // namespace lt
