// lt_setup.h -- device-side triangle setup (lt_setup.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lt {

// One mesh of the concatenated vertex / triangle arrays.
struct MeshSetup {
    uint32_t vbase, tbase;   // first global vertex and triangle
    uint32_t nverts, ntris;
    float m[12];             // rows 0-2 of the row-major transform
    uint32_t has_transform;
    uint32_t pad[3];
};

// pos: 3 floats per global vertex, transformed in place; idx: 3 mesh-local
// vertex indices per global triangle (checked by the host). Writes tri9 (v0,
// v0 - v1, v2 - v0 per triangle) and vidx (3 global vertex indices). meshes
// is a device array of nmesh entries in vbase / tbase order.
cudaError_t setup_triangles_gpu(float *pos, const uint32_t *idx, const MeshSetup *meshes, uint32_t nmesh,
                                uint32_t nvert, uint32_t ntri, float *tri9, uint32_t *vidx, cudaStream_t st);

}  // namespace lt
