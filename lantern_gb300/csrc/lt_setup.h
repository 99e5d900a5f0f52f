// lt_setup.h -- device-side triangle setup (lt_setup.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lt_scene.h"

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

// Area lights from the transformed vertices (pos, after setup_triangles_gpu)
// and the mesh-local indices (idx): lights[i] and the light triangles of
// src[i] (light_tris, 3 float4 per triangle from src[i].tri_first), with the
// host build's arithmetic (lt_scene.h: light_area, light_bounding_sphere,
// light_radiance). src is a device array of nlights entries.
cudaError_t setup_lights_gpu(const float *pos, const uint32_t *idx, const LightSource *src, uint32_t nlights,
                             LightInfo *lights, float4 *light_tris, cudaStream_t st);

}  // namespace lt
