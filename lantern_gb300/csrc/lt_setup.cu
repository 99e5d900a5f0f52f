// lt_setup.cu -- triangle setup on the device for lt_scene_create.
//
// What the reference's AddLMF / AddMesh do per vertex and triangle
// (scene.cpp:451-582) when the scene is handed to Embree: every position is
// moved by the mesh's transform, and each triangle is stored for intersection.
// Here the raw mesh arrays are uploaded once and two kernels produce the arrays
// the GPU BVH builder and the wavefront kernels read: positions transformed in
// place (transform * (p, 1), the reference's float arithmetic, no fused
// multiply-add), then per triangle (v0, v0 - v1, v2 - v0) and its three global
// vertex indices. A third kernel sets up the area lights from the transformed
// vertices: each emissive mesh's triangles for the light-connection test, its
// area, bounding sphere and radiance. Those are sequential float sums in the
// reference (scene.cpp:49-80, 527-534; area_light.h:16-21), so one thread per
// light runs them in the reference's order with the host build's code
// (lt_scene.h) and matches it bit for bit; the light's triangles are written
// by all threads of its block.
#include <cuda_runtime.h>

#include "lt_device.h"
#include "lt_setup.h"

namespace lt {

namespace {

// the mesh owning element `i` of a sequence split at the meshes' `first` offsets
__device__ __forceinline__ uint32_t mesh_of(const MeshSetup *m, uint32_t n, uint32_t i, bool by_tri) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((by_tri ? m[mid].tbase : m[mid].vbase) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(256) k_transform(float *pos, const MeshSetup *meshes, uint32_t nmesh,
                                                   uint32_t nvert) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nvert; v += gridDim.x * blockDim.x) {
        const MeshSetup &M = meshes[mesh_of(meshes, nmesh, v, false)];
        if (!M.has_transform) continue;
        float *p = pos + 3 * (size_t)v;
        const float x = p[0], y = p[1], z = p[2];
        const float *m = M.m;
        p[0] = ((x * m[0] + y * m[1]) + z * m[2]) + 1.0f * m[3];
        p[1] = ((x * m[4] + y * m[5]) + z * m[6]) + 1.0f * m[7];
        p[2] = ((x * m[8] + y * m[9]) + z * m[10]) + 1.0f * m[11];
    }
}

__global__ void __launch_bounds__(256) k_setup_tris(const float *__restrict__ pos, const uint32_t *__restrict__ idx,
                                                    const MeshSetup *meshes, uint32_t nmesh, uint32_t ntri,
                                                    float *__restrict__ tri9, uint32_t *__restrict__ vidx) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntri; t += gridDim.x * blockDim.x) {
        const uint32_t vb = meshes[mesh_of(meshes, nmesh, t, true)].vbase;
        const uint32_t i0 = vb + idx[3 * (size_t)t], i1 = vb + idx[3 * (size_t)t + 1], i2 = vb + idx[3 * (size_t)t + 2];
        const v3 a = ld3(pos + 3 * (size_t)i0), b = ld3(pos + 3 * (size_t)i1), c = ld3(pos + 3 * (size_t)i2);
        const v3 e1 = a - b, e2 = c - a;
        float *o = tri9 + 9 * (size_t)t;
        o[0] = a.x; o[1] = a.y; o[2] = a.z;
        o[3] = e1.x; o[4] = e1.y; o[5] = e1.z;
        o[6] = e2.x; o[7] = e2.y; o[8] = e2.z;
        vidx[3 * (size_t)t] = i0;
        vidx[3 * (size_t)t + 1] = i1;
        vidx[3 * (size_t)t + 2] = i2;
    }
}

// One block per light: the light's triangles in the 12-float layout of the
// traversal (v0, global triangle index | e1, 0 | e2, 0), then, by thread 0,
// area, bounding sphere and radiance.
__global__ void __launch_bounds__(128) k_setup_lights(const float *__restrict__ pos, const uint32_t *__restrict__ idx,
                                                      const LightSource *__restrict__ src, LightInfo *lights,
                                                      float4 *light_tris) {
    const LightSource L = src[blockIdx.x];
    const float *mpos = pos + 3 * (size_t)L.vbase;
    const uint32_t *midx = idx + 3 * (size_t)L.tbase;
    for (uint32_t t = threadIdx.x; t < L.ntris; t += blockDim.x) {
        const uint32_t i0 = midx[3 * t], i1 = midx[3 * t + 1], i2 = midx[3 * t + 2];
        const v3 a = ld3(mpos + 3 * (size_t)i0), b = ld3(mpos + 3 * (size_t)i1), c = ld3(mpos + 3 * (size_t)i2);
        const v3 e1 = a - b, e2 = c - a;
        float4 *o = light_tris + 3 * (size_t)(L.tri_first + t);
        o[0] = make_float4(a.x, a.y, a.z, __uint_as_float(L.tbase + t));
        o[1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
        o[2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
    }
    if (threadIdx.x == 0) {
        LightInfo li;
        li.geom = (int32_t)L.geom;
        li.tri_first = L.tri_first;
        li.tri_count = L.ntris;
        li.area = light_area(mpos, midx, L.ntris);
        li.sphere[0] = li.sphere[1] = li.sphere[2] = li.sphere[3] = 0.0f;
        if (L.nverts) light_bounding_sphere(mpos, L.nverts, li.sphere);
        const v3 rad = light_radiance(L.color, L.power, li.area);
        li.radiance[0] = rad.x;
        li.radiance[1] = rad.y;
        li.radiance[2] = rad.z;
        li.radiance[3] = 0.0f;
        lights[blockIdx.x] = li;
    }
}

}  // namespace

cudaError_t setup_lights_gpu(const float *pos, const uint32_t *idx, const LightSource *src, uint32_t nlights,
                             LightInfo *lights, float4 *light_tris, cudaStream_t st) {
    if (!nlights) return cudaSuccess;
    k_setup_lights<<<nlights, 128, 0, st>>>(pos, idx, src, lights, light_tris);
    return cudaGetLastError();
}

cudaError_t setup_triangles_gpu(float *pos, const uint32_t *idx, const MeshSetup *meshes, uint32_t nmesh,
                                uint32_t nvert, uint32_t ntri, float *tri9, uint32_t *vidx, cudaStream_t st) {
    if (nvert) {
        const uint32_t blocks = (nvert + 255) / 256 < 65535 ? (nvert + 255) / 256 : 65535;
        k_transform<<<blocks, 256, 0, st>>>(pos, meshes, nmesh, nvert);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (ntri) {
        const uint32_t blocks = (ntri + 255) / 256 < 65535 ? (ntri + 255) / 256 : 65535;
        k_setup_tris<<<blocks, 256, 0, st>>>(pos, idx, meshes, nmesh, ntri, tri9, vidx);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

}  // namespace lt
