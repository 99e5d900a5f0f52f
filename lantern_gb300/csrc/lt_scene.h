// lt_scene.h -- host-side scene: flat arrays built from lt_scene_desc, the
// light data of the reference's AddLMF / AreaLight, and the BVH in the layout
// the traversal kernels read.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "lantern_gpu.h"
#include "lt_math.h"

namespace lt {

struct alignas(16) GeomInfo {
    int32_t material;
    int32_t light;        // index into lights, or -1
    int32_t has_normals;
    uint32_t first_tri;   // global index of the mesh's first triangle
};

struct alignas(16) MaterialInfo {
    int32_t bsdf;
    int32_t medium;
    float ior;
    float pad;
    float albedo[4];
};

struct alignas(16) MediumInfo {
    int32_t type;
    float g;
    float sigma_s_mean;  // HG: distance-sampling coefficient (mean of sigma_s)
    float pad;
    float sigma_a[4];
    float sigma_s[4];
};

struct alignas(16) LightInfo {
    int32_t geom;
    float area;
    uint32_t tri_first;   // first of the light's triangles in HostScene::light_tris
    uint32_t tri_count;
    float radiance[4];
    float sphere[4];     // bounding sphere centre, radius
};

// BVH2 node for the device, 64 bytes (four float4):
//  [0] c0.lo.x c0.hi.x c0.lo.y c0.hi.y   [1] c1.lo.x c1.hi.x c1.lo.y c1.hi.y
//  [2] c0.lo.z c0.hi.z c1.lo.z c1.hi.z   [3] c0 ref, c1 ref, c0 count, c1 count
// ref >= 0: inner node index; ref < 0: leaf, ~ref = (first triangle in leaf
// order) << 3 | triangle count.
constexpr uint32_t kLeafBits = 3;
LT_HD int32_t leaf_ref(uint32_t first, uint32_t count) { return ~(int32_t)((first << kLeafBits) | count); }

struct alignas(16) BvhNode {
    float a[4], b[4], c[4];
    int32_t ref[2];
    uint32_t count[2];
};

struct HostScene {
    Camera camera;
    TentFilter filter;
    v3 background;
    std::vector<GeomInfo> geoms;
    std::vector<MaterialInfo> materials;
    std::vector<MediumInfo> media;
    std::vector<LightInfo> lights;
    // global triangle order = mesh order, then index order within the mesh
    std::vector<float> tri_v0e1e2;   // 9 floats per triangle: v0, v0 - v1, v2 - v0
    std::vector<uint32_t> tri_geom;
    std::vector<uint32_t> tri_vidx;  // 3 global vertex indices per triangle
    std::vector<float> vnormal;      // 3 floats per global vertex
    // BVH
    std::vector<BvhNode> nodes;
    std::vector<float> leaf_tris;    // 12 floats per triangle in leaf order: v0,prim | e1,0 | e2,0
    std::vector<float> light_tris;   // the emissive meshes' triangles, same 12-float layout
    uint32_t max_depth = 0;          // deepest leaf (the traversal stack holds 64)
    float build_ms = 0.0f;
};

// Fills `out` from a scene description. Returns LT_OK or an error with `err`.
lt_status build_host_scene(const lt_scene_desc *desc, HostScene *out, std::string *err);

// Binned-SAH BVH2 (32 bins, at most 4 triangles per leaf) over the scene's
// triangles; fills nodes and leaf_tris.
void build_bvh(HostScene *s);

// Scene::ParseJSON subset (scene.cpp:154-446) into a description whose
// arrays live in `storage`.
struct JsonSceneStorage {
    std::vector<lt_material_desc> materials;
    std::vector<lt_medium_desc> media;
    std::vector<lt_mesh_desc> meshes;
    std::vector<std::vector<float>> floats;
    std::vector<std::vector<uint32_t>> uints;
};
lt_status load_scene_json(const char *path, lt_scene_desc *desc, JsonSceneStorage *storage, std::string *err);

}  // namespace lt
