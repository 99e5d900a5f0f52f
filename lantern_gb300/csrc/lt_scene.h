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
    int16_t has_normals;
    int16_t has_texcoords;
    uint32_t first_tri;   // global index of the mesh's first triangle
};

constexpr int32_t kAlbedoConstant = -1, kAlbedoUV = -2;  // MaterialInfo::tex; >= 0: image index

struct alignas(16) MaterialInfo {
    int32_t bsdf;
    int32_t medium;
    float ior;
    int32_t tex;          // kAlbedoConstant, kAlbedoUV or an index into the scene's images
    float albedo[4];
};

struct alignas(16) ImageInfo {
    uint64_t offset;      // first byte in the scene's texel array
    uint32_t width, height, channels, pad;
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

// An emissive mesh whose light data the device computes (device scene setup):
// its vertices and triangles in the concatenated arrays, its first light
// triangle, and AreaLight's constructor arguments.
struct alignas(16) LightSource {
    uint32_t geom, vbase, tbase, nverts, ntris, tri_first;
    float color[3];
    float power;
    uint32_t pad[2];
};

// Light setup of one emissive mesh, shared by the host and device builds so
// that both run the same float operations in the same order (no fused
// multiply-add on either side). `pos` holds the mesh's world-space vertices,
// `idx` its mesh-local triangle indices.
//
// Area: the sequential sum of 0.5 * |(a - b) x (a - c)| over the triangles
// (scene.cpp:527-534).
LT_HD float light_area(const float *pos, const uint32_t *idx, uint32_t ntris) {
    float area = 0.0f;
    for (uint32_t t = 0; t < ntris; ++t) {
        const uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        const v3 a = ld3(pos + 3 * (size_t)i0), b = ld3(pos + 3 * (size_t)i1), c = ld3(pos + 3 * (size_t)i2);
        area += 0.5f * length(cross(a - b, a - c));
    }
    return area;
}

// CalculateBoundingSphere (scene.cpp:49-80): two Ritter passes and a
// tightening pass over the vertices.
LT_HD void light_bounding_sphere(const float *p, uint32_t n, float out[4]) {
    v3 c = ld3(p);
    float r = 0.0001f;
    for (int pass = 0; pass < 2; ++pass) {
        for (uint32_t j = 0; j < n; ++j) {
            v3 pos = ld3(p + 3 * (size_t)j);
            float len = length(pos - c);
            if (len > r) {
                float a = len / r;
                float a2 = a * a;
                r = 0.5f * (a + 1 / a) * r;
                c = (c * (1 + 1 / a2) + pos * (1 - 1 / a2)) * 0.5f;
            }
        }
    }
    for (uint32_t j = 0; j < n; ++j) {
        v3 pos = ld3(p + 3 * (size_t)j);
        v3 d = pos - c;
        float len = length(d);
        if (len > r) {
            r = (r + len) / 2.0f;
            c = c + d * ((len - r) / len);
        }
    }
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = r;
}

// AreaLight's radiance (area_light.h:16-21): color * radiantPower * (float)M_1_PI / area.
LT_HD v3 light_radiance(const float color[3], float power, float area) {
    return ((ld3(color) * power) * kInvPi) / area;
}

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

// Compressed 8-wide node, 80 bytes (five 16-byte words), after Ylitie, Karras
// and Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed
// Wide BVHs" (HPG 2017): child boxes quantised to 8 bits per plane on a grid
// with origin p and per-axis power-of-two cell size 2^(e - 127).
//  [0] p.x p.y p.z | e.x e.y e.z imask        imask bit s: slot s is an inner node
//  [1] base_child base_tri | meta[0..7]       inner children: nodes base_child + rank among
//                                             inner slots; leaves: triangles base_tri + (meta & 31),
//                                             count = popcount(meta >> 5) (1..3, unary)
//  [2] qlo.x[8] qlo.y[8]  [3] qlo.z[8] qhi.x[8]  [4] qhi.y[8] qhi.z[8]
// Slot s holds the child that lies furthest along the octant direction whose
// negative axes are the bits of s, so a ray whose direction has sign bits o
// meets the children roughly in decreasing order of (s ^ o).
struct alignas(16) Bvh8Node {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t base_child, base_tri;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(Bvh8Node) == 80, "Bvh8Node is five 16-byte words");

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
    std::vector<float> vtex;         // 2 floats per global vertex (0 where a mesh has none)
    std::vector<uint8_t> texels;     // all image textures, 8-bit samples
    std::vector<ImageInfo> images;
    // BVH
    std::vector<BvhNode> nodes;
    std::vector<float> leaf_tris;    // 12 floats per triangle in leaf order: v0,prim | e1,0 | e2,0
    std::vector<float> light_tris;   // the emissive meshes' triangles, same 12-float layout
    std::vector<LightSource> light_src;  // device setup: what the device computes the lights from
    uint32_t max_depth = 0;          // deepest leaf (the traversal stack holds 64)
    float build_ms = 0.0f;
};

// Fills `out` from a scene description. Returns LT_OK or an error with `err`.
// With host_setup false the per-triangle arrays (tri_v0e1e2, tri_vidx), the
// vertex arrays (vnormal, vtex) and the lights' geometry (area, bounding
// sphere, radiance, light_tris) stay empty: the device computes them
// (setup_triangles_gpu, setup_lights_gpu) from light_src; the lights' indices,
// the tables and tri_geom are always filled.
lt_status build_host_scene(const lt_scene_desc *desc, HostScene *out, std::string *err, bool host_setup = true);

// transform * (p, 1) for n points (a row-major 4x4 matrix, float arithmetic of
// the reference's transform).
void transform_points(const float *m, const float *in, uint32_t n, float *out);

// Binned-SAH BVH2 (32 bins, at most 4 triangles per leaf) over the scene's
// triangles; fills nodes and leaf_tris.
void build_bvh(HostScene *s);

// Collapses a BVH2 (nodes in BvhNode layout, triangles in leaf order) into
// compressed 8-wide nodes: every wide node takes the BVH2 children of one node
// and keeps opening its largest-area inner child while the children fit in 8
// slots (a leaf needs one slot per 3 triangles); children are placed by octant,
// boxes quantised conservatively. tris8 receives the triangles in wide-leaf
// order (same 12-float layout). Returns the depth of the wide tree.
uint32_t build_bvh8(const std::vector<BvhNode> &nodes, const std::vector<float> &leaf_tris,
                    std::vector<Bvh8Node> *out, std::vector<float> *tris8);

// 4-wide BVH node, 128 bytes (eight 16-byte words), the four child boxes as
// structure of arrays: [0] lo.x [1] hi.x [2] lo.y [3] hi.y [4] lo.z [5] hi.z of
// children 0-3, [6] child refs (BVH2 encoding: inner >= 0, leaf < 0; an unused
// slot holds kEmptyRef4), [7] number of children, 0, 0, 0.
constexpr int32_t kEmptyRef4 = 0x7FFFFFFF;
struct alignas(16) Bvh4Node {
    float lo_x[4], hi_x[4], lo_y[4], hi_y[4], lo_z[4], hi_z[4];
    int32_t ref[4];
    uint32_t count, pad[3];
};

// Collapses a BVH2 into 4-wide nodes: each 4-wide node takes the children of
// one BVH2 node, opening every inner child into its two children (2-4 slots).
// Leaf references are the BVH2's, so the BVH2's leaf-ordered triangles serve
// both trees. Returns the depth of the 4-wide tree.
uint32_t build_bvh4(const std::vector<BvhNode> &nodes, std::vector<Bvh4Node> *out);

// PNG decoding as stbi_load(path, &w, &h, &n, 0) returns it (lt_image.cpp).
lt_status decode_png(const uint8_t *file, size_t size, std::vector<uint8_t> *data, uint32_t *w, uint32_t *h,
                     uint32_t *n, std::string *err);
lt_status load_png(const std::string &path, std::vector<uint8_t> *data, uint32_t *w, uint32_t *h, uint32_t *n,
                   std::string *err);

// Scene::ParseJSON subset (scene.cpp:154-446) into a description whose
// arrays live in `storage`.
struct JsonSceneStorage {
    std::vector<lt_material_desc> materials;
    std::vector<lt_image_desc> images;
    std::vector<std::vector<uint8_t>> bytes;
    std::vector<lt_medium_desc> media;
    std::vector<lt_mesh_desc> meshes;
    std::vector<std::vector<float>> floats;
    std::vector<std::vector<uint32_t>> uints;
};
lt_status load_scene_json(const char *path, lt_scene_desc *desc, JsonSceneStorage *storage, std::string *err);

}  // namespace lt
