// rtc_shim.cpp -- project implementation of the 18 Embree 3 entry points that
// Lantern's scene code calls (scene.cpp:39,46,86,98,116-140,196-198,451-582,605),
// so that the reference integrator links without Embree.
//
// TEST INFRASTRUCTURE ONLY (reference build for the CPU oracle / baseline).
// Embree 3.5 cannot be built from the reference snapshot (its kernels/builders
// directory is missing, and it is x86-only). Geometry buffers are stored as
// given; rtcCommitScene hands every attached triangle mesh to the oracle in
// oracle/lt_oracle.c, whose BVH2 and Moeller-Trumbore test follow Embree's
// arithmetic (triangle_intersector_moeller.h:75-112). rtcIntersect1 then writes
// tfar/u/v/Ng/primID/geomID as Embree does for a closest hit.
#include "embree3/rtcore.h"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../lt_oracle.h"

struct RTCDeviceTy { int refs; };

struct RTCGeometryTy {
    int refs = 1;
    RTCGeometryType type;
    struct Buf { std::vector<unsigned char> data; size_t stride = 0, count = 0; };
    Buf vertex, index, attr[2];
};

struct RTCSceneTy {
    int refs = 1;
    std::vector<RTCGeometryTy *> geoms;
    orc_scene *oracle = nullptr;
    std::vector<float> tri_ng;  // Ng = cross(e2, e1) per global triangle
};

// Closest-hit queries made through rtcIntersect1 (ray counters for Mrays/s).
extern "C" std::atomic<unsigned long long> lt_ref_ray_count;
std::atomic<unsigned long long> lt_ref_ray_count(0);

extern "C" {

RTCDevice rtcNewDevice(const char *) { return new RTCDeviceTy{1}; }
void rtcReleaseDevice(RTCDevice d) { delete d; }

RTCScene rtcNewScene(RTCDevice) { return new RTCSceneTy(); }
void rtcSetSceneFlags(RTCScene, enum RTCSceneFlags) {}
void rtcSetSceneBuildQuality(RTCScene, enum RTCBuildQuality) {}

void rtcReleaseScene(RTCScene s) {
    if (!s) return;
    for (auto *g : s->geoms)
        if (--g->refs == 0) delete g;
    orc_scene_free(s->oracle);
    delete s;
}

RTCGeometry rtcNewGeometry(RTCDevice, enum RTCGeometryType type) {
    if (type != RTC_GEOMETRY_TYPE_TRIANGLE) {
        std::fprintf(stderr, "rtc shim: only triangle geometry is supported\n");
        std::abort();
    }
    auto *g = new RTCGeometryTy();
    g->type = type;
    return g;
}
void rtcSetGeometryBuildQuality(RTCGeometry, enum RTCBuildQuality) {}
void rtcSetGeometryTimeStepCount(RTCGeometry, unsigned int) {}
void rtcSetGeometryVertexAttributeCount(RTCGeometry, unsigned int) {}
void rtcCommitGeometry(RTCGeometry) {}
void rtcReleaseGeometry(RTCGeometry g) {
    if (g && --g->refs == 0) delete g;
}

void *rtcSetNewGeometryBuffer(RTCGeometry g, enum RTCBufferType type, unsigned int slot, enum RTCFormat,
                              size_t stride, size_t count) {
    RTCGeometryTy::Buf *b = nullptr;
    if (type == RTC_BUFFER_TYPE_VERTEX) b = &g->vertex;
    else if (type == RTC_BUFFER_TYPE_INDEX) b = &g->index;
    else if (type == RTC_BUFFER_TYPE_VERTEX_ATTRIBUTE && slot < 2) b = &g->attr[slot];
    if (!b) {
        std::fprintf(stderr, "rtc shim: unsupported buffer\n");
        std::abort();
    }
    b->stride = stride;
    b->count = count;
    b->data.assign(stride * count + 16, 0);
    return b->data.data();
}

unsigned int rtcAttachGeometry(RTCScene s, RTCGeometry g) {
    g->refs++;
    s->geoms.push_back(g);
    return (unsigned int)(s->geoms.size() - 1);
}

RTCGeometry rtcGetGeometry(RTCScene s, unsigned int id) { return id < s->geoms.size() ? s->geoms[id] : nullptr; }

void rtcCommitScene(RTCScene s) {
    orc_scene_free(s->oracle);
    s->oracle = orc_scene_new();
    const float white[3] = {1, 1, 1};
    int mat = orc_add_material(s->oracle, ORC_BSDF_LAMBERT, white, 1.0f, -1);
    for (auto *g : s->geoms) {
        size_t nv = g->vertex.count, nt = g->index.count;
        std::vector<float> pos(nv * 3);
        for (size_t i = 0; i < nv; ++i)
            std::memcpy(&pos[3 * i], g->vertex.data.data() + i * g->vertex.stride, 3 * sizeof(float));
        std::vector<uint32_t> idx(nt * 3);
        for (size_t i = 0; i < nt; ++i)
            std::memcpy(&idx[3 * i], g->index.data.data() + i * g->index.stride, 3 * sizeof(uint32_t));
        std::vector<float> nrm;
        if (g->attr[0].count == nv && nv) {
            nrm.resize(nv * 3);
            for (size_t i = 0; i < nv; ++i)
                std::memcpy(&nrm[3 * i], g->attr[0].data.data() + i * g->attr[0].stride, 3 * sizeof(float));
        }
        orc_add_mesh(s->oracle, pos.data(), (uint32_t)nv, nrm.empty() ? nullptr : nrm.data(), idx.data(),
                     (uint32_t)nt, mat, nullptr, 0.0f);
    }
    orc_scene_commit(s->oracle);
}

void rtcIntersect1(RTCScene s, struct RTCIntersectContext *, struct RTCRayHit *rh) {
    lt_ref_ray_count.fetch_add(1, std::memory_order_relaxed);
    if (!s->oracle) return;
    float org[3] = {rh->ray.org_x, rh->ray.org_y, rh->ray.org_z};
    float dir[3] = {rh->ray.dir_x, rh->ray.dir_y, rh->ray.dir_z};
    float t, u, v;
    uint32_t prim, geom, local;
    if (!orc_intersect1(s->oracle, org, dir, rh->ray.tnear, rh->ray.tfar, &t, &u, &v, &prim, &geom, &local))
        return;
    // Ng = cross(e2, e1) of the hit triangle (triangle_intersector_moeller.h:122)
    RTCGeometryTy *g = s->geoms[geom];
    const uint32_t *ix = (const uint32_t *)(g->index.data.data() + local * g->index.stride);
    const float *p0 = (const float *)(g->vertex.data.data() + ix[0] * g->vertex.stride);
    const float *p1 = (const float *)(g->vertex.data.data() + ix[1] * g->vertex.stride);
    const float *p2 = (const float *)(g->vertex.data.data() + ix[2] * g->vertex.stride);
    float e1[3] = {p0[0] - p1[0], p0[1] - p1[1], p0[2] - p1[2]};
    float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    rh->hit.Ng_x = e2[1] * e1[2] - e2[2] * e1[1];
    rh->hit.Ng_y = e2[2] * e1[0] - e2[0] * e1[2];
    rh->hit.Ng_z = e2[0] * e1[1] - e2[1] * e1[0];
    rh->ray.tfar = t;
    rh->hit.u = u;
    rh->hit.v = v;
    rh->hit.primID = local;
    rh->hit.geomID = geom;
    rh->hit.instID[0] = RTC_INVALID_GEOMETRY_ID;
}

// rtcInterpolate for triangle vertex attributes: P = (1-u-v)*a0 + u*a1 + v*a2
void rtcInterpolate(const struct RTCInterpolateArguments *a) {
    RTCGeometryTy *g = a->geometry;
    const RTCGeometryTy::Buf *b = nullptr;
    if (a->bufferType == RTC_BUFFER_TYPE_VERTEX_ATTRIBUTE && a->bufferSlot < 2) b = &g->attr[a->bufferSlot];
    else if (a->bufferType == RTC_BUFFER_TYPE_VERTEX) b = &g->vertex;
    const uint32_t *ix = (const uint32_t *)(g->index.data.data() + a->primID * g->index.stride);
    const float *q0 = (const float *)(b->data.data() + ix[0] * b->stride);
    const float *q1 = (const float *)(b->data.data() + ix[1] * b->stride);
    const float *q2 = (const float *)(b->data.data() + ix[2] * b->stride);
    float w = 1.0f - a->u - a->v;
    for (unsigned i = 0; i < a->valueCount; ++i) {
        if (a->P) a->P[i] = q0[i] * w + q1[i] * a->u + q2[i] * a->v;
        if (a->dPdu) a->dPdu[i] = q1[i] - q0[i];
        if (a->dPdv) a->dPdv[i] = q2[i] - q0[i];
    }
}

}  // extern "C"
