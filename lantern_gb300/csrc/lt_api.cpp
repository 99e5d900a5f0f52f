// lt_api.cpp -- the C ABI declared in include/lantern_gpu.h.
//
// A context owns a CUDA stream, the device copy of one scene (triangles, BVH,
// shading tables) and the wavefront buffers, which are sized once and reused.
// lt_render queues the wavefront: an initial camera-ray launch, then batches of
// (trace, shade, connect) iterations, reading the queue length back once per
// batch until no path is left.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lantern_gpu.h"
#include "lt_device.h"
#include "lt_bvh_gpu.h"
#include "lt_scene.h"

using namespace lt;

struct lt_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string error;
    LaunchShape shape;

    // scene
    bool has_scene = false;
    HostScene host;
    DevScene dev{};
    std::vector<void *> scene_allocs;
    uint64_t scene_bytes = 0;
    uint32_t num_nodes = 0;
    int32_t bvh_builder = LT_BVH_GPU;

    // wavefront
    Wavefront wave;
    WaveCounters *counters_host = nullptr;  // pinned
    uint32_t *isect_fetch = nullptr;        // device ray counter of lt_intersect

    // scratch for host-memory calls
    void *scratch = nullptr;
    size_t scratch_bytes = 0;

    lt_render_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // stage timing: one event before each stage launch and one after the last
    std::vector<cudaEvent_t> stage_events;
    std::vector<int> stage_of_event;
};

static thread_local std::string g_create_error;

static lt_status fail(lt_ctx *c, lt_status st, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->error = buf;
    else g_create_error = buf;
    return st;
}

#define CUDA_TRY(c, expr)                                                                           \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(c, e_ == cudaErrorMemoryAllocation ? LT_ERR_OOM : LT_ERR_CUDA, "%s: %s (%s:%d)", \
                        #expr, cudaGetErrorString(e_), __FILE__, __LINE__);                         \
    } while (0)

static void free_scene(lt_ctx *c) {
    for (void *p : c->scene_allocs) cudaFree(p);
    c->scene_allocs.clear();
    c->scene_bytes = 0;
    c->has_scene = false;
    c->dev = DevScene{};
}

static void free_wave(lt_ctx *c) {
    if (c->wave.arena) cudaFree(c->wave.arena);
    c->wave = Wavefront{};
}

extern "C" {

int lt_abi_version(void) { return LT_ABI_VERSION; }

lt_status lt_ctx_create(int device, lt_ctx **out) {
    if (!out) return fail(nullptr, LT_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(nullptr, LT_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
    if (device < 0 || device >= n) return fail(nullptr, LT_ERR_INVALID, "device %d out of range", device);
    lt_ctx *c = new (std::nothrow) lt_ctx();
    if (!c) return fail(nullptr, LT_ERR_OOM, "context allocation failed");
    c->device = device;
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&c->counters_host, sizeof(WaveCounters));
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->isect_fetch, 256);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e != cudaSuccess) {
        lt_ctx_destroy(c);
        return fail(nullptr, LT_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    query_launch_shape(device, &c->shape);
    *out = c;
    return LT_OK;
}

void lt_ctx_destroy(lt_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_scene(c);
    free_wave(c);
    if (c->scratch) cudaFree(c->scratch);
    if (c->counters_host) cudaFreeHost(c->counters_host);
    if (c->isect_fetch) cudaFree(c->isect_fetch);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (cudaEvent_t e : c->stage_events) cudaEventDestroy(e);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

const char *lt_last_error(const lt_ctx *c) { return c ? c->error.c_str() : g_create_error.c_str(); }

lt_status lt_set_stream(lt_ctx *c, void *stream) {
    if (!c) return LT_ERR_INVALID;
    c->stream = (cudaStream_t)stream;
    return LT_OK;
}

void *lt_get_stream(const lt_ctx *c) { return c ? (void *)c->stream : nullptr; }

lt_status lt_set_bvh_builder(lt_ctx *c, int32_t builder) {
    if (!c) return LT_ERR_INVALID;
    if (builder != LT_BVH_GPU && builder != LT_BVH_HOST) return fail(c, LT_ERR_INVALID, "unknown BVH builder %d", builder);
    c->bvh_builder = builder;
    return LT_OK;
}

lt_status lt_sync(lt_ctx *c) {
    if (!c) return LT_ERR_INVALID;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return LT_OK;
}

}  // extern "C"

template <typename T>
static lt_status upload(lt_ctx *c, const std::vector<T> &v, const T **dst) {
    size_t bytes = v.size() * sizeof(T);
    void *p = nullptr;
    CUDA_TRY(c, cudaMalloc(&p, bytes ? bytes : 16));
    c->scene_allocs.push_back(p);
    c->scene_bytes += bytes;
    if (bytes) CUDA_TRY(c, cudaMemcpyAsync(p, v.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    *dst = (const T *)p;
    return LT_OK;
}

extern "C" {

lt_status lt_scene_create(lt_ctx *c, const lt_scene_desc *desc) {
    if (!c || !desc) return fail(c, LT_ERR_INVALID, "NULL argument");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    free_scene(c);
    std::string err;
    lt_status st = build_host_scene(desc, &c->host, &err);
    if (st != LT_OK) return fail(c, st, "%s", err.c_str());
    HostScene &h = c->host;
    DevScene &d = c->dev;
    const size_t ntri = h.tri_geom.size();
    if (c->bvh_builder == LT_BVH_GPU && ntri > 4) {
        // binned-SAH build on the device from the triangles in global order
        const float *tri = nullptr;
        if ((st = upload(c, h.tri_v0e1e2, &tri)) != LT_OK) return st;
        GpuBvh gb;
        cudaError_t e = build_bvh_gpu(tri, (uint32_t)ntri, &gb, c->stream);
        cudaFree((void *)tri);
        c->scene_allocs.pop_back();
        c->scene_bytes -= h.tri_v0e1e2.size() * sizeof(float);
        if (e != cudaSuccess)
            return fail(c, e == cudaErrorMemoryAllocation ? LT_ERR_OOM : LT_ERR_CUDA, "GPU BVH build: %s",
                        cudaGetErrorString(e));
        c->scene_allocs.push_back(gb.nodes);
        c->scene_allocs.push_back(gb.leaf_tris);
        c->scene_bytes += (uint64_t)gb.num_nodes * 64 + (uint64_t)ntri * 48;
        d.nodes = (const float4 *)gb.nodes;
        d.tris = (const float4 *)gb.leaf_tris;
        h.nodes.clear();
        h.leaf_tris.clear();
        h.max_depth = gb.max_depth;
        h.build_ms = gb.build_ms;
        c->num_nodes = gb.num_nodes;
    } else {
        build_bvh(&c->host);
        const float *nodes = nullptr, *tris = nullptr;
        std::vector<float> nodes_f(h.nodes.size() * 16);
        memcpy(nodes_f.data(), h.nodes.data(), nodes_f.size() * sizeof(float));
        if ((st = upload(c, nodes_f, &nodes)) != LT_OK) return st;
        if ((st = upload(c, h.leaf_tris, &tris)) != LT_OK) return st;
        d.nodes = (const float4 *)nodes;
        d.tris = (const float4 *)tris;
        c->num_nodes = (uint32_t)h.nodes.size();
    }
    if (h.max_depth >= 64)
        return fail(c, LT_ERR_UNSUPPORTED, "BVH depth %u exceeds the traversal stack", h.max_depth);
    if ((st = upload(c, h.tri_geom, &d.tri_geom)) != LT_OK) return st;
    if ((st = upload(c, h.tri_vidx, &d.tri_vidx)) != LT_OK) return st;
    if ((st = upload(c, h.vnormal, &d.vnormal)) != LT_OK) return st;
    if ((st = upload(c, h.geoms, &d.geoms)) != LT_OK) return st;
    if ((st = upload(c, h.materials, &d.mats)) != LT_OK) return st;
    if ((st = upload(c, h.media, &d.meds)) != LT_OK) return st;
    if ((st = upload(c, h.lights, &d.lights)) != LT_OK) return st;
    const float *ltris = nullptr;
    if ((st = upload(c, h.light_tris, &ltris)) != LT_OK) return st;
    d.light_tris = (const float4 *)ltris;
    d.num_lights = (uint32_t)h.lights.size();
    d.num_tris = (uint32_t)h.tri_geom.size();
    d.background = h.background;
    d.cam = h.camera;
    d.filter = h.filter;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->has_scene = true;
    return LT_OK;
}

lt_status lt_scene_info_get(lt_ctx *c, lt_scene_info *out) {
    if (!c || !out) return LT_ERR_INVALID;
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    out->width = c->host.camera.width;
    out->height = c->host.camera.height;
    out->num_triangles = (uint32_t)c->host.tri_geom.size();
    out->num_meshes = (uint32_t)c->host.geoms.size();
    out->num_lights = (uint32_t)c->host.lights.size();
    out->num_bvh_nodes = c->num_nodes;
    out->num_media = (uint32_t)c->host.media.size();
    out->device_bytes = c->scene_bytes;
    out->build_ms = c->host.build_ms;
    return LT_OK;
}

lt_status lt_scene_mesh_offsets(lt_ctx *c, uint32_t *first, uint32_t capacity) {
    if (!c || !first) return LT_ERR_INVALID;
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    if (capacity < c->host.geoms.size()) return fail(c, LT_ERR_INVALID, "capacity below mesh count");
    for (size_t g = 0; g < c->host.geoms.size(); ++g) first[g] = c->host.geoms[g].first_tri;
    return LT_OK;
}

}  // extern "C"

static lt_status ensure_scratch(lt_ctx *c, size_t bytes) {
    if (c->scratch_bytes >= bytes) return LT_OK;
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    CUDA_TRY(c, cudaMalloc(&c->scratch, bytes));
    c->scratch_bytes = bytes;
    return LT_OK;
}

// Lays the wavefront buffers for `cap` entries out from `base` (each array
// 256-byte aligned); returns the bytes used. With base == nullptr it only sizes.
static size_t carve_wave(char *base, uint32_t cap, Wavefront *w) {
    size_t P = cap, off = 0;
    auto take = [&](size_t n) { char *p = base + off; off += (n + 255) & ~(size_t)255; return p; };
    w->capacity = cap;
    for (int k = 0; k < 2; ++k) {
        PathState &s = w->p[k];
        s.rng = (uint64_t *)take(8 * P);
        s.pixel = (uint32_t *)take(4 * P);
        s.frame = (uint32_t *)take(4 * P);
        s.T = (float *)take(12 * P);
        s.color = (float *)take(12 * P);
        s.bounces = (uint32_t *)take(4 * P);
        s.flags = (uint32_t *)take(4 * P);
        s.iori = (float *)take(4 * P);
    }
    w->ray[0] = (float4 *)take(32 * P);
    w->ray[1] = (float4 *)take(32 * P);
    w->hits = (float4 *)take(16 * P);
    w->cray = (float4 *)take(64 * P);
    w->crec = (float4 *)take(64 * P);
    w->counters = (WaveCounters *)take(sizeof(WaveCounters));
    return off;
}

// Sizes the context's wavefront arena for `cap` entries (one allocation, reused).
static lt_status ensure_wave(lt_ctx *c, uint32_t cap) {
    if (c->wave.capacity >= cap && c->wave.arena) return LT_OK;
    free_wave(c);
    Wavefront sizing;
    size_t bytes = carve_wave(nullptr, cap, &sizing);
    char *a = nullptr;
    CUDA_TRY(c, cudaMalloc((void **)&a, bytes));
    carve_wave(a, cap, &c->wave);
    c->wave.arena = a;
    c->wave.arena_bytes = bytes;
    return LT_OK;
}

static uint32_t default_capacity(unsigned long long total) {
    const unsigned long long kMax = 1ull << 21;  // 2M path slots, ~560 MB
    return (uint32_t)(total < kMax ? total : kMax);
}

extern "C" {

lt_status lt_render(lt_ctx *c, const lt_render_params *p, lt_film *film) {
    if (!c || !p || !film) return fail(c, LT_ERR_INVALID, "NULL argument");
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "lt_render without a scene");
    const uint32_t W = c->host.camera.width, H = c->host.camera.height;
    if (film->width != W || film->height != H)
        return fail(c, LT_ERR_INVALID, "film is %ux%u, scene camera is %ux%u", film->width, film->height, W, H);
    if (!film->rgb || !film->bounces || !film->counts) return fail(c, LT_ERR_INVALID, "film buffers missing");
    CUDA_TRY(c, cudaSetDevice(c->device));
    const size_t npix = (size_t)W * H;
    FilmPtrs f;
    if (film->on_device) {
        f.rgb = film->rgb;
        f.bounces = film->bounces;
        f.counts = film->counts;
    } else {
        lt_status st = ensure_scratch(c, npix * 20 + 512);
        if (st != LT_OK) return st;
        char *s = (char *)c->scratch;
        f.rgb = (float *)s;
        f.bounces = (uint32_t *)(s + ((npix * 12 + 255) & ~(size_t)255));
        f.counts = f.bounces + npix;
        CUDA_TRY(c, cudaMemcpyAsync(f.rgb, film->rgb, npix * 12, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(f.bounces, film->bounces, npix * 4, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(f.counts, film->counts, npix * 4, cudaMemcpyHostToDevice, c->stream));
    }
    RenderArgs a;
    a.width = W;
    a.height = H;
    a.first_frame = p->first_frame;
    a.max_depth = p->max_depth;
    a.rr_depth = p->rr_depth;
    a.total = (unsigned long long)npix * p->spp;
    c->stats = lt_render_stats{};
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    if (a.total > 0 && p->max_depth == 0) {
        CUDA_TRY(c, launch_add_counts(f, (uint32_t)npix, p->spp, c->stream));
        c->stats.kernel_launches = 1;
    } else if (a.total > 0) {
        lt_status st = ensure_wave(c, default_capacity(a.total));
        if (st != LT_OK) return st;
        CUDA_TRY(c, cudaMemsetAsync(c->wave.counters, 0, sizeof(WaveCounters), c->stream));
        CUDA_TRY(c, launch_wave_init(c->dev, c->wave, a, f, c->shape, c->stream));
        uint32_t launches = 1, iters = 0;
        size_t nev = 0;
        c->stage_of_event.clear();
        int cur = 0;
        const int kBatch = 4;
        for (;;) {
            for (int k = 0; k < kBatch; ++k) {
                for (int stage = 0; stage < 3; ++stage) {
                    if (nev == c->stage_events.size()) {
                        cudaEvent_t e;
                        CUDA_TRY(c, cudaEventCreate(&e));
                        c->stage_events.push_back(e);
                    }
                    CUDA_TRY(c, cudaEventRecord(c->stage_events[nev++], c->stream));
                    c->stage_of_event.push_back(stage);
                    CUDA_TRY(c, launch_wave_stage(stage, c->dev, c->wave, a, f, cur, c->shape, c->stream));
                }
                launches += 3;
                cur ^= 1;
                ++iters;
            }
            CUDA_TRY(c, cudaMemcpyAsync(c->counters_host, c->wave.counters, sizeof(WaveCounters),
                                        cudaMemcpyDeviceToHost, c->stream));
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            if (c->counters_host->count[cur] == 0) break;
            if (iters > 4u * (p->max_depth + 8u) * (uint32_t)((a.total + c->wave.capacity - 1) / c->wave.capacity) + 64u)
                return fail(c, LT_ERR_TIMEOUT, "wavefront did not drain after %u iterations", iters);
        }
        c->stats.main_rays = c->counters_host->main_rays;
        c->stats.light_rays = c->counters_host->light_rays;
        c->stats.bsdf_rays = c->counters_host->bsdf_rays;
        c->stats.iterations = iters;
        c->stats.kernel_launches = launches;
        if (nev == c->stage_events.size()) {
            cudaEvent_t e;
            CUDA_TRY(c, cudaEventCreate(&e));
            c->stage_events.push_back(e);
        }
        CUDA_TRY(c, cudaEventRecord(c->stage_events[nev], c->stream));
        CUDA_TRY(c, cudaEventSynchronize(c->stage_events[nev]));
        float acc[3] = {0, 0, 0};
        for (size_t i = 0; i < nev; ++i) {
            float ms = 0.0f;
            CUDA_TRY(c, cudaEventElapsedTime(&ms, c->stage_events[i], c->stage_events[i + 1]));
            acc[c->stage_of_event[i]] += ms;
        }
        c->stats.trace_ms = acc[0];
        c->stats.shade_ms = acc[1];
        c->stats.connect_ms = acc[2];
    }
    c->stats.samples = a.total;
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    if (!film->on_device) {
        CUDA_TRY(c, cudaMemcpyAsync(film->rgb, f.rgb, npix * 12, cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(film->bounces, f.bounces, npix * 4, cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(film->counts, f.counts, npix * 4, cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    return LT_OK;
}

lt_status lt_render_stats_get(lt_ctx *c, lt_render_stats *out) {
    if (!c || !out) return LT_ERR_INVALID;
    *out = c->stats;
    float ms = 0.0f;
    if (cudaEventSynchronize(c->ev1) == cudaSuccess && cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess)
        out->gpu_ms = ms;
    return LT_OK;
}

lt_status lt_intersect(lt_ctx *c, const lt_ray *rays, lt_hit *hits, uint64_t n, int32_t on_device) {
    if (!c || (n && (!rays || !hits))) return fail(c, LT_ERR_INVALID, "NULL argument");
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "lt_intersect without a scene");
    if (n == 0) return LT_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (on_device) {
        if (((uintptr_t)rays & 15u) || ((uintptr_t)hits & 15u))
            return fail(c, LT_ERR_INVALID, "rays and hits must be 16-byte aligned");
        CUDA_TRY(c, launch_intersect(c->dev, (const float4 *)rays, (float4 *)hits, n, c->isect_fetch, c->shape,
                                     c->stream));
        return LT_OK;
    }
    lt_status st = ensure_scratch(c, n * 48);
    if (st != LT_OK) return st;
    float4 *dr = (float4 *)c->scratch;
    float4 *dh = dr + 2 * n;
    CUDA_TRY(c, cudaMemcpyAsync(dr, rays, n * 32, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, launch_intersect(c->dev, dr, dh, n, c->isect_fetch, c->shape, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(hits, dh, n * 16, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return LT_OK;
}

lt_status lt_diff_defaults(lt_ctx *c, float *albedo, float *emission, float *sigma_a, float *sigma_s) {
    if (!c) return LT_ERR_INVALID;
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    const HostScene &h = c->host;
    for (size_t t = 0; t < h.tri_geom.size(); ++t) {
        const GeomInfo &g = h.geoms[h.tri_geom[t]];
        const MaterialInfo &m = h.materials[g.material];
        for (int k = 0; k < 3; ++k) {
            if (albedo) albedo[3 * t + k] = m.albedo[k];
            if (emission) emission[3 * t + k] = g.light >= 0 ? h.lights[g.light].radiance[k] : 0.0f;
        }
    }
    for (size_t i = 0; i < h.media.size(); ++i)
        for (int k = 0; k < 3; ++k) {
            if (sigma_a) sigma_a[3 * i + k] = h.media[i].sigma_a[k];
            if (sigma_s) sigma_s[3 * i + k] = h.media[i].sigma_s[k];
        }
    return LT_OK;
}

static lt_status diff_setup(lt_ctx *c, const lt_render_params *p, const lt_diff_params *dp, DiffParams *P,
                            RenderArgs *a) {
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    if (!dp->albedo || !dp->emission || (c->host.media.size() && (!dp->sigma_a || !dp->sigma_s)))
        return fail(c, LT_ERR_INVALID, "differentiable parameters missing");
    P->albedo = dp->albedo;
    P->emission = dp->emission;
    P->sigma_a = dp->sigma_a;
    P->sigma_s = dp->sigma_s;
    P->albedo_s = dp->albedo_detached ? dp->albedo_detached : dp->albedo;
    P->sigma_a_s = dp->sigma_a_detached ? dp->sigma_a_detached : dp->sigma_a;
    P->sigma_s_s = dp->sigma_s_detached ? dp->sigma_s_detached : dp->sigma_s;
    a->width = c->host.camera.width;
    a->height = c->host.camera.height;
    a->first_frame = p->first_frame;
    a->max_depth = p->max_depth;
    a->rr_depth = p->rr_depth;
    a->total = (unsigned long long)a->width * a->height * p->spp;
    CUDA_TRY(c, cudaSetDevice(c->device));
    return LT_OK;
}

lt_status lt_render_diff(lt_ctx *c, const lt_render_params *p, const lt_diff_params *dp, lt_film *film,
                         float *sample_radiance) {
    if (!c || !p || !dp || !film) return fail(c, LT_ERR_INVALID, "NULL argument");
    DiffParams P;
    RenderArgs a;
    lt_status st = diff_setup(c, p, dp, &P, &a);
    if (st != LT_OK) return st;
    if (!film->on_device || film->width != a.width || film->height != a.height)
        return fail(c, LT_ERR_INVALID, "lt_render_diff needs a device film of the camera's size");
    FilmPtrs f{film->rgb, film->bounces, film->counts};
    c->stats = lt_render_stats{};
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    CUDA_TRY(c, launch_diff_forward(c->dev, P, a, f, sample_radiance, c->shape, c->stream));
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    c->stats.samples = a.total;
    c->stats.kernel_launches = 1;
    return LT_OK;
}

lt_status lt_render_adjoint(lt_ctx *c, const lt_render_params *p, const lt_diff_params *dp, const float *dI,
                            float *g_albedo, float *g_emission, float *g_sigma_a, float *g_sigma_s,
                            const uint32_t *crop, const float *sample_radiance) {
    if (!c || !p || !dp || !dI || !g_albedo || !g_emission) return fail(c, LT_ERR_INVALID, "NULL argument");
    DiffParams P;
    RenderArgs a;
    lt_status st = diff_setup(c, p, dp, &P, &a);
    if (st != LT_OK) return st;
    if (c->host.media.size() && (!g_sigma_a || !g_sigma_s)) return fail(c, LT_ERR_INVALID, "medium gradients missing");
    DiffGrads G{dI, g_albedo, g_emission, g_sigma_a, g_sigma_s, 0, 0, a.width, a.height, sample_radiance};
    if (crop) {
        if (crop[0] > crop[2] || crop[1] > crop[3] || crop[2] > a.width || crop[3] > a.height)
            return fail(c, LT_ERR_INVALID, "crop outside the film");
        G.x0 = crop[0];
        G.y0 = crop[1];
        G.x1 = crop[2];
        G.y1 = crop[3];
    }
    c->stats = lt_render_stats{};
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    CUDA_TRY(c, launch_diff_adjoint(c->dev, P, a, G, (uint32_t)c->host.media.size(), c->shape, c->stream));
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    c->stats.samples = a.total;
    c->stats.kernel_launches = 1;
    return LT_OK;
}

lt_status lt_scene_load_json(lt_ctx *c, const char *path) {
    if (!c || !path) return fail(c, LT_ERR_INVALID, "NULL argument");
    lt_scene_desc desc;
    JsonSceneStorage storage;
    std::string err;
    lt_status st = load_scene_json(path, &desc, &storage, &err);
    if (st != LT_OK) return fail(c, st, "%s", err.c_str());
    return lt_scene_create(c, &desc);
}

}  // extern "C"

// ------------------------------------------------------------------ lt_render_noalloc
// Same wavefront as lt_render, with its state carved out of the fixed device
// array of lt_noalloc.cu instead of a cudaMalloc'd arena. Nothing here
// allocates: no cudaMalloc / cudaFree / cudaMallocHost, no new CUDA events, no
// staging buffers (the film must already be on the device).
#include "lt_noalloc.h"

static Wavefront carve_noalloc(char *a, uint32_t cap) {
    Wavefront w;
    w.arena_bytes = carve_wave(a, cap, &w);
    w.arena = nullptr;  // not owned: never freed
    return w;
}

extern "C" lt_status lt_render_noalloc(lt_ctx *c, const lt_render_params *p, lt_film *film,
                                       uint32_t paths_in_flight) {
    if (!c || !p || !film) return fail(c, LT_ERR_INVALID, "NULL argument");
    if (paths_in_flight == 0 || paths_in_flight > LT_NOALLOC_MAX_PATHS)
        return fail(c, LT_ERR_INVALID, "paths_in_flight = %u; lt_render_noalloc holds 1..%u paths", paths_in_flight,
                    (unsigned)LT_NOALLOC_MAX_PATHS);
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "lt_render_noalloc without a scene");
    const uint32_t W = c->host.camera.width, H = c->host.camera.height;
    if (film->width != W || film->height != H)
        return fail(c, LT_ERR_INVALID, "film is %ux%u, scene camera is %ux%u", film->width, film->height, W, H);
    if (!film->on_device) return fail(c, LT_ERR_INVALID, "lt_render_noalloc needs a device film (on_device = 1)");
    if (!film->rgb || !film->bounces || !film->counts) return fail(c, LT_ERR_INVALID, "film buffers missing");
    CUDA_TRY(c, cudaSetDevice(c->device));
    void *scratch = nullptr;
    CUDA_TRY(c, noalloc_scratch(c->device, &scratch));
    const size_t npix = (size_t)W * H;
    FilmPtrs f;
    f.rgb = film->rgb;
    f.bounces = film->bounces;
    f.counts = film->counts;
    RenderArgs a;
    a.width = W;
    a.height = H;
    a.first_frame = p->first_frame;
    a.max_depth = p->max_depth;
    a.rr_depth = p->rr_depth;
    a.total = (unsigned long long)npix * p->spp;
    c->stats = lt_render_stats{};
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    if (a.total > 0 && p->max_depth == 0) {
        CUDA_TRY(c, launch_add_counts(f, (uint32_t)npix, p->spp, c->stream));
        c->stats.kernel_launches = 1;
    } else if (a.total > 0) {
        uint32_t cap = (uint32_t)(a.total < paths_in_flight ? a.total : paths_in_flight);
        Wavefront w = carve_noalloc((char *)scratch, cap);
        if (w.arena_bytes > kNoAllocScratchBytes)
            return fail(c, LT_ERR_INVALID, "internal: wavefront needs %zu bytes, fixed scratch holds %zu", w.arena_bytes,
                        kNoAllocScratchBytes);
        // the array keeps the previous call's contents: the counters must start at zero
        CUDA_TRY(c, cudaMemsetAsync(w.counters, 0, sizeof(WaveCounters), c->stream));
        CUDA_TRY(c, launch_wave_init(c->dev, w, a, f, c->shape, c->stream));
        uint32_t launches = 1, iters = 0;
        int cur = 0;
        const int kBatch = 4;
        const uint32_t limit = 4u * (p->max_depth + 8u) * (uint32_t)((a.total + cap - 1) / cap) + 64u;
        for (;;) {
            for (int k = 0; k < kBatch; ++k) {
                for (int stage = 0; stage < 3; ++stage)
                    CUDA_TRY(c, launch_wave_stage(stage, c->dev, w, a, f, cur, c->shape, c->stream));
                launches += 3;
                cur ^= 1;
                ++iters;
            }
            CUDA_TRY(c, cudaMemcpyAsync(c->counters_host, w.counters, sizeof(WaveCounters), cudaMemcpyDeviceToHost,
                                        c->stream));
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            if (c->counters_host->count[cur] == 0) break;
            if (iters > limit) return fail(c, LT_ERR_TIMEOUT, "wavefront did not drain after %u iterations", iters);
        }
        c->stats.main_rays = c->counters_host->main_rays;
        c->stats.light_rays = c->counters_host->light_rays;
        c->stats.bsdf_rays = c->counters_host->bsdf_rays;
        c->stats.iterations = iters;
        c->stats.kernel_launches = launches;
    }
    c->stats.samples = a.total;
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    return LT_OK;
}
