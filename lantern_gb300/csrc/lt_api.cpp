// lt_api.cpp -- the C ABI declared in include/lantern_gpu.h.
//
// A context owns a CUDA stream, the device copy of one scene (triangles, BVH2
// and on demand the 4- and 8-wide BVHs, shading tables, textures) and the wavefront
// buffers, which are sized once and reused. lt_render queues the wavefront: an
// initial camera-ray launch, then batches of (trace, shade) iterations, reading
// the queue lengths back once per batch until no path or connection record is
// left. lt_render_batch runs the same loop over many contexts' scenes as one
// captured CUDA graph.
#include <cuda_runtime.h>

#include <cmath>
#include <atomic>
#include <climits>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "lantern_gpu.h"
#include "lt_device.h"
#include "lt_bvh_gpu.h"
#include "lt_noalloc.h"
#include "lt_order.h"
#include "lt_scene.h"
#include "lt_setup.h"

using namespace lt;

// The CUDA runtime behind WorkOrder (lt_order.h).
struct CudaRt {
    using Event = cudaEvent_t;
    using Stream = cudaStream_t;
    int record(Event e, Stream s) { return (int)cudaEventRecord(e, s); }
    int wait(Stream s, Event e) { return (int)cudaStreamWaitEvent(s, e, 0); }
    int sync(Event e) { return (int)cudaEventSynchronize(e); }
};

struct lt_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string error;
    LaunchShape shape;

    // scene
    bool has_scene = false;
    bool has_bvh8 = false, has_bvh4 = false;
    uint32_t bvh8_depth = 0;
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

    // differentiable forward on the wavefront: the path extras (DiffWave) and,
    // when the caller keeps no per-sample radiance, a buffer for it
    void *diff_arena = nullptr;
    size_t diff_arena_bytes = 0;
    uint32_t diff_capacity = 0;
    float *diff_samples = nullptr;
    size_t diff_samples_bytes = 0;

    // launch configuration (lt_set_tuning / lt_autotune_batch); shape is the
    // single-scene instantiation's, batch_shape the batched one's
    lt_tuning tuning{};
    LaunchShape batch_shape;

    // batched rendering: the scene table (pinned host copy + device copy) and
    // the captured loop, rebuilt when its key changes
    SceneTable *table_host = nullptr, *table_dev = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<uintptr_t> graph_key;

    // ordering across stream switches and of host writes into the scene table
    CudaRt rt;
    WorkOrder<CudaRt> order;

    lt_render_stats stats{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // stage timing (lt_set_stage_timing, off by default): an event before and
    // after every stage launch of the wavefront renders
    bool stage_timing = false;
    std::vector<cudaEvent_t> stage_events;
    std::vector<int> stage_of_event;

    // queue trace (lt_set_queue_trace, off by default): k_trace writes each
    // iteration's queue lengths into qtrace_dev; qtrace_rows of the last loop
    uint3 *qtrace_dev = nullptr;
    uint32_t qtrace_cap = 0, qtrace_rows = 0;
};

static thread_local std::string g_create_error;

// NVTX range over one API call (visible in Nsight Systems / ncu timelines;
// no cost without a tool attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

// Allocation fault injection (lt_debug_fail_allocations): after `left` more
// successful device or pinned-host allocations, the next one fails with
// cudaErrorMemoryAllocation without reaching the CUDA runtime.
static std::atomic<uint32_t> g_alloc_left{UINT32_MAX};

static bool injected_alloc_failure() {
    uint32_t left = g_alloc_left.load();
    while (left != UINT32_MAX) {
        if (left == 0) return true;
        if (g_alloc_left.compare_exchange_weak(left, left - 1)) return false;
    }
    return false;
}

// Wavefront iteration cap for failure-handling tests
// (lt_debug_set_iteration_limit); 0 = the library's own bound.
static std::atomic<unsigned long long> g_iteration_limit{0};
// Film pixels that the bound checks of an LT_CHECKS build accept (0: the film's own size).
static std::atomic<uint32_t> g_check_pixels{0};

// Iterations a render may take before it reports LT_ERR_TIMEOUT: every path
// ends within max_depth iterations of its start and at most `cap` work items
// start per iteration, so a render needs about max_depth * total / cap; the
// bound leaves a factor of four and some slack. 64-bit: with few paths in
// flight the product exceeds 32 bits.
static unsigned long long drain_limit(unsigned long long total, uint32_t cap, uint32_t max_depth) {
    const unsigned long long own = 4ull * ((unsigned long long)max_depth + 8ull) * ((total + cap - 1) / cap) + 64ull;
    const unsigned long long dbg = g_iteration_limit.load();
    return dbg && dbg < own ? dbg : own;
}

static cudaError_t dev_malloc(void **p, size_t bytes) {
    if (injected_alloc_failure()) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

static cudaError_t host_malloc(void **p, size_t bytes) {
    if (injected_alloc_failure()) return cudaErrorMemoryAllocation;
    return cudaMallocHost(p, bytes);
}

static lt_status fail(lt_ctx *c, lt_status st, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    try {
        if (c) c->error = buf;
        else g_create_error = buf;
    } catch (...) {  // no memory for the message: the status still goes back
    }
    return st;
}

// A failed device-side bound check recorded in the counters (LT_CHECKS builds).
static lt_status check_failed(lt_ctx *c, const WaveCounters &k) {
    return fail(c, LT_ERR_CHECK, "device bound check failed: %s (index %u)", check_name(k.check), k.check_value);
}

// No C++ exception crosses the C ABI: every entry point's body is a function
// try block ending in LT_CATCH. Host allocation failures (std::bad_alloc, or
// std::length_error for an impossible container size) become LT_ERR_OOM; any
// other exception LT_ERR_INVALID. `c` is the context whose lt_last_error
// carries the message (NULL: the thread's creation error).
#define LT_CATCH(c)                                                                         \
    catch (const std::bad_alloc &) {                                                        \
        return fail(c, LT_ERR_OOM, "host memory allocation failed");                        \
    }                                                                                       \
    catch (const std::length_error &) {                                                     \
        return fail(c, LT_ERR_OOM, "host container size out of range");                     \
    }                                                                                       \
    catch (const std::exception &e_) {                                                      \
        return fail(c, LT_ERR_INVALID, "unexpected host error: %s", e_.what());             \
    }                                                                                       \
    catch (...) {                                                                           \
        return fail(c, LT_ERR_INVALID, "unexpected host error");                            \
    }

#define CUDA_TRY(c, expr)                                                                           \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(c, e_ == cudaErrorMemoryAllocation ? LT_ERR_OOM : LT_ERR_CUDA, "%s: %s (%s:%d)", \
                        #expr, cudaGetErrorString(e_), __FILE__, __LINE__);                         \
    } while (0)

// Frees the context's scene. Any context's queued batched work may read it
// (lt_render_diff_batch and lt_render_adjoint_batch return once queued), so
// the device is synchronised first.
static void free_scene(lt_ctx *c) {
    if (!c->scene_allocs.empty()) cudaDeviceSynchronize();
    for (void *p : c->scene_allocs) cudaFree(p);
    c->scene_allocs.clear();
    c->scene_bytes = 0;
    c->has_scene = false;
    c->has_bvh8 = false;
    c->has_bvh4 = false;
    c->dev = DevScene{};
}

static void free_graph(lt_ctx *c) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->graph_exec = nullptr;
    c->graph = nullptr;
    c->graph_key.clear();
}

static void free_wave(lt_ctx *c) {
    if (c->wave.arena && c->stream) cudaStreamSynchronize(c->stream);  // the context's work is on its stream
    free_graph(c);  // its kernels point into the arena
    if (c->wave.arena) cudaFree(c->wave.arena);
    c->wave = Wavefront{};
}

// Wavefront iterations to queue before the first read of the queue lengths.
// With every sample in flight nothing is regenerated, and every event of a path
// (surface bounce or medium scatter) adds a bounce, so max_depth iterations end
// every path and one more traces the last shade's connection records: a short
// render then needs a single read. Otherwise 4; the loop checks the queues
// after each batch either way, so the bound only saves synchronisations.
static uint32_t first_batch(unsigned long long total, uint32_t cap, uint32_t max_depth) {
    return total <= cap && max_depth < 64u ? max_depth + 1u : 4u;
}

static void default_tuning(lt_tuning *t) {
    *t = lt_tuning{};
    t->trace_threads = 128;
    t->shade_threads = 256;
    t->loop_iterations = 2;
    t->bvh_width = 2;
}

// Block counts of both kernel instantiations for the tuning's thread counts.
static void apply_tuning(lt_ctx *c) {
    for (LaunchShape *ls : {&c->shape, &c->batch_shape}) {
        ls->bvh_width = (int)c->tuning.bvh_width;
        ls->trace_threads = (int)c->tuning.trace_threads;
        ls->shade_threads = (int)c->tuning.shade_threads;
    }
    // the batched shade kernel holds 256 threads per block at most
    if (c->batch_shape.shade_threads > 256) c->batch_shape.shade_threads = 256;
    query_launch_shape(c->device, false, &c->shape);
    query_launch_shape(c->device, true, &c->batch_shape);
}

extern "C" {

int lt_abi_version(void) { return LT_ABI_VERSION; }

lt_status lt_ctx_create(int device, lt_ctx **out) try {
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
    if (e == cudaSuccess) e = host_malloc((void **)&c->counters_host, sizeof(WaveCounters));
    if (e == cudaSuccess) e = dev_malloc((void **)&c->isect_fetch, 256);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->order.switch_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->order.table_ev, cudaEventDisableTiming);
    // lt_render_noalloc's set-up: load the module holding its fixed scratch
    // array (reserving the array on this device) and the wavefront kernels now,
    // so that no call of it loads code or data onto the device
    void *noalloc_ptr = nullptr;
    if (e == cudaSuccess) e = noalloc_scratch(device, &noalloc_ptr);
    if (e == cudaSuccess) e = preload_wave_kernels();
    if (e != cudaSuccess) {
        lt_ctx_destroy(c);
        return fail(nullptr, LT_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    default_tuning(&c->tuning);
    apply_tuning(c);
    *out = c;
    return LT_OK;
} LT_CATCH(nullptr)

void lt_ctx_destroy(lt_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->own_stream && c->own_stream != c->stream) cudaStreamSynchronize(c->own_stream);
    free_scene(c);
    free_wave(c);
    if (c->table_dev) cudaFree(c->table_dev);
    if (c->table_host) cudaFreeHost(c->table_host);
    if (c->scratch) cudaFree(c->scratch);
    if (c->diff_arena) cudaFree(c->diff_arena);
    if (c->diff_samples) cudaFree(c->diff_samples);
    if (c->counters_host) cudaFreeHost(c->counters_host);
    if (c->isect_fetch) cudaFree(c->isect_fetch);
    if (c->qtrace_dev) cudaFree(c->qtrace_dev);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->order.switch_ev) cudaEventDestroy(c->order.switch_ev);
    if (c->order.table_ev) cudaEventDestroy(c->order.table_ev);
    for (cudaEvent_t e : c->stage_events) cudaEventDestroy(e);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

const char *lt_last_error(const lt_ctx *c) { return c ? c->error.c_str() : g_create_error.c_str(); }

lt_status lt_set_stream(lt_ctx *c, void *stream) try {
    if (!c) return LT_ERR_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    // work queued on the old stream comes before anything queued on the new one
    CUDA_TRY(c, (cudaError_t)c->order.switch_stream(c->rt, c->stream, (cudaStream_t)stream));
    c->stream = (cudaStream_t)stream;
    return LT_OK;
} LT_CATCH(c)

void *lt_get_stream(const lt_ctx *c) { return c ? (void *)c->stream : nullptr; }

lt_status lt_set_bvh_builder(lt_ctx *c, int32_t builder) try {
    if (!c) return LT_ERR_INVALID;
    if (builder != LT_BVH_GPU && builder != LT_BVH_HOST) return fail(c, LT_ERR_INVALID, "unknown BVH builder %d", builder);
    c->bvh_builder = builder;
    return LT_OK;
} LT_CATCH(c)

lt_status lt_sync(lt_ctx *c) try {
    if (!c) return LT_ERR_INVALID;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return LT_OK;
} LT_CATCH(c)

lt_status lt_trim(lt_ctx *c) try {
    if (!c) return LT_ERR_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (c->own_stream != c->stream) CUDA_TRY(c, cudaStreamSynchronize(c->own_stream));
    free_wave(c);  // with the captured batch loop, which points into it
    if (c->diff_arena) cudaFree(c->diff_arena);
    c->diff_arena = nullptr;
    c->diff_arena_bytes = 0;
    c->diff_capacity = 0;
    if (c->diff_samples) cudaFree(c->diff_samples);
    c->diff_samples = nullptr;
    c->diff_samples_bytes = 0;
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    return LT_OK;
} LT_CATCH(c)

}  // extern "C"

// Temporary device buffers of one call, freed when it returns (after the
// call's work on `stream`, which may still read them, has finished).
struct Temp {
    cudaStream_t stream;
    std::vector<void *> ptrs;
    cudaError_t alloc(void **p, size_t bytes) {
        cudaError_t e = dev_malloc(p, bytes);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
    ~Temp() {
        if (!ptrs.empty()) cudaStreamSynchronize(stream);
        for (void *p : ptrs) cudaFree(p);
    }
};

// A device buffer owned by the context's scene.
static lt_status scene_alloc(lt_ctx *c, size_t bytes, void **p) {
    CUDA_TRY(c, dev_malloc(p, bytes));
    c->scene_allocs.push_back(*p);
    c->scene_bytes += bytes;
    return LT_OK;
}

template <typename T>
static lt_status upload(lt_ctx *c, const std::vector<T> &v, const T **dst) {
    size_t bytes = v.size() * sizeof(T);
    void *p = nullptr;
    CUDA_TRY(c, dev_malloc(&p, bytes ? bytes : 16));
    c->scene_allocs.push_back(p);
    c->scene_bytes += bytes;
    if (bytes) CUDA_TRY(c, cudaMemcpyAsync(p, v.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    *dst = (const T *)p;
    return LT_OK;
}

// Builds the compressed 8-wide BVH of the context's scene from its BVH2 (read
// back from the device when the GPU built it) and uploads it.
static lt_status ensure_bvh8(lt_ctx *c) {
    if (c->has_bvh8) return LT_OK;
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    HostScene &h = c->host;
    std::vector<BvhNode> nodes = h.nodes;
    std::vector<float> tris = h.leaf_tris;
    if (nodes.empty()) {
        nodes.resize(c->num_nodes);
        tris.resize(12 * h.tri_geom.size());
        CUDA_TRY(c, cudaMemcpyAsync(nodes.data(), c->dev.nodes, nodes.size() * sizeof(BvhNode),
                                    cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(tris.data(), c->dev.tris, tris.size() * sizeof(float), cudaMemcpyDeviceToHost,
                                    c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    std::vector<Bvh8Node> n8;
    std::vector<float> t8;
    const uint32_t depth = build_bvh8(nodes, tris, &n8, &t8);
    if (2 * depth + 2 > 64)
        return fail(c, LT_ERR_UNSUPPORTED, "8-wide BVH depth %u exceeds the traversal stack", depth);
    std::vector<float> nf(n8.size() * 20);
    memcpy(nf.data(), n8.data(), nf.size() * sizeof(float));
    const float *d_nodes = nullptr, *d_tris = nullptr;
    lt_status st = upload(c, nf, &d_nodes);
    if (st == LT_OK) st = upload(c, t8, &d_tris);
    if (st != LT_OK) return st;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->dev.nodes8 = (const float4 *)d_nodes;
    c->dev.tris8 = (const float4 *)d_tris;
    c->dev.num_nodes8 = (uint32_t)n8.size();
    c->bvh8_depth = depth;
    c->has_bvh8 = true;
    return LT_OK;
}

// The wide BVH a tuning's width needs (4 or 8: built once per scene).
static lt_status ensure_width(lt_ctx *c, uint32_t width);

extern "C" {

lt_status lt_scene_create(lt_ctx *c, const lt_scene_desc *desc) try {
    NvtxRange nvtx_("lt_scene_create");
    if (!c || !desc) return fail(c, LT_ERR_INVALID, "NULL argument");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    free_scene(c);
    size_t ntri = 0, nvert = 0;
    for (uint32_t g = 0; g < desc->num_meshes; ++g) {
        ntri += desc->meshes[g].num_triangles;
        nvert += desc->meshes[g].num_vertices;
    }
    // GPU builder: transform and triangle setup on the device as well
    const bool gpu_setup = c->bvh_builder == LT_BVH_GPU && ntri > 4;
    std::string err;
    lt_status st = build_host_scene(desc, &c->host, &err, !gpu_setup);
    if (st != LT_OK) return fail(c, st, "%s", err.c_str());
    HostScene &h = c->host;
    DevScene &d = c->dev;
    if (gpu_setup) {
        // raw mesh arrays -> device, then transform + triangle setup (lt_setup.cu)
        Temp tmp{c->stream, {}};
        float *d_pos = nullptr, *d_tri = nullptr, *d_nrm = nullptr, *d_tex = nullptr;
        uint32_t *d_idx = nullptr, *d_vidx = nullptr;
        MeshSetup *d_meshes = nullptr;
        CUDA_TRY(c, tmp.alloc((void **)&d_pos, nvert * 12 + 16));
        CUDA_TRY(c, tmp.alloc((void **)&d_idx, ntri * 12));
        CUDA_TRY(c, tmp.alloc((void **)&d_tri, ntri * 36));
        CUDA_TRY(c, tmp.alloc((void **)&d_meshes, desc->num_meshes * sizeof(MeshSetup) + 16));
        if ((st = scene_alloc(c, nvert * 12 + 16, (void **)&d_nrm)) != LT_OK) return st;
        if ((st = scene_alloc(c, nvert * 8 + 16, (void **)&d_tex)) != LT_OK) return st;
        if ((st = scene_alloc(c, ntri * 12, (void **)&d_vidx)) != LT_OK) return st;
        std::vector<MeshSetup> ms(desc->num_meshes);
        size_t vb = 0, tb = 0;
        for (uint32_t g = 0; g < desc->num_meshes; ++g) {
            const lt_mesh_desc &m = desc->meshes[g];
            MeshSetup &M = ms[g];
            memset(&M, 0, sizeof M);
            M.vbase = (uint32_t)vb;
            M.tbase = (uint32_t)tb;
            M.nverts = m.num_vertices;
            M.ntris = m.num_triangles;
            if (m.transform) {
                M.has_transform = 1;
                memcpy(M.m, m.transform, 12 * sizeof(float));
            }
            const size_t nv = m.num_vertices, nt = m.num_triangles;
            if (nv) {
                CUDA_TRY(c, cudaMemcpyAsync(d_pos + 3 * vb, m.positions, nv * 12, cudaMemcpyHostToDevice, c->stream));
                if (m.normals)
                    CUDA_TRY(c, cudaMemcpyAsync(d_nrm + 3 * vb, m.normals, nv * 12, cudaMemcpyHostToDevice, c->stream));
                else
                    CUDA_TRY(c, cudaMemsetAsync(d_nrm + 3 * vb, 0, nv * 12, c->stream));
                if (m.texcoords)
                    CUDA_TRY(c, cudaMemcpyAsync(d_tex + 2 * vb, m.texcoords, nv * 8, cudaMemcpyHostToDevice, c->stream));
                else
                    CUDA_TRY(c, cudaMemsetAsync(d_tex + 2 * vb, 0, nv * 8, c->stream));
            }
            if (nt) CUDA_TRY(c, cudaMemcpyAsync(d_idx + 3 * tb, m.indices, nt * 12, cudaMemcpyHostToDevice, c->stream));
            vb += nv;
            tb += nt;
        }
        CUDA_TRY(c, cudaMemcpyAsync(d_meshes, ms.data(), ms.size() * sizeof(MeshSetup), cudaMemcpyHostToDevice,
                                    c->stream));
        CUDA_TRY(c, setup_triangles_gpu(d_pos, d_idx, d_meshes, desc->num_meshes, (uint32_t)nvert, (uint32_t)ntri,
                                        d_tri, d_vidx, c->stream));
        // area lights from the transformed vertices: light triangles, area,
        // bounding sphere, radiance (read back for the host's copy)
        if (h.lights.size() > kMaxLights)
            return fail(c, LT_ERR_UNSUPPORTED, "%zu lights: at most %u", h.lights.size(), kMaxLights);
        const size_t nl = h.lights.size();
        size_t nlt = 0;
        for (const LightSource &ls : h.light_src) nlt += ls.ntris;
        LightSource *d_src = nullptr;
        LightInfo *d_lights = nullptr;
        float4 *d_ltris = nullptr;
        CUDA_TRY(c, tmp.alloc((void **)&d_src, nl * sizeof(LightSource) + 16));
        if ((st = scene_alloc(c, nl * sizeof(LightInfo) + 16, (void **)&d_lights)) != LT_OK) return st;
        if ((st = scene_alloc(c, nlt * 48 + 16, (void **)&d_ltris)) != LT_OK) return st;
        if (nl) {
            CUDA_TRY(c, cudaMemcpyAsync(d_src, h.light_src.data(), nl * sizeof(LightSource), cudaMemcpyHostToDevice,
                                        c->stream));
            CUDA_TRY(c, setup_lights_gpu(d_pos, d_idx, d_src, (uint32_t)nl, d_lights, d_ltris, c->stream));
            CUDA_TRY(c, cudaMemcpyAsync(h.lights.data(), d_lights, nl * sizeof(LightInfo), cudaMemcpyDeviceToHost,
                                        c->stream));
        }
        d.lights = d_lights;
        d.light_tris = d_ltris;
        d.vnormal = d_nrm;
        d.vtex = d_tex;
        d.tri_vidx = d_vidx;
        // binned-SAH build on the device from the triangles in global order
        GpuBvh gb;
        cudaError_t e = build_bvh_gpu(d_tri, (uint32_t)ntri, &gb, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
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
    if (h.lights.size() > kMaxLights || h.media.size() > kMaxMedia)
        return fail(c, LT_ERR_UNSUPPORTED, "%zu lights / %zu media: at most %u and %u", h.lights.size(),
                    h.media.size(), kMaxLights, kMaxMedia);
    if ((st = upload(c, h.tri_geom, &d.tri_geom)) != LT_OK) return st;
    if (!gpu_setup) {
        if ((st = upload(c, h.tri_vidx, &d.tri_vidx)) != LT_OK) return st;
        if ((st = upload(c, h.vnormal, &d.vnormal)) != LT_OK) return st;
        if ((st = upload(c, h.vtex, &d.vtex)) != LT_OK) return st;
    }
    if ((st = upload(c, h.texels, &d.texels)) != LT_OK) return st;
    if ((st = upload(c, h.images, &d.images)) != LT_OK) return st;
    if ((st = upload(c, h.geoms, &d.geoms)) != LT_OK) return st;
    if ((st = upload(c, h.materials, &d.mats)) != LT_OK) return st;
    if ((st = upload(c, h.media, &d.meds)) != LT_OK) return st;
    if (!gpu_setup) {  // the device set the lights up otherwise (above)
        if ((st = upload(c, h.lights, &d.lights)) != LT_OK) return st;
        const float *ltris = nullptr;
        if ((st = upload(c, h.light_tris, &ltris)) != LT_OK) return st;
        d.light_tris = (const float4 *)ltris;
    }
    d.num_lights = (uint32_t)h.lights.size();
    d.num_tris = (uint32_t)h.tri_geom.size();
    d.num_nodes = c->num_nodes;
    d.num_geoms = (uint32_t)h.geoms.size();
    d.num_mats = (uint32_t)h.materials.size();
    d.num_media = (uint32_t)h.media.size();
    d.background = h.background;
    d.cam = h.camera;
    d.filter = h.filter;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->has_scene = true;
    return ensure_width(c, c->tuning.bvh_width);
} LT_CATCH(c)

lt_status lt_scene_destroy(lt_ctx *c) try {
    if (!c) return LT_ERR_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    free_graph(c);  // its scene table entries point into the scene
    free_scene(c);
    c->host = HostScene{};
    return LT_OK;
} LT_CATCH(c)

lt_status lt_scene_info_get(lt_ctx *c, lt_scene_info *out) try {
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
} LT_CATCH(c)

lt_status lt_scene_lights_get(lt_ctx *c, lt_light_info *out, uint32_t capacity) try {
    if (!c || (capacity && !out)) return fail(c, LT_ERR_INVALID, "NULL argument");
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    const std::vector<LightInfo> &L = c->host.lights;
    if (capacity < L.size()) return fail(c, LT_ERR_INVALID, "capacity %u below the %zu lights", capacity, L.size());
    for (size_t i = 0; i < L.size(); ++i) {
        lt_light_info &o = out[i];
        o.mesh = (uint32_t)L[i].geom;
        o.num_triangles = L[i].tri_count;
        o.area = L[i].area;
        memcpy(o.sphere, L[i].sphere, sizeof o.sphere);
        memcpy(o.radiance, L[i].radiance, sizeof o.radiance);
    }
    return LT_OK;
} LT_CATCH(c)

lt_status lt_scene_mesh_offsets(lt_ctx *c, uint32_t *first, uint32_t capacity) try {
    if (!c || !first) return LT_ERR_INVALID;
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    if (capacity < c->host.geoms.size()) return fail(c, LT_ERR_INVALID, "capacity below mesh count");
    for (size_t g = 0; g < c->host.geoms.size(); ++g) first[g] = c->host.geoms[g].first_tri;
    return LT_OK;
} LT_CATCH(c)

}  // extern "C"

static lt_status ensure_scratch(lt_ctx *c, size_t bytes) {
    if (c->scratch_bytes >= bytes) return LT_OK;
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    CUDA_TRY(c, dev_malloc(&c->scratch, bytes));
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
    w->check_pixels = g_check_pixels.load();
    return off;
}

// Wavefront sizes. Without a paths_in_flight tuning a context's arena holds up
// to kDefaultPaths slots (16M, 4.6 GB); fewer, longer iterations amortise each
// launch's tail: on the 1.3M-triangle workload (67M samples) 2M slots give
// 941 Msamples/s, 8M 1268, 16M 1341, the whole render (64M) 1498.
constexpr unsigned long long kDefaultPaths = 1ull << 24, kMinDefaultPaths = 1ull << 20, kMaxPaths = 1ull << 26;

// Sizes the context's wavefront arena for *cap entries (one allocation,
// reused). With `shrink` (the default size), an allocation that fails is
// retried at half the size down to kMinDefaultPaths; *cap is the size obtained.
static lt_status ensure_wave(lt_ctx *c, uint32_t *cap, bool shrink) {
    if (c->wave.capacity >= *cap && c->wave.arena) return LT_OK;
    free_wave(c);
    for (;;) {
        Wavefront sizing;
        const size_t bytes = carve_wave(nullptr, *cap, &sizing);
        char *a = nullptr;
        const cudaError_t e = dev_malloc((void **)&a, bytes);
        if (e == cudaSuccess) {
            carve_wave(a, *cap, &c->wave);
            c->wave.arena = a;
            c->wave.arena_bytes = bytes;
            return LT_OK;
        }
        cudaGetLastError();
        if (!shrink || e != cudaErrorMemoryAllocation || *cap / 2 < kMinDefaultPaths)
            return fail(c, e == cudaErrorMemoryAllocation ? LT_ERR_OOM : LT_ERR_CUDA,
                        "wavefront arena of %zu bytes: %s", bytes, cudaGetErrorString(e));
        *cap /= 2;
    }
}

// Paths in flight for `total` work items (never more than the work): the
// tuning's count, else kDefaultPaths. Allocates the arena.
static lt_status prepare_wave(lt_ctx *c, unsigned long long total, uint32_t *cap_out) {
    const bool fixed = c->tuning.paths_in_flight != 0;
    const unsigned long long cap = fixed ? c->tuning.paths_in_flight : kDefaultPaths;
    uint32_t n = (uint32_t)(total < cap ? total : cap);
    const lt_status st = ensure_wave(c, &n, !fixed);
    *cap_out = n;
    return st;
}

// The context's arena laid out for `cap` entries (cap <= the arena's capacity).
static Wavefront wave_view(const lt_ctx *c, uint32_t cap) {
    Wavefront w;
    w.arena_bytes = carve_wave((char *)c->wave.arena, cap, &w);
    w.arena = c->wave.arena;
    w.qtrace = c->qtrace_dev;
    w.qtrace_cap = c->qtrace_cap;
    return w;
}

// Builds the 4-wide BVH of the context's scene from its BVH2 (read back from
// the device when the GPU built it) and uploads it; its leaves index the
// BVH2's triangles.
static lt_status ensure_bvh4(lt_ctx *c) {
    if (c->has_bvh4) return LT_OK;
    if (!c->has_scene) return fail(c, LT_ERR_STATE, "no scene");
    std::vector<BvhNode> nodes = c->host.nodes;
    if (nodes.empty()) {
        nodes.resize(c->num_nodes);
        CUDA_TRY(c, cudaMemcpyAsync(nodes.data(), c->dev.nodes, nodes.size() * sizeof(BvhNode),
                                    cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    std::vector<Bvh4Node> n4;
    const uint32_t depth = build_bvh4(nodes, &n4);
    if (3 * depth + 1 > 64)
        return fail(c, LT_ERR_UNSUPPORTED, "4-wide BVH depth %u exceeds the traversal stack", depth);
    std::vector<float> nf(n4.size() * 32);
    memcpy(nf.data(), n4.data(), nf.size() * sizeof(float));
    const float *d_nodes = nullptr;
    lt_status st = upload(c, nf, &d_nodes);
    if (st != LT_OK) return st;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->dev.nodes4 = (const float4 *)d_nodes;
    c->dev.num_nodes4 = (uint32_t)n4.size();
    c->has_bvh4 = true;
    return LT_OK;
}

static lt_status ensure_width(lt_ctx *c, uint32_t width) {
    if (width == 8) return ensure_bvh8(c);
    if (width == 4) return ensure_bvh4(c);
    return LT_OK;
}

// The wavefront loop of one render over `w`: camera rays, then batches of
// (trace, shade) iterations, reading the queue lengths back after each batch
// until no path ray, camera ray or connection record is left. With
// stage_timing a pair of events brackets every kernel launch, so that
// lt_render_stats gets each stage's kernel time (init_ms, trace_ms, shade_ms)
// apart from the time the stream waits for the host between batches; without
// it nothing is created or allocated. Fills c->stats (except samples and gpu_ms).
// `init` and `stage(stage, cur)` launch the kernels (plain or differentiable);
// an iteration is `per_iteration` launches.
template <class Init, class Stage>
static lt_status run_loop(lt_ctx *c, const Wavefront &w, const RenderArgs &a, bool stage_timing,
                          uint32_t per_iteration, Init init, Stage launch_stage) {
    const uint32_t cap = w.capacity;
    size_t nev = 0;
    if (stage_timing) c->stage_of_event.clear();
    constexpr int kStageInit = kStages;  // the camera-ray kernel, after the two loop stages
    // records the event before (after = false) or after a launch of `stage`
    auto mark = [&](int stage, bool after) -> cudaError_t {
        if (!stage_timing) return cudaSuccess;
        if (nev == c->stage_events.size()) {
            cudaEvent_t e;
            const cudaError_t ce = cudaEventCreate(&e);
            if (ce != cudaSuccess) return ce;
            c->stage_events.push_back(e);
        }
        if (!after) c->stage_of_event.push_back(stage);
        return cudaEventRecord(c->stage_events[nev++], c->stream);
    };
    CUDA_TRY(c, cudaMemsetAsync(w.counters, 0, sizeof(WaveCounters), c->stream));
    CUDA_TRY(c, mark(kStageInit, false));
    CUDA_TRY(c, init());
    CUDA_TRY(c, mark(kStageInit, true));
    uint32_t launches = 1;
    unsigned long long iters = 0;
    int cur = 0;
    const unsigned long long limit = drain_limit(a.total, cap, a.max_depth);
    // Iterations launched between two reads of the queue lengths. While work
    // items remain, at most `cap` of them start per iteration, so the loop
    // cannot end within remaining / cap iterations.
    unsigned long long batch = first_batch(a.total, cap, a.max_depth);
    for (;;) {
        if (batch > limit - iters) batch = limit - iters;  // iters < limit here
        for (unsigned long long k = 0; k < batch; ++k) {
            for (int stage = 0; stage < kStages; ++stage) {
                CUDA_TRY(c, mark(stage, false));
                CUDA_TRY(c, launch_stage(stage, cur));
                CUDA_TRY(c, mark(stage, true));
            }
            launches += per_iteration;
            cur ^= 1;
            ++iters;
        }
        CUDA_TRY(c, cudaMemcpyAsync(c->counters_host, w.counters, sizeof(WaveCounters), cudaMemcpyDeviceToHost,
                                    c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if (c->counters_host->check) return check_failed(c, *c->counters_host);
        // done when no path ray is queued and the last shade emitted no connection
        if (c->counters_host->count[cur] == 0 && c->counters_host->rcount[cur] == 0 &&
            c->counters_host->ccount[cur ^ 1] == 0)
            break;
        if (iters >= limit) return fail(c, LT_ERR_TIMEOUT, "wavefront did not drain after %llu iterations", iters);
        const unsigned long long next = c->counters_host->work_next;
        const unsigned long long left_iters = next < a.total ? (a.total - next) / cap : 0;
        batch = left_iters > 4 ? (left_iters < 64 ? left_iters : 64ull) : 4ull;
    }
    const WaveCounters &k = *c->counters_host;
    c->stats.main_rays = k.main_rays;
    c->stats.light_rays = k.light_rays;
    c->stats.bsdf_rays = k.bsdf_rays;
    c->stats.nonfinite_samples = k.nonfinite;
    c->stats.light_traversals = k.light_traversals;
    c->stats.iterations = (uint32_t)iters;
    c->qtrace_rows = w.qtrace ? (k.trace_launches < w.qtrace_cap ? k.trace_launches : w.qtrace_cap) : 0u;
    c->stats.kernel_launches = launches;
    if (stage_timing) {  // the stream has been synchronised: every event has completed
        float acc[kStages + 1] = {0, 0, 0};
        for (size_t i = 0; i + 1 < nev; i += 2) {
            float ms = 0.0f;
            CUDA_TRY(c, cudaEventElapsedTime(&ms, c->stage_events[i], c->stage_events[i + 1]));
            acc[c->stage_of_event[i / 2]] += ms;
        }
        c->stats.trace_ms = acc[kStageTrace];
        c->stats.shade_ms = acc[kStageShade];
        c->stats.init_ms = acc[kStageInit];
    }
    return LT_OK;
}

static lt_status run_wave(lt_ctx *c, const Wavefront &w, const RenderArgs &a, const FilmPtrs &f, bool stage_timing) {
    return run_loop(
        c, w, a, stage_timing, launches_per_iteration(c->shape),
        [&]() { return launch_wave_init(c->dev, w, a, f, c->shape, c->stream); },
        [&](int stage, int cur) { return launch_wave_stage(stage, c->dev, w, a, f, cur, c->shape, c->stream); });
}

extern "C" {

lt_status lt_render(lt_ctx *c, const lt_render_params *p, lt_film *film) try {
    NvtxRange nvtx_("lt_render");
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
        uint32_t cap = 0;
        lt_status st = prepare_wave(c, a.total, &cap);
        if (st != LT_OK) return st;
        const Wavefront w = wave_view(c, cap);
        if ((st = run_wave(c, w, a, f, c->stage_timing)) != LT_OK) return st;
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
} LT_CATCH(c)

lt_status lt_render_stats_get(lt_ctx *c, lt_render_stats *out) try {
    if (!c || !out) return LT_ERR_INVALID;
    *out = c->stats;
    float ms = 0.0f;
    if (cudaEventSynchronize(c->ev1) == cudaSuccess && cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess)
        out->gpu_ms = ms;
    if (out->trace_ms + out->shade_ms + out->init_ms > 0.0f) {
        const float busy = out->trace_ms + out->shade_ms + out->init_ms;
        out->idle_ms = out->gpu_ms > busy ? out->gpu_ms - busy : 0.0f;
    }
    return LT_OK;
} LT_CATCH(c)

lt_status lt_intersect(lt_ctx *c, const lt_ray *rays, lt_hit *hits, uint64_t n, int32_t on_device) try {
    NvtxRange nvtx_("lt_intersect");
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
} LT_CATCH(c)

lt_status lt_diff_defaults(lt_ctx *c, float *albedo, float *emission, float *sigma_a, float *sigma_s) try {
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
} LT_CATCH(c)

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

// Lays the differentiable forward's path extras out from `base` for `cap`
// paths (each array 256-byte aligned); returns the bytes used (base may be
// nullptr to size).
static size_t carve_dwave(char *base, uint32_t cap, DiffWave *d) {
    const size_t P = cap;
    size_t off = 0;
    auto take = [&](size_t n) { char *p = base + off; off += (n + 255) & ~(size_t)255; return p; };
    for (int k = 0; k < 2; ++k) {
        d->C[k] = (float *)take(12 * P);
        d->Ts[k] = (float *)take(12 * P);
        d->rec[k] = (uint2 *)take(8 * P);
        d->fin_id[k] = (uint4 *)take(16 * P);
        d->fin_C[k] = (float4 *)take(16 * P);
        d->fin_rec[k] = (uint2 *)take(8 * P);
        d->pend[k] = (uint32_t *)take(4 * P);
    }
    d->res = (float4 *)take(32 * P);  // two connection records per path
    d->aux = (float2 *)take(16 * P);
    d->gres = (float4 *)take(64 * P);
    d->sample_I = nullptr;
    d->bytes = off;
    return off;
}

static lt_status ensure_dwave(lt_ctx *c, uint32_t cap, DiffWave *d) {
    if (c->diff_capacity < cap || !c->diff_arena) {
        if (c->diff_arena) {
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            cudaFree(c->diff_arena);
        }
        c->diff_arena = nullptr;
        c->diff_capacity = 0;
        DiffWave sizing;
        const size_t bytes = carve_dwave(nullptr, cap, &sizing);
        CUDA_TRY(c, dev_malloc(&c->diff_arena, bytes));
        c->diff_arena_bytes = bytes;
        c->diff_capacity = cap;
    }
    carve_dwave((char *)c->diff_arena, cap, d);
    return LT_OK;
}

// The wavefront of a differentiable forward for `total` samples: the plain
// arena (prepare_wave) and the path extras for as many paths. When the extras
// do not fit, the number of paths in flight is halved (down to
// kMinDefaultPaths) rather than failing: the plain arena then serves a
// smaller view. Returns the capacity in *cap.
static lt_status prepare_dwave(lt_ctx *c, unsigned long long total, uint32_t *cap, Wavefront *w, DiffWave *d) {
    lt_status st = prepare_wave(c, total, cap);
    if (st != LT_OK) return st;
    for (;;) {
        st = ensure_dwave(c, *cap, d);
        if (st == LT_OK) break;
        if (st != LT_ERR_OOM || *cap / 2 < kMinDefaultPaths) return st;
        cudaGetLastError();
        *cap /= 2;
    }
    *w = wave_view(c, *cap);
    return LT_OK;
}

static lt_status ensure_diff_samples(lt_ctx *c, size_t bytes) {
    if (c->diff_samples_bytes >= bytes && c->diff_samples) return LT_OK;
    if (c->diff_samples) {
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        cudaFree(c->diff_samples);
    }
    c->diff_samples = nullptr;
    c->diff_samples_bytes = 0;
    CUDA_TRY(c, dev_malloc((void **)&c->diff_samples, bytes));
    c->diff_samples_bytes = bytes;
    return LT_OK;
}

}  // extern "C"

// The differentiable forward on the wavefront over a.total samples of scene
// `dev` into film f, every sample's radiance into sample_I, on c's arena and
// stream; then the film's colour sums in sample order. Fills c->stats as
// run_loop does.
static lt_status diff_wave(lt_ctx *c, const DevScene &dev, const DiffParams &P, const RenderArgs &a,
                           const FilmPtrs &f, float *sample_I) {
    uint32_t cap = 0;
    Wavefront w;
    DiffWave d;
    lt_status st = prepare_dwave(c, a.total, &cap, &w, &d);
    if (st != LT_OK) return st;
    d.sample_I = sample_I;
    st = run_loop(
        c, w, a, c->stage_timing, kStages + 1u, [&]() { return launch_dwave_init(dev, P, d, w, a, f, c->shape, c->stream); },
        [&](int stage, int cur) { return launch_dwave_stage(stage, dev, P, d, w, a, f, cur, c->shape, c->stream); });
    if (st != LT_OK) return st;
    CUDA_TRY(c, launch_diff_film(d.sample_I, a, f, c->stream));
    c->stats.kernel_launches += 1;
    return LT_OK;
}

extern "C" {

lt_status lt_render_diff(lt_ctx *c, const lt_render_params *p, const lt_diff_params *dp, lt_film *film,
                         float *sample_radiance) try {
    NvtxRange nvtx_("lt_render_diff");
    if (!c || !p || !dp || !film) return fail(c, LT_ERR_INVALID, "NULL argument");
    DiffParams P;
    RenderArgs a;
    lt_status st = diff_setup(c, p, dp, &P, &a);
    if (st != LT_OK) return st;
    if (!film->on_device || film->width != a.width || film->height != a.height)
        return fail(c, LT_ERR_INVALID, "lt_render_diff needs a device film of the camera's size");
    if (!film->rgb || !film->bounces || !film->counts) return fail(c, LT_ERR_INVALID, "film buffers missing");
    FilmPtrs f{film->rgb, film->bounces, film->counts};
    const uint32_t npix = a.width * a.height;
    c->stats = lt_render_stats{};
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    if (a.total > 0 && p->max_depth == 0) {  // the bounce loop never runs: every sample's radiance is 0
        if (sample_radiance) CUDA_TRY(c, cudaMemsetAsync(sample_radiance, 0, a.total * 12, c->stream));
        CUDA_TRY(c, launch_add_counts(f, npix, p->spp, c->stream));
        c->stats.kernel_launches = 1;
    } else if (a.total > 0) {
        if (!sample_radiance) {
            if ((st = ensure_diff_samples(c, a.total * 12)) != LT_OK) return st;
            sample_radiance = c->diff_samples;
        }
        if ((st = diff_wave(c, c->dev, P, a, f, sample_radiance)) != LT_OK) return st;
    }
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    c->stats.samples = a.total;
    return LT_OK;
} LT_CATCH(c)

}  // extern "C"

// The adjoint on the wavefront over a.total samples of scene `dev` (the
// crop's, G.x0..y1): the forward's paths replayed from their seeds on c's
// arena and stream. Fills c->stats as run_loop does.
static lt_status adjoint_wave(lt_ctx *c, const DevScene &dev, const DiffParams &P, const RenderArgs &a,
                              const DiffGrads &G) {
    uint32_t cap = 0;
    Wavefront w;
    DiffWave d;
    lt_status st = prepare_dwave(c, a.total, &cap, &w, &d);
    if (st != LT_OK) return st;
    return run_loop(
        c, w, a, c->stage_timing, kStages + 1u, [&]() { return launch_awave_init(dev, P, d, G, w, a, c->shape, c->stream); },
        [&](int stage, int cur) { return launch_awave_stage(stage, dev, P, d, G, w, a, cur, c->shape, c->stream); });
}

extern "C" {

lt_status lt_render_adjoint(lt_ctx *c, const lt_render_params *p, const lt_diff_params *dp, const float *dI,
                            float *g_albedo, float *g_emission, float *g_sigma_a, float *g_sigma_s,
                            const uint32_t *crop, const float *sample_radiance) try {
    NvtxRange nvtx_("lt_render_adjoint");
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
    const unsigned long long crop_samples =
        (unsigned long long)(G.x1 - G.x0) * (G.y1 - G.y0) * (a.total / ((unsigned long long)a.width * a.height));
    if (sample_radiance && crop_samples > 0 && p->max_depth > 0) {
        RenderArgs aa = a;
        aa.total = crop_samples;
        if ((st = adjoint_wave(c, c->dev, P, aa, G)) != LT_OK) return st;
    } else if (!sample_radiance) {
        // without the forward's radiance: one thread replays each sample twice
        // (the adjoint's work counter: 8 bytes of the context's counter block, after lt_intersect's)
        CUDA_TRY(c, launch_diff_adjoint(c->dev, P, a, G, (uint32_t)c->host.media.size(),
                                        (unsigned long long *)(c->isect_fetch + 16), c->shape, c->stream));
        c->stats.kernel_launches = 1;
    }
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    c->stats.samples = crop_samples;
    return LT_OK;
} LT_CATCH(c)

lt_status lt_scene_load_json(lt_ctx *c, const char *path) try {
    if (!c || !path) return fail(c, LT_ERR_INVALID, "NULL argument");
    lt_scene_desc desc;
    JsonSceneStorage storage;
    std::string err;
    lt_status st = load_scene_json(path, &desc, &storage, &err);
    if (st != LT_OK) return fail(c, st, "%s", err.c_str());
    return lt_scene_create(c, &desc);
} LT_CATCH(c)

}  // extern "C"

// ------------------------------------------------------------------ lt_render_noalloc
// Same wavefront as lt_render, with its state carved out of the fixed device
// array of lt_noalloc.cu instead of a cudaMalloc'd arena. Nothing here
// allocates: no cudaMalloc / cudaFree / cudaMallocHost, no new CUDA events, no
// staging buffers (the film must already be on the device).
static Wavefront carve_noalloc(char *a, uint32_t cap) {
    Wavefront w;
    w.arena_bytes = carve_wave(a, cap, &w);
    w.arena = nullptr;  // not owned: never freed
    return w;
}

extern "C" lt_status lt_render_noalloc(lt_ctx *c, const lt_render_params *p, lt_film *film,
                                       uint32_t paths_in_flight) try {
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
        // the array keeps the previous call's contents: run_wave zeroes the
        // counters before anything reads them
        lt_status st = run_wave(c, w, a, f, false);
        if (st != LT_OK) return st;
    }
    c->stats.samples = a.total;
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    return LT_OK;
} LT_CATCH(c)

// ------------------------------------------------------------------ tuning
extern "C" lt_status lt_get_tuning(const lt_ctx *c, lt_tuning *out) {
    if (!c || !out) return LT_ERR_INVALID;
    *out = c->tuning;
    return LT_OK;
}

static bool valid_threads(uint32_t t) { return t == 64 || t == 128 || t == 256; }
static bool valid_shade_threads(uint32_t t) { return valid_threads(t) || t == 512; }

extern "C" lt_status lt_set_queue_trace(lt_ctx *c, uint32_t rows) try {
    if (!c) return LT_ERR_INVALID;
    if (rows > LT_QUEUE_TRACE_MAX_ROWS)
        return fail(c, LT_ERR_INVALID, "%u rows; the queue trace holds at most %u", rows, LT_QUEUE_TRACE_MAX_ROWS);
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // no queued kernel still writes the old rows
    if (c->qtrace_dev) cudaFree(c->qtrace_dev);
    c->qtrace_dev = nullptr;
    c->qtrace_cap = c->qtrace_rows = 0;
    if (rows) {
        CUDA_TRY(c, dev_malloc((void **)&c->qtrace_dev, (size_t)rows * sizeof(uint3)));
        c->qtrace_cap = rows;
    }
    return LT_OK;
} LT_CATCH(c)

extern "C" lt_status lt_queue_trace_get(lt_ctx *c, lt_queue_lengths *out, uint32_t capacity, uint32_t *rows) try {
    if (!c || !rows || (capacity && !out)) return fail(c, LT_ERR_INVALID, "NULL argument");
    *rows = c->qtrace_rows;
    const uint32_t n = c->qtrace_rows < capacity ? c->qtrace_rows : capacity;
    if (n) {
        static_assert(sizeof(lt_queue_lengths) == sizeof(uint3), "queue trace row layout");
        CUDA_TRY(c, cudaSetDevice(c->device));
        CUDA_TRY(c, cudaMemcpyAsync(out, c->qtrace_dev, (size_t)n * sizeof(uint3), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    return LT_OK;
} LT_CATCH(c)

extern "C" lt_status lt_set_stage_timing(lt_ctx *c, int32_t on) try {
    if (!c) return LT_ERR_INVALID;
    c->stage_timing = on != 0;
    return LT_OK;
} LT_CATCH(c)

extern "C" lt_status lt_set_tuning(lt_ctx *c, const lt_tuning *t) try {
    if (!c || !t) return fail(c, LT_ERR_INVALID, "NULL argument");
    lt_tuning n;
    default_tuning(&n);
    n.paths_in_flight = t->paths_in_flight;
    if (t->trace_threads) n.trace_threads = t->trace_threads;
    if (t->shade_threads) n.shade_threads = t->shade_threads;
    if (t->loop_iterations) n.loop_iterations = t->loop_iterations;
    if (t->bvh_width) n.bvh_width = t->bvh_width;
    n.ms = t->ms;
    if (!valid_threads(n.trace_threads) || !valid_shade_threads(n.shade_threads))
        return fail(c, LT_ERR_INVALID, "threads per block must be 64, 128 or 256 (512 also for the shade kernel)");
    if (n.loop_iterations != 2 && n.loop_iterations != 4 && n.loop_iterations != 8)
        return fail(c, LT_ERR_INVALID, "loop_iterations must be 2, 4 or 8");
    if (n.bvh_width != 2 && n.bvh_width != 4 && n.bvh_width != 8)
        return fail(c, LT_ERR_UNSUPPORTED, "BVH width %u: the widths built are 2, 4 and 8", n.bvh_width);
    if (n.paths_in_flight && (n.paths_in_flight < 1024 || n.paths_in_flight > kMaxPaths))
        return fail(c, LT_ERR_INVALID, "paths_in_flight %u outside 1024..67108864", n.paths_in_flight);
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (c->has_scene) {
        lt_status st = ensure_width(c, n.bvh_width);
        if (st != LT_OK) return st;
    }
    c->tuning = n;
    apply_tuning(c);
    return LT_OK;
} LT_CATCH(c)

// ------------------------------------------------------------------ lt_render_batch
// Captures the batched loop for wavefront `w`: memset(counters), camera rays,
// then a while node whose body runs loop_iterations (trace, shade)
// iterations and the condition kernel. Captured on the context's own stream in
// thread-local mode, so other threads' CUDA calls are not affected.
static lt_status build_batch_graph(lt_ctx *c, const Wavefront &w) {
    std::vector<uintptr_t> key = {(uintptr_t)c->wave.arena, w.capacity, (uintptr_t)c->table_dev,
                                  (uintptr_t)c->batch_shape.trace_threads, (uintptr_t)c->batch_shape.trace_blocks,
                                  (uintptr_t)c->batch_shape.shade_threads, (uintptr_t)c->batch_shape.shade_blocks,
                                  (uintptr_t)c->batch_shape.bvh_width, c->tuning.loop_iterations,
                                  (uintptr_t)c->batch_shape.tail_blocks, (uintptr_t)c->batch_shape.coop_limit,
                                  (uintptr_t)w.check_pixels, (uintptr_t)w.qtrace, (uintptr_t)w.qtrace_cap};
    if (c->graph_exec && key == c->graph_key) return LT_OK;
    free_graph(c);
    cudaStream_t cs = c->own_stream;
    CUDA_TRY(c, cudaGraphCreate(&c->graph, 0));
    cudaGraphConditionalHandle h;
    CUDA_TRY(c, cudaGraphConditionalHandleCreate(&h, c->graph, 1, cudaGraphCondAssignDefault));

    // prologue, then the while node appended to the capture
    CUDA_TRY(c, cudaStreamBeginCaptureToGraph(cs, c->graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};  // the rest zero
    cudaError_t e = cudaMemsetAsync(w.counters, 0, sizeof(WaveCounters), cs);
    if (e == cudaSuccess) e = launch_batch_init(c->table_dev, w, c->batch_shape, cs);
    if (e == cudaSuccess) {
        cudaStreamCaptureStatus status;
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        e = cudaStreamGetCaptureInfo(cs, &status, nullptr, nullptr, &deps, nullptr, &ndeps);
        if (e == cudaSuccess) {
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t cond;
            e = cudaGraphAddNode(&cond, c->graph, deps, nullptr, ndeps, &cp);
            if (e == cudaSuccess)
                e = cudaStreamUpdateCaptureDependencies(cs, &cond, nullptr, 1, cudaStreamSetCaptureDependencies);
        }
    }
    cudaGraph_t captured = nullptr;
    cudaError_t e_end = cudaStreamEndCapture(cs, &captured);
    CUDA_TRY(c, e);
    CUDA_TRY(c, e_end);

    // loop body
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CUDA_TRY(c, cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int cur = 0;
    for (uint32_t k = 0; k < c->tuning.loop_iterations && e == cudaSuccess; ++k) {
        for (int stage = 0; stage < kStages && e == cudaSuccess; ++stage)
            e = launch_batch_stage(stage, c->table_dev, w, cur, c->batch_shape, cs);
        cur ^= 1;
    }
    if (e == cudaSuccess) e = launch_loop_condition(w, c->table_dev, h, cur, c->tuning.loop_iterations, cs);
    e_end = cudaStreamEndCapture(cs, &captured);
    CUDA_TRY(c, e);
    CUDA_TRY(c, e_end);
    CUDA_TRY(c, cudaGraphInstantiate(&c->graph_exec, c->graph, 0));
    c->graph_key = key;
    return LT_OK;
}

// The scene table's host and device copies; waits until the last queued
// reader of the table (and with it the upload from the pinned host copy) has
// completed, so that the host may rewrite the pinned copy.
static lt_status ensure_table(lt_ctx *c) {
    if (!c->table_host) {
        CUDA_TRY(c, host_malloc((void **)&c->table_host, sizeof(SceneTable)));
        CUDA_TRY(c, dev_malloc((void **)&c->table_dev, sizeof(SceneTable)));
    }
    CUDA_TRY(c, (cudaError_t)c->order.before_table_write(c->rt));
    return LT_OK;
}

extern "C" lt_status lt_render_batch(lt_ctx *c, lt_ctx *const *scenes, const lt_render_params *params,
                                     lt_film *films, uint32_t n) try {
    NvtxRange nvtx_("lt_render_batch");
    if (!c || (n && (!scenes || !params || !films))) return fail(c, LT_ERR_INVALID, "NULL argument");
    if (n > LT_MAX_BATCH) return fail(c, LT_ERR_INVALID, "%u scenes; a batch holds at most %u", n, LT_MAX_BATCH);
    CUDA_TRY(c, cudaSetDevice(c->device));
    lt_status st0 = ensure_table(c);
    if (st0 != LT_OK) return st0;
    SceneTable &T = *c->table_host;
    uint32_t count = 0, max_depth = 0, launches = 0;
    unsigned long long total = 0;
    c->stats = lt_render_stats{};
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    // A scene whose samples fill the wavefront by themselves gains nothing from
    // the others' company and runs with the single-scene kernels after the
    // captured loop (64-scene workload: 295.3 ms all in the loop, 285.6 ms with
    // its five 1024x1024 x 64-spp scenes alone).
    const unsigned long long wave_limit = c->tuning.paths_in_flight ? c->tuning.paths_in_flight : kDefaultPaths;
    std::vector<uint32_t> alone;
    unsigned long long alone_max = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const lt_ctx *s = scenes[i];
        const lt_render_params &p = params[i];
        const lt_film &f = films[i];
        if (!s || !s->has_scene) return fail(c, LT_ERR_STATE, "batch scene %u: no scene", i);
        if (s->device != c->device) return fail(c, LT_ERR_INVALID, "batch scene %u is on another device", i);
        if ((c->tuning.bvh_width == 8 && !s->has_bvh8) || (c->tuning.bvh_width == 4 && !s->has_bvh4)) {
            lt_status sb = ensure_width(const_cast<lt_ctx *>(s), c->tuning.bvh_width);
            if (sb != LT_OK) return fail(c, sb, "batch scene %u: %s", i, s->error.c_str());
        }
        const uint32_t W = s->host.camera.width, H = s->host.camera.height;
        if (!f.on_device || f.width != W || f.height != H || !f.rgb || !f.bounces || !f.counts)
            return fail(c, LT_ERR_INVALID, "batch film %u: needs device buffers of %ux%u", i, W, H);
        const unsigned long long items = (unsigned long long)W * H * p.spp;
        if (items == 0) continue;
        FilmPtrs fp{f.rgb, f.bounces, f.counts};
        if (p.max_depth == 0) {  // the bounce loop never runs
            CUDA_TRY(c, launch_add_counts(fp, W * H, p.spp, c->stream));
            ++launches;
            continue;
        }
        if (items >= wave_limit) {
            alone.push_back(i);
            if (items > alone_max) alone_max = items;
            continue;
        }
        SceneSlot &slot = T.slots[count];
        slot.s = s->dev;
        slot.a = RenderArgs{W, H, p.first_frame, p.max_depth, p.rr_depth, items};
        slot.f = fp;
        T.begin[count] = total;
        total += items;
        if (p.max_depth > max_depth) max_depth = p.max_depth;
        ++count;
    }
    uint32_t cap_max = 0;  // one arena for the loop and the scenes alone
    if (count || !alone.empty()) {
        lt_status st = prepare_wave(c, total > alone_max ? total : alone_max, &cap_max);
        if (st != LT_OK) return st;
    }
    if (count) {
        lt_status st = LT_OK;
        const uint32_t cap = (uint32_t)(total < cap_max ? total : cap_max);
        const Wavefront w = wave_view(c, cap);
        T.count = count;
        T.pad = 0;
        T.total = total;
        T.iteration_limit = drain_limit(total, cap, max_depth);
        CUDA_TRY(c, cudaMemcpyAsync(c->table_dev, c->table_host, offsetof(SceneTable, slots), cudaMemcpyHostToDevice,
                                    c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(c->table_dev->slots, T.slots, count * sizeof(SceneSlot), cudaMemcpyHostToDevice,
                                    c->stream));
        if ((st = build_batch_graph(c, w)) != LT_OK) return st;
        CUDA_TRY(c, cudaGraphLaunch(c->graph_exec, c->stream));
        CUDA_TRY(c, (cudaError_t)c->order.table_read_queued(c->rt, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(c->counters_host, w.counters, sizeof(WaveCounters), cudaMemcpyDeviceToHost,
                                    c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        const WaveCounters &k = *c->counters_host;
        if (k.check) return check_failed(c, k);
        if (k.error == 2) return fail(c, LT_ERR_TIMEOUT, "batched wavefront did not drain in %llu iterations", k.iterations);
        c->stats.main_rays = k.main_rays;
        c->stats.light_rays = k.light_rays;
        c->stats.bsdf_rays = k.bsdf_rays;
        c->stats.iterations = (uint32_t)k.iterations;
        launches += 1 + launches_per_iteration(c->batch_shape) * (uint32_t)k.iterations +
                    (uint32_t)(k.iterations / c->tuning.loop_iterations);
        c->stats.light_traversals = k.light_traversals;
        c->stats.nonfinite_samples = k.nonfinite;
        c->qtrace_rows = w.qtrace ? (k.trace_launches < w.qtrace_cap ? k.trace_launches : w.qtrace_cap) : 0u;
    }
    lt_render_stats acc = c->stats;
    for (uint32_t i : alone) {
        const lt_ctx *s = scenes[i];
        const lt_render_params &p = params[i];
        const uint32_t W = s->host.camera.width, H = s->host.camera.height;
        const RenderArgs a{W, H, p.first_frame, p.max_depth, p.rr_depth, (unsigned long long)W * H * p.spp};
        const FilmPtrs fp{films[i].rgb, films[i].bounces, films[i].counts};
        const Wavefront w = wave_view(c, (uint32_t)(a.total < cap_max ? a.total : cap_max));
        const lt_status st = run_loop(
            c, w, a, false, launches_per_iteration(c->shape),
            [&]() { return launch_wave_init(s->dev, w, a, fp, c->shape, c->stream); },
            [&](int stage, int cur) { return launch_wave_stage(stage, s->dev, w, a, fp, cur, c->shape, c->stream); });
        if (st != LT_OK) return st;
        launches += c->stats.kernel_launches;
        acc.iterations += c->stats.iterations;
        acc.main_rays += c->stats.main_rays;
        acc.light_rays += c->stats.light_rays;
        acc.bsdf_rays += c->stats.bsdf_rays;
        acc.light_traversals += c->stats.light_traversals;
        acc.nonfinite_samples += c->stats.nonfinite_samples;
        total += a.total;
    }
    c->stats = acc;
    c->stats.samples = total;
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->stats.kernel_launches = launches;
    return LT_OK;
} LT_CATCH(c)

// ------------------------------------------------------------------ lt_autotune_batch
extern "C" lt_status lt_autotune_batch(lt_ctx *c, lt_ctx *const *scenes, const lt_render_params *params, uint32_t n,
                                       uint32_t spp_cap, lt_tuning *best) try {
    if (!c || !n || !scenes || !params) return fail(c, LT_ERR_INVALID, "NULL argument or empty batch");
    if (n > LT_MAX_BATCH) return fail(c, LT_ERR_INVALID, "%u scenes; a batch holds at most %u", n, LT_MAX_BATCH);
    if (spp_cap == 0) spp_cap = 1;
    CUDA_TRY(c, cudaSetDevice(c->device));
    // scratch films, one per scene, and the capped render parameters
    std::vector<lt_render_params> prm(params, params + n);
    std::vector<size_t> off(n);
    size_t bytes = 0;
    for (uint32_t i = 0; i < n; ++i) {
        if (!scenes[i] || !scenes[i]->has_scene) return fail(c, LT_ERR_STATE, "batch scene %u: no scene", i);
        if (prm[i].spp > spp_cap) prm[i].spp = spp_cap;
        off[i] = bytes;
        bytes += ((size_t)scenes[i]->host.camera.width * scenes[i]->host.camera.height * 20 + 255) & ~(size_t)255;
    }
    lt_status st = ensure_scratch(c, bytes);
    if (st != LT_OK) return st;
    std::vector<lt_film> films(n);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t W = scenes[i]->host.camera.width, H = scenes[i]->host.camera.height;
        char *b = (char *)c->scratch + off[i];
        films[i].rgb = (float *)b;
        films[i].bounces = (uint32_t *)(b + (size_t)W * H * 12);
        films[i].counts = films[i].bounces + (size_t)W * H;
        films[i].width = W;
        films[i].height = H;
        films[i].on_device = 1;
    }
    auto measure = [&](const lt_tuning &t, float *ms) -> lt_status {
        lt_status s2 = lt_set_tuning(c, &t);
        if (s2 != LT_OK) return s2;
        float best_ms = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {  // the first run also captures the graph
            CUDA_TRY(c, cudaMemsetAsync(c->scratch, 0, bytes, c->stream));
            if ((s2 = lt_render_batch(c, scenes, prm.data(), films.data(), n)) != LT_OK) return s2;
            float m = 0.0f;
            CUDA_TRY(c, cudaEventElapsedTime(&m, c->ev0, c->ev1));
            if (rep > 0 && m < best_ms) best_ms = m;
        }
        *ms = best_ms;
        return LT_OK;
    };
    lt_tuning cur = c->tuning;
    float cur_ms = 0.0f;
    if ((st = measure(cur, &cur_ms)) != LT_OK) return st;
    const uint32_t widths[] = {2, 8};
    const uint32_t paths[] = {1u << 20, 1u << 22, 1u << 24, 1u << 26};
    const uint32_t threads[] = {64, 128, 256};
    const uint32_t iters[] = {2, 4, 8};
    for (int coord = 0; coord < 5; ++coord) {
        const uint32_t *vals = coord == 0 ? widths : coord == 1 ? paths : coord == 4 ? iters : threads;
        const int nv = coord == 0 ? 2 : coord == 1 ? 4 : 3;
        for (int v = 0; v < nv; ++v) {
            lt_tuning t = cur;
            uint32_t *field = coord == 0   ? &t.bvh_width
                              : coord == 1 ? &t.paths_in_flight
                              : coord == 2 ? &t.trace_threads
                              : coord == 3 ? &t.shade_threads
                                           : &t.loop_iterations;
            if (*field == vals[v]) continue;
            *field = vals[v];
            float ms = 0.0f;
            if ((st = measure(t, &ms)) != LT_OK) return st;
            if (ms < cur_ms) {
                cur = t;
                cur_ms = ms;
            }
        }
    }
    cur.ms = cur_ms;
    if ((st = lt_set_tuning(c, &cur)) != LT_OK) return st;
    if (best) *best = c->tuning;
    return LT_OK;
} LT_CATCH(c)

// ------------------------------------------------------------------ lt_resolve
extern "C" lt_status lt_resolve(lt_ctx *c, const lt_film *film, int32_t tonemap, float exposure_stops, float *rgba,
                                uint8_t *rgba8, lt_spp_range *spp) try {
    NvtxRange nvtx_("lt_resolve");
    if (!c || !film) return fail(c, LT_ERR_INVALID, "NULL argument");
    if (tonemap != LT_TONEMAP_CLAMP && tonemap != LT_TONEMAP_FILMIC)
        return fail(c, LT_ERR_INVALID, "unknown tone mapper %d", tonemap);
    if (!film->rgb || !film->counts) return fail(c, LT_ERR_INVALID, "film buffers missing");
    CUDA_TRY(c, cudaSetDevice(c->device));
    const size_t npix = (size_t)film->width * film->height;
    if (npix > 0xFFFFFFFFull) return fail(c, LT_ERR_INVALID, "film too large");
    const float exposure = exp2f(exposure_stops);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    // scratch: [stats][film rgb, counts when on the host][outputs when on the host]
    const bool host = !film->on_device;
    size_t need = al(sizeof(SppStats));
    if (host) need += al(npix * 12) + al(npix * 4) + (rgba ? al(npix * 16) : 0) + (rgba8 ? al(npix * 4) : 0);
    lt_status st = ensure_scratch(c, need);
    if (st != LT_OK) return st;
    char *s = (char *)c->scratch;
    SppStats *d_stats = (SppStats *)s;
    s += al(sizeof(SppStats));
    const float *d_rgb = film->rgb;
    const uint32_t *d_counts = film->counts;
    float4 *d_out = (float4 *)rgba;
    uchar4 *d_out8 = (uchar4 *)rgba8;
    if (host) {
        float *r = (float *)s;
        s += al(npix * 12);
        uint32_t *n = (uint32_t *)s;
        s += al(npix * 4);
        CUDA_TRY(c, cudaMemcpyAsync(r, film->rgb, npix * 12, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(n, film->counts, npix * 4, cudaMemcpyHostToDevice, c->stream));
        d_rgb = r;
        d_counts = n;
        if (rgba) { d_out = (float4 *)s; s += al(npix * 16); }
        if (rgba8) { d_out8 = (uchar4 *)s; s += al(npix * 4); }
    } else if (((uintptr_t)rgba & 15u) || ((uintptr_t)rgba8 & 3u)) {
        return fail(c, LT_ERR_INVALID, "rgba must be 16-byte and rgba8 4-byte aligned");
    }
    CUDA_TRY(c, launch_resolve(d_rgb, d_counts, (uint32_t)npix, tonemap, exposure, d_out, d_out8, d_stats,
                               c->shape.sms, c->stream));
    if (host) {
        if (rgba) CUDA_TRY(c, cudaMemcpyAsync(rgba, d_out, npix * 16, cudaMemcpyDeviceToHost, c->stream));
        if (rgba8) CUDA_TRY(c, cudaMemcpyAsync(rgba8, d_out8, npix * 4, cudaMemcpyDeviceToHost, c->stream));
    }
    if (spp || host) {
        SppStats h{};
        CUDA_TRY(c, cudaMemcpyAsync(c->counters_host, d_stats, sizeof h, cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        memcpy(&h, c->counters_host, sizeof h);
        if (spp) {
            spp->min_spp = h.min_spp;
            spp->max_spp = h.max_spp;
            spp->sum_spp = h.sum_spp;
        }
    }
    return LT_OK;
} LT_CATCH(c)

// ------------------------------------------------------------------ batched differentiable rendering
// Jobs of a batched adjoint with at least this many samples fill the GPU by
// themselves: they run one after the other on the single-scene wavefront
// (whose trace stage sums the connection terms in shared memory), the others
// together on one wavefront. On the 32 adjoints of the 64-scene workload:
// everything on one wavefront 219 ms, one by one 204 ms, this split 186 ms
// (2^26: 192 ms). The batched differentiable forward sends the jobs that fill
// the wavefront by themselves (the tuning's paths in flight) to the
// single-scene wavefront the same way (its 32 forwards: 166.6 ms all together,
// 158.6 ms with the two of 2^26 samples alone).
constexpr unsigned long long kAdjointAloneSamples = 1ull << 24;

// A job's parameters with the detached copies defaulted to the parameters.
static DiffParams job_params(const lt_diff_job &j) {
    DiffParams P;
    P.albedo = j.dp.albedo;
    P.emission = j.dp.emission;
    P.sigma_a = j.dp.sigma_a;
    P.sigma_s = j.dp.sigma_s;
    P.albedo_s = j.dp.albedo_detached ? j.dp.albedo_detached : j.dp.albedo;
    P.sigma_a_s = j.dp.sigma_a_detached ? j.dp.sigma_a_detached : j.dp.sigma_a;
    P.sigma_s_s = j.dp.sigma_s_detached ? j.dp.sigma_s_detached : j.dp.sigma_s;
    return P;
}

// Batched differentiable forward (adjoint false) or adjoint over one scene
// table. The forward runs the differentiable wavefront over the work items of
// all jobs (as lt_render_batch does for plain renders) and returns when it
// has finished. The adjoint runs on the wavefront when every job that has
// samples to replay brings the forward's per-sample radiance (jobs of
// kAdjointAloneSamples or more one by one, the rest together; it returns when
// finished); otherwise it is one persistent launch over sample chunks of all
// jobs' pixels and returns once queued.
static lt_status diff_batch(lt_ctx *c, const lt_diff_job *jobs, uint32_t n, bool adjoint) {
    NvtxRange nvtx_("diff_batch");
    if (!c || (n && !jobs)) return fail(c, LT_ERR_INVALID, "NULL argument");
    if (n > LT_MAX_BATCH) return fail(c, LT_ERR_INVALID, "%u jobs; a batch holds at most %u", n, LT_MAX_BATCH);
    CUDA_TRY(c, cudaSetDevice(c->device));
    bool wave = !adjoint;  // the wavefront (forward, or adjoint replaying the forward's samples)
    if (adjoint) {
        wave = true;
        for (uint32_t i = 0; i < n; ++i) {
            const lt_ctx *s = jobs[i].scene;
            if (!s || !s->has_scene) continue;  // rejected below
            const unsigned long long total =
                (unsigned long long)s->host.camera.width * s->host.camera.height * jobs[i].params.spp;
            if (total && jobs[i].params.max_depth && !jobs[i].sample_radiance) wave = false;
        }
    }
    lt_status st = ensure_table(c);
    if (st != LT_OK) return st;
    SceneTable &T = *c->table_host;
    uint32_t count = 0, max_depth = 0, launches = 0;
    unsigned long long pixels = 0, samples = 0, items = 0, internal = 0;
    c->stats = lt_render_stats{};
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    std::vector<size_t> internal_at;  // per slot: offset into the internal sample buffer, or SIZE_MAX
    struct Alone {
        uint32_t job;
        size_t internal;  // forward without sample_radiance: offset into the internal sample buffer
    };
    std::vector<Alone> alone;  // jobs run one by one on the single-scene wavefront
    const unsigned long long alone_from =
        adjoint ? kAdjointAloneSamples : (c->tuning.paths_in_flight ? c->tuning.paths_in_flight : kDefaultPaths);
    for (uint32_t i = 0; i < n; ++i) {
        const lt_diff_job &j = jobs[i];
        const lt_ctx *s = j.scene;
        if (!s || !s->has_scene) return fail(c, LT_ERR_STATE, "job %u: no scene", i);
        if (s->device != c->device) return fail(c, LT_ERR_INVALID, "job %u is on another device", i);
        const HostScene &h = s->host;
        const uint32_t W = h.camera.width, H = h.camera.height;
        const bool media = !h.media.empty();
        if (!j.dp.albedo || !j.dp.emission || (media && (!j.dp.sigma_a || !j.dp.sigma_s)))
            return fail(c, LT_ERR_INVALID, "job %u: differentiable parameters missing", i);
        if (!adjoint && (!j.film.on_device || j.film.width != W || j.film.height != H || !j.film.rgb ||
                         !j.film.bounces || !j.film.counts))
            return fail(c, LT_ERR_INVALID, "job %u: needs a device film of %ux%u", i, W, H);
        if (adjoint && (!j.d_loss_d_film || !j.grad_albedo || !j.grad_emission ||
                        (media && (!j.grad_sigma_a || !j.grad_sigma_s))))
            return fail(c, LT_ERR_INVALID, "job %u: adjoint inputs or gradient arrays missing", i);
        const unsigned long long total = (unsigned long long)W * H * j.params.spp;
        if (total == 0) continue;
        samples += total;
        if (j.params.max_depth == 0) {  // no bounce: every sample's radiance is 0, gradients are 0
            if (!adjoint) {
                if (j.sample_radiance) CUDA_TRY(c, cudaMemsetAsync(j.sample_radiance, 0, total * 12, c->stream));
                CUDA_TRY(c, launch_add_counts(FilmPtrs{j.film.rgb, j.film.bounces, j.film.counts}, W * H,
                                              j.params.spp, c->stream));
                ++launches;
            }
            continue;
        }
        if (wave && total >= alone_from) {
            alone.push_back(Alone{i, SIZE_MAX});
            if (!adjoint && !j.sample_radiance) {
                alone.back().internal = (size_t)internal;
                internal += (total * 12 + 255) & ~255ull;
            }
            continue;
        }
        SceneSlot &sl = T.slots[count];
        DiffSlot &d = T.diff[count];
        sl.s = s->dev;
        sl.a = RenderArgs{W, H, j.params.first_frame, j.params.max_depth, j.params.rr_depth, total};
        sl.f = FilmPtrs{j.film.rgb, j.film.bounces, j.film.counts};
        d.p = job_params(j);
        d.g = DiffGrads{j.d_loss_d_film, j.grad_albedo, j.grad_emission, j.grad_sigma_a, j.grad_sigma_s,
                        0, 0, W, H, adjoint ? j.sample_radiance : nullptr};
        d.sample_I = adjoint ? nullptr : j.sample_radiance;
        d.num_media = (uint32_t)h.media.size();
        internal_at.push_back(SIZE_MAX);
        if (!adjoint && !j.sample_radiance) {  // the forward needs every sample's radiance
            internal_at.back() = (size_t)internal;
            internal += (total * 12 + 255) & ~255ull;
        }
        T.begin[count] = items;
        T.pbegin[count] = pixels;
        T.ibegin[count] = items;
        pixels += (unsigned long long)W * H;
        // work items: the samples on the wavefront; else chunks of kAdjointChunkSamples samples
        const unsigned long long chunks = (j.params.spp + kAdjointChunkSamples - 1) / kAdjointChunkSamples;
        items += wave ? total : (unsigned long long)W * H * chunks;
        if (j.params.max_depth > max_depth) max_depth = j.params.max_depth;
        ++count;
    }
    c->stats.samples = samples;
    if (internal) {
        if ((st = ensure_diff_samples(c, (size_t)internal)) != LT_OK) return st;
        for (uint32_t k = 0; k < count; ++k)
            if (internal_at[k] != SIZE_MAX) T.diff[k].sample_I = (float *)((char *)c->diff_samples + internal_at[k]);
    }
    if (count) {
        T.count = count;
        T.pad = 0;
        T.total = wave ? items : 0;
        T.total_items = items;
        T.total_pixels = pixels;
        T.fetch = 0;
        uint32_t cap = 0;
        Wavefront w;
        DiffWave dw;
        if (wave && (st = prepare_dwave(c, items, &cap, &w, &dw)) != LT_OK) return st;
        T.iteration_limit = wave ? drain_limit(items, cap, max_depth) : 0;
        CUDA_TRY(c, cudaMemcpyAsync(c->table_dev, c->table_host, offsetof(SceneTable, slots),
                                    cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(c->table_dev->slots, T.slots, count * sizeof(SceneSlot), cudaMemcpyHostToDevice,
                                    c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(c->table_dev->diff, T.diff, count * sizeof(DiffSlot), cudaMemcpyHostToDevice,
                                    c->stream));
        if (!wave) {
            CUDA_TRY(c, launch_diff_adjoint_batch(c->table_dev, c->shape, c->stream));
            ++launches;
        } else {
            RenderArgs all{};
            all.max_depth = max_depth;
            all.total = items;
            const SceneTable *t = c->table_dev;
            if (adjoint)
                st = run_loop(
                    c, w, all, c->stage_timing, kStages + 1u,
                    [&]() { return launch_awave_batch_init(t, dw, w, c->batch_shape, c->stream); },
                    [&](int stage, int cur) {
                        return launch_awave_batch_stage(stage, t, dw, w, cur, c->batch_shape, c->stream);
                    });
            else
                st = run_loop(
                    c, w, all, c->stage_timing, kStages + 1u,
                    [&]() { return launch_dwave_batch_init(t, dw, w, c->batch_shape, c->stream); },
                    [&](int stage, int cur) {
                        return launch_dwave_batch_stage(stage, t, dw, w, cur, c->batch_shape, c->stream);
                    });
            if (st != LT_OK) return st;
            launches += c->stats.kernel_launches;
            if (!adjoint) {
                CUDA_TRY(c, launch_diff_film_batch(t, pixels, c->shape.sms, c->stream));
                ++launches;
            }
        }
        CUDA_TRY(c, (cudaError_t)c->order.table_read_queued(c->rt, c->stream));
    }
    lt_render_stats acc = c->stats;
    for (const Alone &al : alone) {
        const lt_diff_job &j = jobs[al.job];
        const HostScene &h = j.scene->host;
        const uint32_t W = h.camera.width, H = h.camera.height;
        const RenderArgs a{W, H, j.params.first_frame, j.params.max_depth, j.params.rr_depth,
                           (unsigned long long)W * H * j.params.spp};
        const DiffParams P = job_params(j);
        if (adjoint) {
            const DiffGrads G{j.d_loss_d_film, j.grad_albedo, j.grad_emission, j.grad_sigma_a, j.grad_sigma_s,
                              0, 0, W, H, j.sample_radiance};
            if ((st = adjoint_wave(c, j.scene->dev, P, a, G)) != LT_OK) return st;
        } else {
            float *smp = al.internal == SIZE_MAX ? j.sample_radiance : (float *)((char *)c->diff_samples + al.internal);
            const FilmPtrs f{j.film.rgb, j.film.bounces, j.film.counts};
            if ((st = diff_wave(c, j.scene->dev, P, a, f, smp)) != LT_OK) return st;
        }
        launches += c->stats.kernel_launches;
        acc.iterations += c->stats.iterations;
        acc.main_rays += c->stats.main_rays;
        acc.light_rays += c->stats.light_rays;
        acc.bsdf_rays += c->stats.bsdf_rays;
        acc.light_traversals += c->stats.light_traversals;
        acc.nonfinite_samples += c->stats.nonfinite_samples;
        acc.trace_ms += c->stats.trace_ms;
        acc.shade_ms += c->stats.shade_ms;
        acc.init_ms += c->stats.init_ms;
    }
    c->stats = acc;
    c->stats.kernel_launches = launches;
    c->stats.samples = samples;
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    return LT_OK;
}

extern "C" lt_status lt_render_diff_batch(lt_ctx *c, const lt_diff_job *jobs, uint32_t n) try {
    return diff_batch(c, jobs, n, false);
} LT_CATCH(c)

extern "C" lt_status lt_render_adjoint_batch(lt_ctx *c, const lt_diff_job *jobs, uint32_t n) try {
    return diff_batch(c, jobs, n, true);
} LT_CATCH(c)

// ------------------------------------------------------------------ lt_image_load
extern "C" lt_status lt_image_load(const char *path, uint8_t *texels, size_t capacity, uint32_t *width,
                                   uint32_t *height, uint32_t *channels) try {
    if (!path || !width || !height || !channels) return fail(nullptr, LT_ERR_INVALID, "NULL argument");
    std::vector<uint8_t> data;
    std::string err;
    lt_status st = load_png(path, &data, width, height, channels, &err);
    if (st != LT_OK) return fail(nullptr, st, "%s", err.c_str());
    if (texels) {
        if (capacity < data.size())
            return fail(nullptr, LT_ERR_INVALID, "%s: needs %zu bytes, buffer holds %zu", path, data.size(), capacity);
        memcpy(texels, data.data(), data.size());
    }
    return LT_OK;
} LT_CATCH(nullptr)

extern "C" void lt_debug_fail_allocations(uint32_t after) { g_alloc_left.store(after); }

extern "C" void lt_debug_set_iteration_limit(uint64_t limit) { g_iteration_limit.store(limit); }

extern "C" void lt_debug_set_check_pixel_limit(uint32_t pixels) { g_check_pixels.store(pixels); }
