// lt_device.h -- device-side scene and wavefront state shared by the kernels
// (lt_kernels.cu) and the host driver (lt_api.cpp).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lt_math.h"
#include "lt_scene.h"

namespace lt {

// Scene as the kernels see it; passed by value (lives in the constant bank).
struct DevScene {
    const float4 *nodes;        // BvhNode, 4 float4 each
    const float4 *tris;         // leaf order, 3 float4 each: (v0, prim bits) (e1, 0) (e2, 0)
    const uint32_t *tri_geom;   // per global triangle
    const uint32_t *tri_vidx;   // 3 per global triangle
    const float *vnormal;       // 3 per vertex
    const float *vtex;          // 2 per vertex
    const uint8_t *texels;      // image textures
    const ImageInfo *images;
    const GeomInfo *geoms;
    const MaterialInfo *mats;
    const MediumInfo *meds;
    const LightInfo *lights;
    const float4 *light_tris;   // emissive meshes' triangles, 3 float4 each
    const float4 *nodes8;       // compressed 8-wide BVH (Bvh8Node, 5 float4 each), or null
    const float4 *tris8;        // triangles in 8-wide leaf order, 3 float4 each
    const float4 *nodes4;       // 4-wide BVH (Bvh4Node, 8 float4 each; leaves index `tris`), or null
    uint32_t num_nodes4;
    uint32_t num_lights;
    uint32_t num_tris;
    uint32_t num_nodes8;
    uint32_t num_nodes;         // BVH2 nodes
    uint32_t num_geoms, num_mats, num_media;
    v3 background;
    Camera cam;
    TentFilter filter;
};

// Path state, structure of arrays over `capacity` entries. It is kept in
// queue order: shade reads entry q of the current buffer and writes the
// surviving path to its compacted position in the other one, so every access
// is coalesced.
struct PathState {
    uint64_t *rng;     // PCG32 state (increment = frame | 1)
    uint32_t *pixel;
    uint32_t *frame;
    float *T;          // throughput, 3 planes of capacity
    uint32_t *bounces;
    uint32_t *flags;   // bits 0-7 sampled lobe, bits 8-23 medium index + 1
    float *iori;
};

// Kinds of the device-side bound checks of an LT_CHECKS build (recorded in
// WaveCounters::check) and the names the host reports them by.
enum CheckKind : uint32_t {
    kChkSlot = 1,  // path queue slot
    kChkRecord,    // connection record
    kChkOutSlot,   // output queue slot
    kChkNode,      // BVH node
    kChkLeaf,      // leaf triangle range
    kChkStack,     // traversal stack
    kChkPrim,      // hit primitive
    kChkScene,     // scene slot of a batch
    kChkLight,
    kChkMedium,
    kChkPixel,     // film pixel
    kChkGeom,      // mesh of a triangle
    kChkMaterial,
    kChkKinds
};
inline const char *check_name(uint32_t kind) {
    static const char *const names[kChkKinds] = {"none", "path queue slot", "connection record", "output queue slot",
                                                 "BVH node", "leaf triangles", "traversal stack", "hit primitive",
                                                 "scene slot", "light", "medium", "film pixel", "mesh", "material"};
    return kind < kChkKinds ? names[kind] : "unknown";
}

struct WaveCounters {
    uint32_t count[2];           // path-ray queue lengths (ping-pong by iteration parity): continuing paths
    uint32_t rcount[2];          // and regenerated paths (camera rays), kept apart at the top of the queue
    uint32_t ccount[2];          // connection records written by k_shade(parity)
    unsigned long long work_next; // next (pixel, frame) work item
    unsigned long long main_rays, light_rays, bsdf_rays;
    uint32_t trace_fetch;         // k_trace's persistent-thread counter, zeroed by the launch before
    uint32_t error;               // nonzero: a device-side bound was exceeded
    unsigned long long light_traversals;  // connection rays that needed an occlusion query
    unsigned long long iterations;        // wavefront iterations of a captured loop
    unsigned long long nonfinite;         // film contributions with a NaN or infinite channel
    uint32_t fcount[2];                   // differentiable forward: finishing entries by parity
    uint32_t check;                       // builds with LT_CHECKS: code of the first failed bound check
    uint32_t check_value;                 // and the index it rejected
    uint32_t trace_launches;              // k_trace launches of this loop (the queue trace's next row)
};

struct Wavefront {
    uint32_t capacity = 0;
    PathState p[2] = {};                    // ping-pong, in queue order
    float4 *ray[2] = {nullptr, nullptr};    // 2 float4 per entry: (org, tnear) (dir, tfar)
    float4 *hits = nullptr;                 // (t, u, v, prim bits)
    float4 *cray = nullptr;                 // 2 float4 per record: (org, kind|light) (dir, light distance)
    float4 *crec = nullptr;                 // 2 float4 per record: (f, bsdf pdf) (throughput, pixel)
    WaveCounters *counters = nullptr;
    uint32_t check_pixels = 0;              // builds with LT_CHECKS: film pixels the checks accept (0: all)
    uint3 *qtrace = nullptr;                // queue lengths per iteration (lt_set_queue_trace), or null
    uint32_t qtrace_cap = 0;                // rows of qtrace
    void *arena = nullptr;
    size_t arena_bytes = 0;
};

// The differentiable estimator on the wavefront (lt_render_diff, and the
// adjoint of lt_render_adjoint): what a path carries beyond PathState
// (ping-pong in queue order like it), the result of every connection record,
// the paths that finished while their last records were still to be traced,
// and the per-sample radiance. The adjoint also keeps, per path, the triangle
// whose albedo term waits for the records of its bounce (pend), per record the
// triangle it was sampled on and the factor f / albedo of the sample (aux),
// and, in its batched form, the two gradient terms that the trace stage
// computes for the next shade to add (gres).
constexpr uint32_t kNoRecord = 0xFFFFFFFFu;
struct DiffWave {
    float *C[2];         // radiance gathered so far, 3 planes of capacity
    float *Ts[2];        // throughput with the detached parameters (roulette), 3 planes
    uint2 *rec[2];       // the path's light and BSDF records of the previous shade, or kNoRecord
    float4 *res;         // per connection record: its contribution (rgb), w = 1 when it contributes
    uint4 *fin_id[2];    // finishing paths (by parity): (pixel, frame, scene slot, pending triangle)
    float4 *fin_C[2];    //   radiance gathered before their last records
    uint2 *fin_rec[2];   //   those records
    uint32_t *pend[2];   // adjoint: triangle of the previous bounce's deferred albedo term, or kMiss
    float2 *aux;         // adjoint, per connection record: (shading triangle, f / albedo of its sample)
    float4 *gres;        // batched adjoint, 2 per record: (albedo term, light triangle hit), (emission term, 0)
    float *sample_I;     // 3 floats per sample at ((frame - first_frame) * W * H + pixel)
    size_t bytes = 0;
};

struct FilmPtrs {
    float *rgb;
    uint32_t *bounces;
    uint32_t *counts;
};

struct RenderArgs {
    uint32_t width, height;
    uint32_t first_frame;
    uint32_t max_depth, rr_depth;
    unsigned long long total;  // width * height * spp
};

// Grid and block sizes of the stage kernels. The threads per block are chosen
// (64, 128 or 256; the autotuner may change them); the block counts follow from
// the occupancy of the kernel at that size (persistent grids: one full wave).
struct LaunchShape {
    int sms = 0;
    int bvh_width = 2;  // 2: BVH2 traversal; 4: 4-wide; 8: compressed 8-wide
    int trace_threads = 128, shade_threads = 128;
    int trace_blocks = 0, shade_blocks = 0, isect_blocks = 0;
    int diff_blocks = 0;
    int dtrace_blocks = 0, dshade_blocks = 0;  // differentiable forward on the wavefront
    int dtrace_batch_blocks = 0, dshade_batch_blocks = 0;
    int diff_adj_batch_blocks = 0;
    int atrace_blocks = 0, ashade_blocks = 0;  // adjoint on the wavefront
    int atrace_batch_blocks = 0, ashade_batch_blocks = 0;
    // plain renders with the BVH2: iterations of at most coop_limit rays are
    // traced by k_trace_tail (one warp per ray) on tail_blocks blocks
    int tail_blocks = 0;
    uint32_t coop_limit = 0;
    // the same kernel for the differentiable forward and the adjoint (always BVH2)
    int dtail_blocks = 0, dtail_batch_blocks = 0, atail_blocks = 0, atail_batch_blocks = 0;
};
// Kernel launches per wavefront iteration of a plain render with this shape
// (the differentiable ones always launch three: trace, small-iteration trace, shade).
inline uint32_t launches_per_iteration(const LaunchShape &ls) { return ls.coop_limit ? 3u : 2u; }

// Parameters of the differentiable render (device arrays): per-triangle RGB
// albedo and emission, per-medium RGB sigma_a / sigma_s, and the detached
// copies that drive sampling (roulette throughput, medium distances).
struct DiffParams {
    const float *albedo, *emission, *sigma_a, *sigma_s;
    const float *albedo_s, *sigma_a_s, *sigma_s_s;
};

// Adjoint inputs/outputs: d loss / d film colour sum per pixel (W*H*3), the
// gradient arrays (accumulated), and the pixel rectangle [x0, x1) x [y0, y1).
struct DiffGrads {
    const float *dI;
    float *albedo, *emission, *sigma_a, *sigma_s;
    uint32_t x0, y0, x1, y1;
    const float *sample_I;  // per-sample radiance from the forward pass, or null (replay twice)
};

// Samples per work item of the adjoint (a pixel's samples in chunks).
constexpr uint32_t kAdjointChunkSamples = 8;

// Limits of the bit fields that carry a scene slot, a light and a medium index
// in the path flags and connection records.
constexpr uint32_t kMaxBatchScenes = 2048;
constexpr uint32_t kMaxLights = 1u << 20;
constexpr uint32_t kMaxMedia = 8190;

// One scene of a batched render.
struct SceneSlot {
    DevScene s;
    RenderArgs a;
    FilmPtrs f;
};

// The scenes of a batch as the kernels read them (device memory, rewritten
// before each batched render). The work items of all scenes form one
// sequence: slot i owns [begin[i], begin[i] + slots[i].a.total).
// Differentiable parameters and outputs of one slot of a batched
// differentiable render (whole film: the crop is the full image).
struct DiffSlot {
    DiffParams p;
    DiffGrads g;
    float *sample_I;  // forward: per-sample radiance out, or null
    uint32_t num_media;
};

struct SceneTable {
    uint32_t count;
    uint32_t pad;
    unsigned long long total;            // work items of all slots (wavefront)
    unsigned long long iteration_limit;  // a captured loop stops here (counters->error = 2)
    unsigned long long total_pixels;     // pixels of all slots (differentiable kernels)
    unsigned long long fetch;            // pixel counter of the differentiable kernels, 0 on upload
    unsigned long long total_items;      // batched adjoint: sample chunks of all slots
    unsigned long long begin[kMaxBatchScenes];
    unsigned long long pbegin[kMaxBatchScenes];
    unsigned long long ibegin[kMaxBatchScenes];  // batched adjoint: first sample chunk of each slot
    SceneSlot slots[kMaxBatchScenes];
    DiffSlot diff[kMaxBatchScenes];
};

// Sample-count range of a film (lt_resolve), reduced on the device.
struct SppStats {
    uint32_t min_spp, max_spp;
    unsigned long long sum_spp;
};

// launcher (lt_resolve.cu): tonemap 0 = clamp, 1 = filmic; out / out8 / stats may be null
cudaError_t launch_resolve(const float *rgb, const uint32_t *counts, uint32_t npix, int tonemap, float exposure,
                           float4 *out, uchar4 *out8, SppStats *stats, int sms, cudaStream_t st);

// launchers (lt_kernels.cu)
// Loads the single-scene wavefront kernels (camera rays, trace, shade, counts)
// onto the current device, so that their first launch loads no code.
cudaError_t preload_wave_kernels();
// Fills the block counts of *out for its thread counts; `batch` selects the
// ManyScenes instantiations of the stage kernels.
void query_launch_shape(int device, bool batch, LaunchShape *out);
cudaError_t launch_intersect(const DevScene &s, const float4 *rays, float4 *hits, unsigned long long n,
                             uint32_t *fetch, const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_add_counts(const FilmPtrs &f, uint32_t npix, uint32_t spp, cudaStream_t st);
// differentiable forward on the wavefront: camera rays (with the path extras
// of d), then per iteration k_trace (connection records resolved into d.res)
// and k_dshade; last, the film from the per-sample radiance, per pixel in
// sample order (the film does not depend on the order in which samples finished)
cudaError_t launch_dwave_init(const DevScene &s, const DiffParams &p, const DiffWave &d, const Wavefront &w,
                              const RenderArgs &a, const FilmPtrs &f, const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_dwave_stage(int stage, const DevScene &s, const DiffParams &p, const DiffWave &d,
                               const Wavefront &w, const RenderArgs &a, const FilmPtrs &f, int cur,
                               const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_diff_film(const float *sample_I, const RenderArgs &a, const FilmPtrs &f, cudaStream_t st);
// the same for the scenes of a batch's table (lt_render_diff_batch): work items
// begin[], per-slot sample radiance and films in t->diff / t->slots
cudaError_t launch_dwave_batch_init(const SceneTable *t, const DiffWave &d, const Wavefront &w, const LaunchShape &ls,
                                    cudaStream_t st);
cudaError_t launch_dwave_batch_stage(int stage, const SceneTable *t, const DiffWave &d, const Wavefront &w, int cur,
                                     const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_diff_film_batch(const SceneTable *t, unsigned long long total_pixels, int sms, cudaStream_t st);
cudaError_t launch_diff_adjoint(const DevScene &s, const DiffParams &p, const RenderArgs &a, const DiffGrads &g,
                                uint32_t num_media, unsigned long long *fetch, const LaunchShape &ls,
                                cudaStream_t st);
// adjoint on the wavefront (lt_render_adjoint with the forward's per-sample
// radiance g.sample_I): the differentiable forward's paths replayed over the
// crop's samples (a.total = spp * crop pixels), gradient terms added per block
// in shared memory; leaves the film alone
cudaError_t launch_awave_init(const DevScene &s, const DiffParams &p, const DiffWave &d, const DiffGrads &g,
                              const Wavefront &w, const RenderArgs &a, const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_awave_stage(int stage, const DevScene &s, const DiffParams &p, const DiffWave &d,
                               const DiffGrads &g, const Wavefront &w, const RenderArgs &a, int cur,
                               const LaunchShape &ls, cudaStream_t st);
// the same over the jobs of a batch's table (lt_render_adjoint_batch, every
// job with its per-sample radiance): work items begin[] as the forward's
cudaError_t launch_awave_batch_init(const SceneTable *t, const DiffWave &d, const Wavefront &w, const LaunchShape &ls,
                                    cudaStream_t st);
cudaError_t launch_awave_batch_stage(int stage, const SceneTable *t, const DiffWave &d, const Wavefront &w, int cur,
                                     const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_wave_init(const DevScene &s, const Wavefront &w, const RenderArgs &a, const FilmPtrs &f,
                             const LaunchShape &ls, cudaStream_t st);
// Per wavefront iteration: k_trace (path rays of this iteration + connection
// rays of the previous shade), then k_shade.
enum WaveStage { kStageTrace = 0, kStageShade = 1 };
constexpr int kStages = 2;
cudaError_t launch_wave_stage(int stage, const DevScene &s, const Wavefront &w, const RenderArgs &a,
                              const FilmPtrs &f, int cur, const LaunchShape &ls, cudaStream_t st);
// batched render over a scene table (lt_render_batch)
cudaError_t launch_batch_init(const SceneTable *t, const Wavefront &w, const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_batch_stage(int stage, const SceneTable *t, const Wavefront &w, int cur, const LaunchShape &ls,
                               cudaStream_t st);
// Condition kernel of a captured loop: counters->iterations += iters; the
// while node `h` continues while path queue `cur` or the connection records
// of parity cur ^ 1 are not empty and the iteration limit of `t` is not reached.
// batched adjoint over the sample chunks of t's slots (ibegin, total_items) and their diff entries
cudaError_t launch_diff_adjoint_batch(SceneTable *t, const LaunchShape &ls, cudaStream_t st);
cudaError_t launch_loop_condition(const Wavefront &w, const SceneTable *t, cudaGraphConditionalHandle h, int cur,
                                  uint32_t iters, cudaStream_t st);

}  // namespace lt
