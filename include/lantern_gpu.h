/*
 * lantern_gpu.h -- C ABI of the GB300 path-tracing library (liblantern_gpu.so).
 *
 * The library renders Lantern scenes on one GPU with hand-written sm_103a CUDA:
 * a wavefront integrator (camera rays, closest-hit traversal, shading with
 * next-event estimation and MIS, light connection, Russian roulette, film
 * accumulation) over the library's own BVH. It replaces, at the same contract:
 *
 *   - Integrator::RenderFrame            source/core/integrator/integrator.{h:24-51,cpp:28-43}
 *   - Scene::LoadSceneFromJSON           source/core/scene/scene.{h:71,cpp:82-91,154-582}
 *   - rtcCommitScene / rtcIntersect1     (Embree, called at scene.cpp:86,116-121)
 *
 * Plain pointers and sizes only; no exceptions cross this boundary. Every call
 * returns an lt_status; lt_last_error() gives the message of the last failure
 * on that context. One host thread drives one context; all GPU work is issued
 * on the context's stream. lt_render returns when the render has finished
 * (it reads the wavefront's queue lengths to know when to stop, so its film
 * writes are complete, device or host film); lt_intersect returns once its
 * work is queued (device buffers) or finished (host buffers).
 */
#ifndef LANTERN_GPU_H
#define LANTERN_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: lt_render_stats gained init_ms and idle_ms; lt_light_info, lt_scene_lights_get,
 * lt_trim and lt_debug_set_iteration_limit were added.
 * 3: LT_ERR_CHECK, lt_debug_set_check_pixel_limit and the queue trace
 * (lt_set_queue_trace, lt_queue_trace_get) were added. */
#define LT_ABI_VERSION 3

typedef enum lt_status {
    LT_OK = 0,
    LT_ERR_INVALID = 1,     /* bad argument */
    LT_ERR_CUDA = 2,        /* CUDA runtime error */
    LT_ERR_OOM = 3,         /* device or host allocation failed */
    LT_ERR_TIMEOUT = 4,     /* a bounded device-side wait ran out */
    LT_ERR_IO = 5,          /* file missing or unreadable */
    LT_ERR_PARSE = 6,       /* malformed scene JSON or LMF */
    LT_ERR_UNSUPPORTED = 7, /* feature outside this build */
    LT_ERR_STATE = 8,       /* call out of order (e.g. render without a scene) */
    LT_ERR_CHECK = 9        /* a device-side bound check failed (liblantern_gpu_checked.so only) */
} lt_status;

typedef struct lt_ctx lt_ctx;

/* ---------------------------------------------------------------- context */
/* Creates a context on CUDA device `device` with its own stream. */
lt_status lt_ctx_create(int device, lt_ctx **out);
void lt_ctx_destroy(lt_ctx *ctx);
/* Message of the last failing call on ctx (or of the last failing
 * lt_ctx_create on this thread when ctx is NULL). Never NULL. */
const char *lt_last_error(const lt_ctx *ctx);
/* Issue all further work on `stream` (a cudaStream_t; NULL is CUDA's legacy
 * default stream). A new context uses a non-blocking stream of its own, which
 * lt_get_stream returns before any lt_set_stream call. Work the context queued
 * on its previous stream comes first: the new stream waits for it on the
 * device (an event), the host does not block. */
lt_status lt_set_stream(lt_ctx *ctx, void *stream);
void *lt_get_stream(const lt_ctx *ctx);
/* Waits for all work queued on the context's stream. */
lt_status lt_sync(lt_ctx *ctx);
/* Frees the context's work buffers -- the wavefront arenas (up to
 * paths_in_flight x 464 bytes), the per-sample radiance buffer of the
 * differentiable forward and the staging buffer of host-memory calls -- and
 * keeps its scene; the next call that needs them allocates them again. For
 * applications that keep many contexts alive (one per scene): an idle context
 * otherwise holds its buffers until it is destroyed. Waits for the context's
 * work first. No counterpart in the reference, whose integrator allocates
 * nothing per render. */
lt_status lt_trim(lt_ctx *ctx);
int lt_abi_version(void);

/* ---------------------------------------------------------------- scene */
/* BSDFs of source/core/materials/bsdfs: LambertBSDF, MirrorBSDF,
 * IdealSpecularDielectric. Albedo is a constant texture. */
enum { LT_BSDF_LAMBERT = 0, LT_BSDF_MIRROR = 1, LT_BSDF_DIELECTRIC = 2 };
/* Media of source/core/materials/media (NonScattering, IsotropicScattering),
 * plus LT_MEDIUM_HG: RGB sigma_s and a Henyey-Greenstein phase (extension). */
enum { LT_MEDIUM_NON_SCATTERING = 1, LT_MEDIUM_ISOTROPIC = 2, LT_MEDIUM_HG = 3 };

/* Albedo textures (materials/textures): ConstantTexture, UVTexture (albedo =
 * (u, v, 0) of the hit's texture coordinate) and ImageTexture (nearest texel
 * at (round(u * width), round((1 - v) * height)), 8-bit value / 256). */
enum { LT_ALBEDO_CONSTANT = 0, LT_ALBEDO_UV = 1, LT_ALBEDO_IMAGE = 2 };

typedef struct lt_material_desc {
    int32_t bsdf;      /* LT_BSDF_* */
    float albedo[3];   /* LT_ALBEDO_CONSTANT */
    float ior;         /* dielectric only */
    int32_t medium;    /* index into lt_scene_desc.media, or -1 */
    int32_t albedo_kind;  /* LT_ALBEDO_*; 0 = constant */
    uint32_t image;       /* LT_ALBEDO_IMAGE: index into lt_scene_desc.images */
} lt_material_desc;

/* An image texture: 8-bit samples, rows from the top, `channels` (1-4) per
 * texel -- what stbi_load(path, &w, &h, &n, 0) returns (image_cache.cpp:23-31). */
typedef struct lt_image_desc {
    const uint8_t *texels;
    uint32_t width, height, channels;
} lt_image_desc;

typedef struct lt_medium_desc {
    int32_t type;      /* LT_MEDIUM_* */
    float sigma_a[3];  /* per unit length */
    float sigma_s[3];  /* isotropic: all three equal */
    float g;           /* HG anisotropy; 0 for the reference media */
} lt_medium_desc;

typedef struct lt_mesh_desc {
    const float *positions;   /* num_vertices * 3, world space */
    const float *normals;     /* num_vertices * 3, or NULL */
    const uint32_t *indices;  /* num_triangles * 3 */
    uint32_t num_vertices;
    uint32_t num_triangles;
    int32_t material;         /* index into lt_scene_desc.materials */
    int32_t emissive;         /* nonzero: the mesh is an area light */
    float emission_color[3];  /* AreaLight: radiance = color * power / (pi * area) */
    float radiant_power;
    const float *texcoords;   /* num_vertices * 2, or NULL (the hit's texture coordinate is then (0, 0)) */
    const float *transform;   /* 16 floats, row-major: positions become transform * (p, 1) as the
                               * reference's AddLMF / AddMesh compute it (scene.cpp:456-461,517-522);
                               * normals are used as given (scene.cpp:481-482,560). NULL = identity */
} lt_mesh_desc;

typedef struct lt_camera_desc {
    float phi, theta, radius; /* spherical orbit about target (pinhole_camera.cpp:27-40) */
    float fov;                /* horizontal field of view, radians */
    float target[3];
    uint32_t width, height;
} lt_camera_desc;

typedef struct lt_scene_desc {
    lt_camera_desc camera;
    float background[3];
    const lt_material_desc *materials;
    uint32_t num_materials;
    const lt_medium_desc *media;
    uint32_t num_media;
    const lt_mesh_desc *meshes; /* geomID = position in this array */
    uint32_t num_meshes;
    const lt_image_desc *images;
    uint32_t num_images;
} lt_scene_desc;

/* Uploads the scene and builds its BVH; replaces any previous scene.
 * Replaces Scene::ParseJSON's AddMesh/AddLMF + rtcCommitScene
 * (scene.cpp:451-582, :86): the library computes each light's area, bounding
 * sphere and radiance the way AddLMF and AreaLight's constructor do (on the
 * device with the GPU builder: the vertex transform, triangle setup, light
 * setup and BVH build all run there). */
lt_status lt_scene_create(lt_ctx *ctx, const lt_scene_desc *desc);

/* Frees the context's scene (its device arrays, BVHs and captured batch loop)
 * and keeps the context; renders then fail with LT_ERR_STATE until a new
 * scene is created. Replaces the Scene destructor's frees (scene.cpp:584-606).
 * Waits for the context's stream first. */
lt_status lt_scene_destroy(lt_ctx *ctx);

/* Which builder lt_scene_create uses for the BVH (rtcCommitScene's job):
 * LT_BVH_GPU (default) -- binned SAH (32 bins, <= 4 triangles per leaf) built
 * level by level on the device; LT_BVH_HOST -- the same algorithm on the host
 * CPU. Both make the same splits. */
enum { LT_BVH_GPU = 0, LT_BVH_HOST = 1 };
lt_status lt_set_bvh_builder(lt_ctx *ctx, int32_t builder);

/* Scene::LoadSceneFromJSON (scene.h:71): reads a Lantern scene JSON and the
 * LMF files it names (triangle LMF with normals and texture coordinates,
 * transform, constant / uv / image albedo, media, emission), generates its
 * "grid" and "geosphere" primitives as CreateGrid / CreateGeosphere do
 * (geometry_generator.cpp:214-356,515-566; scene.cpp:408-426), decodes PNG
 * image textures (lt_image_load), then lt_scene_create. */
lt_status lt_scene_load_json(lt_ctx *ctx, const char *path);

/* Decodes a PNG file as the scene loader reads image textures, matching
 * stbi_load(path, &w, &h, &n, 0): 8-bit samples; grey 1, grey+alpha 2, RGB 3,
 * RGBA 4 channels (palette -> RGB or RGBA, a tRNS key adds alpha, 16-bit keeps
 * the high byte); not interlaced. Fills width/height/channels; copies the
 * texels (width*height*channels bytes) when `texels` is not NULL and
 * `capacity` is large enough. No context and no GPU: errors are read with
 * lt_last_error(NULL). */
lt_status lt_image_load(const char *path, uint8_t *texels, size_t capacity, uint32_t *width, uint32_t *height,
                        uint32_t *channels);

typedef struct lt_scene_info {
    uint32_t width, height;
    uint32_t num_triangles, num_meshes, num_lights;
    uint32_t num_bvh_nodes;
    uint64_t device_bytes;    /* scene + BVH bytes on the device */
    float build_ms;           /* BVH build time */
    uint32_t num_media;
} lt_scene_info;
lt_status lt_scene_info_get(lt_ctx *ctx, lt_scene_info *out);

/* The scene's area lights (Scene::GetLight / AreaLight, scene.h:74-79,
 * area_light.h:16-21): per emissive mesh, in mesh order, its mesh index
 * (geomID), triangle count, area (the sequential sum of scene.cpp:527-534),
 * bounding sphere (CalculateBoundingSphere, scene.cpp:49-80) and radiance
 * (color * radiant_power / (pi * area)). With the GPU builder the device
 * computes them from the transformed vertices, with the host builder the host
 * does; both give the same bits. `out` holds `capacity` entries (at least the
 * scene's num_lights). */
typedef struct lt_light_info {
    uint32_t mesh;
    uint32_t num_triangles;
    float area;
    float sphere[4];   /* centre x, y, z, radius */
    float radiance[3];
} lt_light_info;
lt_status lt_scene_lights_get(lt_ctx *ctx, lt_light_info *out, uint32_t capacity);

/* Per-mesh geometry offsets: first global triangle index of each mesh
 * (global triangle index = first[geomID] + primID). `first` holds num_meshes. */
lt_status lt_scene_mesh_offsets(lt_ctx *ctx, uint32_t *first, uint32_t capacity);

/* ---------------------------------------------------------------- film + render */
typedef struct lt_film {
    float *rgb;          /* width*height*3: colour sums (FrameBuffer::ColorData) */
    uint32_t *bounces;   /* width*height: summed path lengths (FrameBuffer::Bounces) */
    uint32_t *counts;    /* width*height: sample counts (FrameBuffer::ColorSampleCount) */
    uint32_t width, height;
    int32_t on_device;   /* 1: device pointers; 0: host memory (copied in and out) */
} lt_film;

typedef struct lt_render_params {
    uint32_t spp;          /* samples per pixel in this call (= RenderFrame calls) */
    uint32_t first_frame;  /* frame number of the first sample (Integrator::m_frameNumber) */
    uint32_t max_depth;    /* loop bound; the reference's constant is 1500 (integrator.cpp:114) */
    uint32_t rr_depth;     /* roulette when bounces > rr_depth; the reference's is 3 (:235) */
} lt_render_params;

/* Integrator::RenderFrame, spp times: adds one sample per pixel per frame to
 * the film (colour, path length, count), as integrator.cpp:245-249 does. The
 * sampler of sample (pixel, frame) is PCG32 seeded with MurmurHash3(pixel,
 * frame) and sequence frame -- the reference's per-tile seeding
 * (integrator.cpp:84-89) keyed by pixel instead of tile. */
lt_status lt_render(lt_ctx *ctx, const lt_render_params *params, lt_film *film);

/* lt_render without any device or host allocation. No counterpart in the
 * reference (its CPU integrator has nothing to allocate on a device).
 *
 * For callers that cannot have the library allocate GPU memory while they run:
 * an application that gives the library a fixed memory budget up front and
 * forbids allocations afterwards, or an interactive loop in which cudaMalloc /
 * cudaFree (which can synchronise the whole device) would stall other work.
 * The wavefront state lives in a fixed array inside liblantern_gpu.so of
 * LT_NOALLOC_MAX_PATHS path slots (about 18.9 MB), reserved on every GPU on
 * which a context is created, until the process exits. Same sampling, same film
 * semantics and same result as lt_render; only the number of paths in flight
 * is bounded.
 *
 * - film must be on the device (on_device = 1): host films need staging memory.
 * - paths_in_flight: path slots to use, 1..LT_NOALLOC_MAX_PATHS; anything else
 *   is rejected with LT_ERR_INVALID. More slots keep more of the GPU busy.
 * - Set-up happens in lt_ctx_create, with the device current: the array's
 *   module and the wavefront kernels are loaded and the array's device address
 *   is looked up (cudaGetSymbolAddress) and kept, so no call of
 *   lt_render_noalloc allocates or loads anything on the device.
 * - All calls in the process share the one array per device: calls whose GPU
 *   work overlaps (other threads, other contexts, other streams) race and
 *   corrupt each other. Serialise them. The array keeps the last call's
 *   contents; each call clears what it needs before use.
 * - No per-stage timing is recorded (lt_render_stats: trace_ms and shade_ms
 *   are 0; the ray, iteration and non-finite counts are filled as lt_render's). */
#define LT_NOALLOC_MAX_PATHS 65536
lt_status lt_render_noalloc(lt_ctx *ctx, const lt_render_params *params, lt_film *film,
                            uint32_t paths_in_flight);

typedef struct lt_render_stats {
    uint64_t main_rays;      /* closest-hit queries of path segments */
    uint64_t light_rays;     /* light-sample connection rays (AreaLight::SampleLi) */
    uint64_t bsdf_rays;      /* BSDF-sample MIS rays (AreaLight::PdfLi) */
    uint64_t samples;
    uint32_t iterations;     /* wavefront iterations */
    uint32_t kernel_launches;
    float gpu_ms;            /* device time of the last lt_render, first kernel to last */
    float trace_ms;          /* kernel time of the trace stage (path rays + connection rays);
                              * this and shade_ms, init_ms, idle_ms with stage timing only */
    float shade_ms;          /* ... of the shade stage (regenerated camera rays included) */
    uint64_t light_traversals; /* connection rays traced (the rest were resolved against the light alone) */
    uint64_t nonfinite_samples; /* film contributions with a NaN or infinite channel (e.g. a mesh
                                 * without normals shades with normalize(0), integrator.cpp:182) */
    float init_ms;           /* kernel time of the first camera rays */
    float idle_ms;           /* gpu_ms - init_ms - trace_ms - shade_ms: time between the render's
                              * kernels (the stream waiting for the host between batches of
                              * iterations, queue-length reads) */
} lt_render_stats;
lt_status lt_render_stats_get(lt_ctx *ctx, lt_render_stats *out);

/* Stage timing (on != 0): the wavefront renders of ctx (lt_render and the
 * differentiable calls) record an event before and after every kernel launch
 * and fill trace_ms, shade_ms, init_ms and idle_ms of lt_render_stats. Off by
 * default: the events cost the gaps between launches (a 256x256 render at
 * 16 spp 1.164 ms with them, 1.081 ms without; 1 spp 0.616 vs 0.533 ms). No
 * counterpart in the reference. */
lt_status lt_set_stage_timing(lt_ctx *ctx, int32_t on);

/* Queue trace: the wavefront's queue lengths at the start of every iteration,
 * as the trace kernel reads them (path rays that continue, paths that start
 * with a camera ray, connection records of the previous shade), recorded on
 * the device by that kernel. lt_set_queue_trace(ctx, rows) allocates room for
 * `rows` iterations (at most LT_QUEUE_TRACE_MAX_ROWS; 0, the initial state,
 * frees it and records nothing); call it outside a render, since it allocates.
 * lt_queue_trace_get copies up to `capacity` rows of the context's last
 * wavefront loop (an lt_render, one scene of a batch that renders alone, or a
 * batch's captured loop; lt_render_noalloc records none) into `out` (host
 * memory) and sets *rows to the number recorded. Summed over the rows,
 * path_rays + camera_rays is lt_render_stats.main_rays and
 * connection_records is light_traversals. No counterpart in the reference,
 * which has no queues; its per-pixel bounce counts are the film's Bounces. */
#define LT_QUEUE_TRACE_MAX_ROWS 65536u
typedef struct lt_queue_lengths {
    uint32_t path_rays;           /* continuing paths' rays (queue bottom) */
    uint32_t camera_rays;         /* paths started this iteration from a work item (queue top) */
    uint32_t connection_records;  /* light-sample and BSDF-MIS records of the previous shade */
} lt_queue_lengths;
lt_status lt_set_queue_trace(lt_ctx *ctx, uint32_t rows);
lt_status lt_queue_trace_get(lt_ctx *ctx, lt_queue_lengths *out, uint32_t capacity, uint32_t *rows);

/* ---------------------------------------------------------------- resolve */
/* The visualizer's final pass into a headless buffer (the window, swapchain and
 * GLSL pass are not part of this library). Per pixel, as
 * visualizer.cpp:352-364 and final_resolve_ps.glsl:24-43 compute it:
 *   c = exp2f(exposure_stops) * (ColorData / ColorSampleCount, 1)   (visualizer.cpp:1308)
 *   LT_TONEMAP_CLAMP:  c = clamp(c, 0, 1)
 *   LT_TONEMAP_FILMIC: x = max(0, c - 0.004); c = clamp(x(6.2x + 0.5) / (x(6.2x + 1.7) + 0.06), 0, 1); alpha = 1
 * rgba (4 floats per pixel) and rgba8 (4 bytes per pixel, round(c * 255) as
 * the swapchain's UNORM format stores it) may each be NULL; both are device
 * pointers when film->on_device, else host memory. spp (optional, host)
 * receives the minimum, maximum and sum of the sample counts. A pixel with no
 * samples divides by zero as the reference does. */
enum { LT_TONEMAP_CLAMP = 0, LT_TONEMAP_FILMIC = 1 };
typedef struct lt_spp_range { uint32_t min_spp, max_spp; uint64_t sum_spp; } lt_spp_range;
lt_status lt_resolve(lt_ctx *ctx, const lt_film *film, int32_t tonemap, float exposure_stops, float *rgba,
                     uint8_t *rgba8, lt_spp_range *spp);

/* ---------------------------------------------------------------- batching and tuning */
/* Extension with no counterpart in the reference, whose integrator renders one
 * scene per Integrator (integrator.cpp:28-43): the wavefront's launch
 * configuration, and many scenes rendered together in one captured loop. */
typedef struct lt_tuning {
    uint32_t paths_in_flight;  /* wavefront path slots of this context, 1024..67,108,864 (288 B
                                  each); 0 = min(samples, 16,777,216), halved while the
                                  allocation fails (down to 1,048,576) */
    uint32_t trace_threads;    /* threads per block of the trace kernel: 64, 128 or 256 */
    uint32_t shade_threads;    /* ... of the shade kernel: 64, 128, 256 or 512 (lt_render_batch's
                                  shade kernel uses at most 256) */
    uint32_t loop_iterations;  /* wavefront iterations per body of lt_render_batch's loop: 2, 4 or 8 */
    uint32_t bvh_width;        /* children per BVH node: 2 (BVH2), 4 (4-wide) or 8 (compressed 8-wide);
                                  the wide trees are built from the BVH2 on first use */
    float ms;                  /* lt_autotune_batch: device time of the chosen tuning on its sample */
} lt_tuning;
/* The context's tuning; it applies to lt_render, lt_render_batch and the
 * tuner's starting point. Zero fields of lt_set_tuning keep their defaults
 * (0 paths = automatic, 128 trace threads, 256 shade threads, 2 iterations,
 * width 2). Width 8 builds
 * the scene's compressed 8-wide BVH from its BVH2 (Ylitie, Karras, Laine, HPG
 * 2017 node layout), width 4 an uncompressed 4-wide one sharing the BVH2's
 * triangles; lt_scene_create then builds it for every new scene. */
lt_status lt_get_tuning(const lt_ctx *ctx, lt_tuning *out);
lt_status lt_set_tuning(lt_ctx *ctx, const lt_tuning *t);

/* Renders scenes[i] (contexts that hold a scene, all on ctx's device; ctx may
 * be one of them) with params[i] into films[i], as n lt_render calls would,
 * but together: the work items of all scenes form one sequence over one
 * wavefront owned by ctx, so that paths of every scene share each launch. The
 * iteration loop is captured once into a CUDA graph (a while node whose
 * condition kernel stops when no path is left) and the whole batch runs as one
 * graph launch on ctx's stream; the graph is kept and reused while the
 * wavefront and tuning stay the same. A scene whose samples fill the wavefront
 * by themselves (at least paths_in_flight of ctx's tuning, 16M by default)
 * gains nothing from the others' company: it is rendered after the loop with
 * the single-scene kernels on the same wavefront.
 * - films must be on the device (on_device = 1), of each camera's size, and
 *   must not overlap;
 * - n <= LT_MAX_BATCH; each scene may have at most 1,048,576 lights and 8,190 media;
 * - returns after the batch has finished (the film writes are complete);
 * - the scene contexts must not be in use by other threads during the call
 *   (with bvh_width 4 or 8 the call builds their wide BVHs on first use). */
#define LT_MAX_BATCH 2048
lt_status lt_render_batch(lt_ctx *ctx, lt_ctx *const *scenes, const lt_render_params *params, lt_film *films,
                          uint32_t n);

/* Autotuner: renders the batch (into scratch films, spp capped at spp_cap) under
 * candidate tunings -- BVH width 2 or 8, paths in flight, threads per block of each
 * stage, iterations per loop body -- by coordinate descent from ctx's tuning,
 * keeps the fastest in ctx and returns it in *best (may be NULL). Trying width
 * 8 builds the 8-wide BVH of every scene of the batch. */
lt_status lt_autotune_batch(lt_ctx *ctx, lt_ctx *const *scenes, const lt_render_params *params, uint32_t n,
                            uint32_t spp_cap, lt_tuning *best);

/* ---------------------------------------------------------------- differentiable rendering */
/* Extension with no counterpart in the reference: gradients of an image loss
 * with respect to per-triangle albedo, per-triangle emission and per-medium
 * sigma_a / sigma_s, by path replay (each sample is re-traced from its
 * (pixel, frame) seed; no path is stored).
 *
 * The differentiable estimator is the render loop with per-triangle albedo and
 * emission (emission counts on emissive meshes only), the RGB medium form
 * (distance sampled with the mean of the detached sigma_s; isotropic media
 * sample with the detached sigma_s[0]), and the roulette probability taken from
 * a throughput computed with the detached parameter copies. With the detached
 * copies equal to the parameters it traces the same paths as lt_render.
 * All arrays are device memory. */
typedef struct lt_diff_params {
    const float *albedo;            /* num_triangles * 3 */
    const float *emission;          /* num_triangles * 3 (radiance) */
    const float *sigma_a;           /* num_media * 3 */
    const float *sigma_s;           /* num_media * 3 */
    const float *albedo_detached;   /* sampling copies; NULL = the parameters themselves */
    const float *sigma_a_detached;
    const float *sigma_s_detached;
} lt_diff_params;

/* The scene's own values as parameters, into HOST arrays of num_triangles*3
 * (albedo, emission) and num_media*3 (sigma_a, sigma_s). */
lt_status lt_diff_defaults(lt_ctx *ctx, float *albedo, float *emission, float *sigma_a, float *sigma_s);

/* Forward render of the differentiable estimator into a device film
 * (additive, as lt_render), on the same wavefront as lt_render: every sample's
 * radiance is gathered in the estimator's order and the colour sums are added
 * per pixel in sample order, so the film is the same on every run (finite
 * differences see no summation-order noise). Returns when the render has
 * finished. sample_radiance (device, optional): receives every sample's
 * radiance, 3 floats at ((frame - first_frame) * W * H + pixel); with it the
 * adjoint replays each path once instead of twice (without it the library
 * keeps such a buffer of its own). */
lt_status lt_render_diff(lt_ctx *ctx, const lt_render_params *params, const lt_diff_params *dp, lt_film *film,
                         float *sample_radiance);

/* Adjoint: given d_loss_d_film (W*H*3, derivative of the loss with respect to
 * the film's colour sums) adds d loss / d parameter to the four gradient arrays
 * (same shapes as the parameters; not cleared). crop = {x0, y0, x1, y1} limits
 * the pixels whose samples are replayed, or NULL for the whole film.
 * sample_radiance: from lt_render_diff with the same parameters and render
 * params; with it the paths are replayed on the forward's wavefront (gradient
 * terms summed per block in shared memory; returns when finished), without it
 * (NULL) one thread replays each sample twice (returns once queued). Both
 * forms add the same terms; only the order of the float sums differs. */
lt_status lt_render_adjoint(lt_ctx *ctx, const lt_render_params *params, const lt_diff_params *dp,
                            const float *d_loss_d_film, float *grad_albedo, float *grad_emission,
                            float *grad_sigma_a, float *grad_sigma_s, const uint32_t *crop,
                            const float *sample_radiance);

/* Batched forms of lt_render_diff and lt_render_adjoint: each job names a
 * scene (a context holding one, on ctx's device), its render params and
 * differentiable parameters; all jobs run together on ctx's stream. Per job
 * the results are those of the single-scene call over the whole film (no crop).
 * - lt_render_diff_batch: the work items of all jobs share one wavefront owned
 *   by ctx (as lt_render_batch's; a job that fills the wavefront by itself, at
 *   least the tuning's paths in flight, runs alone on it after the others);
 *   film (device, additive) and sample_radiance (optional, as lt_render_diff's)
 *   are outputs, the same bits as the single-scene call gives. Returns when the
 *   batch has finished.
 * - lt_render_adjoint_batch: d_loss_d_film and sample_radiance are inputs,
 *   the four gradient arrays outputs (accumulated; sigma arrays may be NULL for
 *   scenes without media). When every job brings its sample_radiance, the
 *   samples of the jobs below 2^24 samples are replayed together on one
 *   wavefront owned by ctx, the larger jobs one by one on it, and the call
 *   returns when finished; otherwise it is one persistent launch over chunks of
 *   8 samples of all jobs' pixels (warps take 32 chunks at a time from a shared
 *   counter) that replays each sample twice, and the call returns once the work
 *   is queued. Jobs must not share gradient arrays.
 * n <= LT_MAX_BATCH. */
typedef struct lt_diff_job {
    lt_ctx *scene;
    lt_render_params params;
    lt_diff_params dp;
    lt_film film;
    float *sample_radiance;
    const float *d_loss_d_film;
    float *grad_albedo, *grad_emission, *grad_sigma_a, *grad_sigma_s;
} lt_diff_job;
lt_status lt_render_diff_batch(lt_ctx *ctx, const lt_diff_job *jobs, uint32_t n);
lt_status lt_render_adjoint_batch(lt_ctx *ctx, const lt_diff_job *jobs, uint32_t n);

/* ---------------------------------------------------------------- rays */
typedef struct lt_ray { float org[3]; float tnear; float dir[3]; float tfar; } lt_ray; /* 32 B */
typedef struct lt_hit { float t, u, v; uint32_t prim; } lt_hit; /* 16 B; prim = global
                                                               * triangle index, 0xFFFFFFFF = miss */

/* rtcIntersect1 (Embree, scene.cpp:116-121) for n rays: closest hit with
 * Embree's Moeller-Trumbore acceptance rule (tnear exclusive, tfar inclusive).
 * rays/hits are device pointers when on_device, else host memory. */
lt_status lt_intersect(lt_ctx *ctx, const lt_ray *rays, lt_hit *hits, uint64_t n, int32_t on_device);

/* ---------------------------------------------------------------- fault injection */
/* For failure-handling tests: after `after` more successful device or pinned
 * host allocations by the library, the next one fails as out-of-memory
 * (LT_ERR_OOM) without reaching the CUDA runtime. UINT32_MAX (the initial
 * state) turns injection off. Process-wide. No counterpart in the reference. */
void lt_debug_fail_allocations(uint32_t after);

/* For failure-handling tests: caps the wavefront iterations of every render
 * (lt_render, lt_render_noalloc, lt_render_batch) at `limit`. A render whose
 * wavefront has not drained by then stops and returns LT_ERR_TIMEOUT, the
 * status of the library's own bound (about 4 x (max_depth + 8) x the number of
 * wavefront refills); the film then holds part of the samples. 0 (the initial
 * state) = the library's own bound only. Process-wide. The reference has no
 * such bound (its loop constant is 1500 bounces, integrator.cpp:114) and
 * reports failures as bool + printf (scene.cpp:200-213). */
void lt_debug_set_iteration_limit(uint64_t limit);

/* Bound-checked build. liblantern_gpu_checked.so is this library with its
 * kernels compiled with -DLT_CHECKS=1: the wavefront's trace, small-iteration
 * trace and shade kernels (plain, batched and differentiable) and the BVH2 and
 * 4-wide traversals check every queue slot, connection record, BVH node, leaf
 * range, traversal stack entry, hit primitive, scene slot, light, medium, mesh,
 * material and film pixel index they form against its array before the access
 * (the 8-wide traversal bounds its indices in both builds). A failed check
 * records its kind and the index (the first failure of a render wins), skips
 * the access, and the render's later kernels return at once; the render call
 * then returns LT_ERR_CHECK, its message naming the check and the index. The
 * stand-in for compute-sanitizer, which this library's test machines cannot
 * run. In the plain library the checks compile to nothing (the same registers
 * and spills per kernel) and this status never occurs.
 *
 * For the checked build's own tests: film pixel checks accept only pixels
 * below `pixels` (0, the initial state: the film's own size), so that a normal
 * render fails a check whose access would have been in bounds. Applies to
 * wavefronts laid out after the call; process-wide; ignored by the plain
 * library. No counterpart in the reference. */
void lt_debug_set_check_pixel_limit(uint32_t pixels);

#ifdef __cplusplus
}
#endif
#endif
