/*
 * lt_oracle.h -- CPU restatement of Lantern's per-pixel path-tracing loop.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker that the CUDA path is compared
 * with; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it. The shipped library never links or calls it.
 *
 * Parity: pinned. Two ways, both in tests/:
 *  - the reference integrator itself (source/core/integrator/integrator.cpp and
 *    the camera/material/light/sampler sources it calls) is compiled from the
 *    reference tree by oracle/build_ref.sh against a project rtc* shim that
 *    calls this file's intersector; with the reference's per-tile sampler
 *    keying (LT_KEY_TILE) this restatement reproduces its films bit for bit;
 *  - golden vectors produced by that build are committed in tests/golden/.
 * The reference has no tests or golden data of its own; Embree 3.5 (the
 * reference's intersector, third_party/embree) cannot be built from the
 * snapshot, so intersection follows Embree's published Moeller-Trumbore
 * arithmetic (kernels/geometry/triangle_intersector_moeller.h:75-112) and is
 * checked against brute force.
 */
#ifndef LT_ORACLE_H
#define LT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* sampler keying: per 8x8 tile and frame (integrator.cpp:75-96), or per
 * (pixel, frame) as the GPU path does */
enum { LT_KEY_TILE = 0, LT_KEY_PIXEL = 1 };

enum { ORC_BSDF_LAMBERT = 0, ORC_BSDF_MIRROR = 1, ORC_BSDF_DIELECTRIC = 2 };
enum { ORC_MED_NON_SCATTERING = 1, ORC_MED_ISOTROPIC = 2, ORC_MED_HG = 3 };

typedef struct orc_scene orc_scene;

orc_scene *orc_scene_new(void);
void orc_scene_free(orc_scene *s);

/* camera (pinhole_camera.cpp:27-40) and background colour */
void orc_set_camera(orc_scene *s, float phi, float theta, float radius, uint32_t width,
                    uint32_t height, const float target[3], float fov);
void orc_set_background(orc_scene *s, const float rgb[3]);

/* material/medium tables; return the new index */
int orc_add_medium(orc_scene *s, int type, const float sigma_a[3], const float sigma_s[3], float g);
/* the reference's medium parameters: absorption colour at a distance, and a
 * scattering distance (isotropic only) */
int orc_add_medium_ref(orc_scene *s, int type, const float color[3], float at_distance,
                       float scattering_distance);
int orc_add_material(orc_scene *s, int bsdf, const float albedo[3], float ior, int medium);

/* One mesh (geomID = call order, as rtcAttachGeometry numbers them).
 * positions are world space (3 floats per vertex); normals may be NULL.
 * emission_color may be NULL (no light). Returns geomID. */
int orc_add_mesh(orc_scene *s, const float *positions, uint32_t num_verts, const float *normals,
                 const uint32_t *indices, uint32_t num_tris, int material,
                 const float *emission_color, float radiant_power);

/* Build the BVH2 over all meshes. Returns 0 on success. */
int orc_scene_commit(orc_scene *s);

/* Albedo textures (before commit): an 8-bit image (rows from the top,
 * channels 1-4) -> its index; a material's texture: -1 constant albedo,
 * -2 uv, >= 0 image index; a mesh's per-vertex texture coordinates (2 floats
 * per vertex of that mesh). */
int orc_add_image(orc_scene *s, const uint8_t *texels, uint32_t w, uint32_t h, uint32_t ch);
void orc_set_material_texture(orc_scene *s, int mat, int tex);
void orc_set_mesh_texcoords(orc_scene *s, int geom_id, const float *tc);

/* Light data derived at load (scene.cpp:49-80,463-473; area_light.h:16-21). */
void orc_light_info(const orc_scene *s, int light, float *area, float sphere[4], float radiance[3]);
uint32_t orc_num_triangles(const orc_scene *s);

/* Closest hit for n rays of 8 floats (org.xyz, tnear, dir.xyz, tfar).
 * hits: 4 words per ray (t, u, v as float bits; prim = global triangle index
 * or 0xFFFFFFFF). use_bvh=0 tests every triangle. counters (may be NULL):
 * per ray [node visits, triangle tests]. */
void orc_intersect(const orc_scene *s, const float *rays, uint32_t *hits, uint64_t n,
                   int use_bvh, uint32_t *counters, int threads);

/* One closest-hit query; returns 1 on a hit and fills t/u/v, the global
 * triangle index and its (geomID, primID within the geometry). */
int orc_intersect1(const orc_scene *s, const float org[3], const float dir[3], float tnear, float tfar,
                   float *t, float *u, float *v, uint32_t *prim, uint32_t *geom_id, uint32_t *local_prim);

/* Render frames [first_frame, first_frame + num_frames) additively.
 * films: rgb (W*H*3 floats), bounces (W*H), counts (W*H). With LT_KEY_TILE and
 * two films (film_b non-NULL) frames alternate B, A, B, ... as in the
 * reference's swap (integrator.cpp:35) with A the film passed first.
 * ray_counts (may be NULL): [main, light-sample, bsdf-mis] rays traced. */
typedef struct {
    uint32_t max_depth; /* reference: 1500 (integrator.cpp:114) */
    uint32_t rr_depth;  /* Russian roulette when bounces > rr_depth (reference: 3) */
    uint32_t keying;    /* LT_KEY_TILE or LT_KEY_PIXEL */
    uint32_t threads;
} orc_render_opts;

void orc_render(const orc_scene *s, const orc_render_opts *o, uint32_t first_frame,
                uint32_t num_frames, float *rgb_a, uint32_t *bounces_a, uint32_t *counts_a,
                float *rgb_b, uint32_t *bounces_b, uint32_t *counts_b, uint64_t *ray_counts);

/* One path for (pixel, frame) with pixel keying; writes colour and bounces.
 * Used by tests for path-by-path checks. */
void orc_render_path(const orc_scene *s, const orc_render_opts *o, uint32_t x, uint32_t y,
                     uint32_t frame, float color[3], uint32_t *bounces);

/* Read-only scene views for the differentiable reference (lt_diff_ref.cpp).
 * cam = origin, mx, my, mz (3 floats each), tanx, tany. */
void orc_camera_info(const orc_scene *s, float cam[14], uint32_t *w, uint32_t *h);
void orc_background_info(const orc_scene *s, float rgb[3]);
int orc_num_lights(const orc_scene *s);
int orc_num_media(const orc_scene *s);
int orc_light_geom(const orc_scene *s, int i);
uint32_t orc_tri_geom(const orc_scene *s, uint32_t prim);
void orc_geom_info(const orc_scene *s, uint32_t g, int *material, int *light, int *has_normals);
void orc_material_info(const orc_scene *s, int m, int *bsdf, float albedo[3], float *ior, int *medium);
void orc_medium_info(const orc_scene *s, int m, int *type, float sa[3], float ss[3], float *g);
void orc_tri_normals(const orc_scene *s, uint32_t prim, float n[9]);

/* Differentiable estimator and its gradient (oracle/lt_diff_ref.cpp), in
 * double (fp64 != 0) or float. Parameters as for lt_render_diff (host arrays,
 * detached copies = the parameters). dI: d loss / d film colour sum (W*H*3).
 * crop = x0, y0, x1, y1. Outputs: film colour sums of the crop's pixels (W*H*3,
 * other pixels untouched) and gradients (accumulated, double). */
void orc_diff_render(const orc_scene *s, int fp64, const float *albedo, const float *emission,
                     const float *sigma_a, const float *sigma_s, uint32_t spp, uint32_t first_frame,
                     uint32_t max_depth, uint32_t rr_depth, const uint32_t crop[4], const float *dI,
                     double *rgb, double *g_albedo, double *g_emission, double *g_sigma_a, double *g_sigma_s,
                     int threads);

/* Final resolve (visualizer.cpp:352-364, final_resolve_ps.glsl:24-43): per
 * pixel c = exp2f(exposure_stops) * (rgb / count, 1), tone mapped by clamp
 * (tonemap 0) or the filmic curve (1); rgba8 = round(c * 255). Either output
 * may be NULL; spp_minmax / spp_sum (optional) get the sample-count range. */
void orc_resolve(const float *rgb, const uint32_t *counts, uint64_t npix, int tonemap, float exposure_stops,
                 float *rgba, uint8_t *rgba8, uint32_t spp_minmax[2], uint64_t *spp_sum);

/* Building blocks, exported for golden-vector checks against the reference. */
void orc_pcg_stream(uint64_t seed, uint64_t seq, uint32_t n, uint32_t *out_uint, float *out_float);
uint32_t orc_tile_seed(uint32_t tile, uint32_t frame);
float orc_filter_sample(float x);
void orc_camera_ray(const orc_scene *s, uint32_t x, uint32_t y, float u, float v, float out_dir[3],
                    float out_org[3]);

#ifdef __cplusplus
}
#endif
#endif
