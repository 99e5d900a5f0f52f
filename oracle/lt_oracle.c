/*
 * lt_oracle.c -- CPU restatement of Lantern's per-pixel path-tracing loop.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (see lt_oracle.h).
 * Compile with -ffp-contract=off: every float operation below is meant to be
 * the single-rounded IEEE operation the reference source spells out, in the
 * reference's order, so that the x86 container and the aarch64 GPU host agree
 * bit for bit and agree with the reference build in oracle/_ref.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the Lantern source tree).
 */
#include "lt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.14159265358979323846f
#define INV_PI_F 0.318309886183790671538f /* (float)M_1_PI */

/* ------------------------------------------------------------------ vectors */
typedef struct { float x, y, z; } v3;

static inline v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 muls(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 divs(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
/* vector dot/cross as the scalar Embree-math compatibility header defines them
 * for the reference build ((x + y) + z) */
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float length(v3 a) { return sqrtf(dot(a, a)); }
static inline v3 normalize(v3 a) { return muls(a, 1.0f / sqrtf(dot(a, a))); }
static inline int all_zero(v3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; } /* vector_math.h:17-22 */
static inline v3 ld3(const float *p) { return mk(p[0], p[1], p[2]); }

/* ------------------------------------------------------------------ sampler */
/* PCG32 XSH-RR, math/uniform_sampler.h:17-57 */
typedef struct { uint64_t state, seq; } pcg;

static inline uint32_t pcg_next(pcg *g) {
    uint64_t old = g->state;
    g->state = old * 6364136223846793005ULL + (g->seq | 1u);
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}
static inline void pcg_init(pcg *g, uint64_t seed, uint64_t seq) {
    g->state = seed;
    g->seq = seq;
    (void)pcg_next(g);
}
static inline float pcg_float(pcg *g) {
    uint32_t bits = (pcg_next(g) >> 9u) | 0x3F800000u;
    float f;
    memcpy(&f, &bits, 4);
    return f - 1.0f;
}
static inline uint32_t pcg_discrete(pcg *g, uint32_t range) {
    return (uint32_t)((float)range * pcg_float(g));
}

/* MurmurHash3 mix/finalize, integrator.cpp:46-72 */
static inline uint32_t hash_mix(uint32_t h, uint32_t k) {
    k *= 0xcc9e2d51u;
    k = (k << 15) | (k >> 17);
    k *= 0x1b873593u;
    h ^= k;
    h = ((h << 13) | (h >> 19)) * 5u + 0xe6546b64u;
    return h;
}
static inline uint32_t hash_fin(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
uint32_t orc_tile_seed(uint32_t tile, uint32_t frame) {
    return hash_fin(hash_mix(hash_mix(0u, tile), frame));
}

void orc_pcg_stream(uint64_t seed, uint64_t seq, uint32_t n, uint32_t *ou, float *of) {
    pcg g;
    pcg_init(&g, seed, seq);
    for (uint32_t i = 0; i < n; ++i) {
        if (ou) ou[i] = pcg_next(&g);
        else of[i] = pcg_float(&g);
    }
}

/* ------------------------------------------------------------------ tent filter */
/* ReconstructionFilter PreCompute/Sample, camera/reconstruction_filter.cpp:34-87,106-142
 * (Tent, width 1, 32 bins). */
#define NBINS 32
static float g_cdf[NBINS + 1];
static float g_bin_size;
static pthread_once_t g_filter_once = PTHREAD_ONCE_INIT;

static void filter_init(void) {
    const float width = 1.0f;
    g_bin_size = width / (NBINS - 1);
    float norm = 0.0f, pdf[NBINS];
    for (uint32_t i = 0; i < NBINS - 1; ++i) {
        float t = width - fabsf((float)i * g_bin_size);
        pdf[i] = t;
        norm += t;
    }
    pdf[NBINS - 1] = 0.0f;
    for (uint32_t i = 0; i < NBINS - 1; ++i) pdf[i] /= norm;
    g_cdf[0] = 0.0f;
    for (uint32_t i = 1; i < NBINS; ++i) g_cdf[i] = g_cdf[i - 1] + pdf[i - 1];
    g_cdf[NBINS] = 1.0f;
}

float orc_filter_sample(float x) {
    pthread_once(&g_filter_once, filter_init);
    int negative = x < 0.5f;
    x = negative ? x * 2.0f : (x - 0.5f) * 2.0f;
    uint32_t index = NBINS;
    for (uint32_t i = 1; i < NBINS + 1; ++i) {
        if (x < g_cdf[i]) { index = i - 1; break; }
    }
    float pdf = g_cdf[index + 1] - g_cdf[index];
    float u = g_bin_size * ((float)index + ((x - g_cdf[index]) / pdf));
    return negative ? -u : u;
}

/* ------------------------------------------------------------------ scene */
typedef struct { int bsdf; v3 albedo; float ior; int medium; int tex; } material; /* tex: -1 constant, -2 uv, >= 0 image */
typedef struct { uint8_t *texels; uint32_t w, h, ch; } image;
typedef struct { int type; v3 sigma_a; v3 sigma_s; float g; } medium;
typedef struct { int geom; v3 radiance; float area; float sphere[4]; } light;
typedef struct { uint32_t tri_begin, tri_count; int material, light, has_normals, has_texcoords; uint32_t vbase, nverts; } geom;

typedef struct { float lo[3], hi[3]; int32_t left, right; uint32_t first, count; } bnode;

struct orc_scene {
    /* camera, pinhole_camera.cpp:27-40 and pinhole_camera.h:216-236 */
    uint32_t width, height;
    v3 origin, mx, my, mz;
    float tanx, tany;
    v3 background;

    material *mats; int nmats, cmats;
    medium *meds; int nmeds, cmeds;
    light *lights; int nlights, clights;
    geom *geoms; int ngeoms, cgeoms;

    /* triangles: v0, e1 = v0 - v1, e2 = v2 - v0 (Embree Triangle4 layout,
     * kernels/geometry/triangle.h:54) */
    float *tri; uint32_t ntris, ctris;
    uint32_t *tri_geom;
    uint32_t *tri_vidx;
    float *vnormal; uint32_t nverts, cverts;
    float *vtex;       /* 2 per vertex, 0 where a mesh has none */
    image *images; int nimages, cimages;

    bnode *nodes; uint32_t nnodes;
    uint32_t *order; /* BVH leaf order -> triangle index */
};

#define GROW(ptr, n, cap, extra, type)                                           \
    do {                                                                         \
        if ((n) + (extra) > (cap)) {                                             \
            size_t nc = (cap) ? (size_t)(cap) : 16;                              \
            while (nc < (size_t)(n) + (extra)) nc *= 2;                          \
            ptr = (type *)realloc(ptr, nc * sizeof(type));                       \
            cap = nc;                                                            \
        }                                                                        \
    } while (0)

orc_scene *orc_scene_new(void) {
    orc_scene *s = (orc_scene *)calloc(1, sizeof(orc_scene));
    pthread_once(&g_filter_once, filter_init);
    return s;
}

void orc_scene_free(orc_scene *s) {
    if (!s) return;
    free(s->mats); free(s->meds); free(s->lights); free(s->geoms);
    free(s->tri); free(s->tri_geom); free(s->tri_vidx); free(s->vnormal); free(s->vtex);
    for (int i = 0; i < s->nimages; ++i) free(s->images[i].texels);
    free(s->images);
    free(s->nodes); free(s->order);
    free(s);
}

void orc_set_camera(orc_scene *s, float phi, float theta, float radius, uint32_t w, uint32_t h,
                    const float target[3], float fov) {
    s->width = w;
    s->height = h;
    s->tanx = tanf(fov * 0.5f);
    s->tany = tanf(fov * 0.5f * (float)h / (float)w);
    v3 t = ld3(target);
    float x = radius * sinf(phi) * sinf(theta);
    float y = radius * cosf(phi);
    float z = radius * sinf(phi) * cosf(theta);
    s->origin = add(t, mk(x, y, z));
    const float up = 1.0f;
    v3 za = normalize(sub(s->origin, t));
    v3 xa;
    if (za.x == 0.0f && (za.y == 1.0f || za.y == -1.0f) && za.z == 0.0f)
        xa = normalize(cross(mk(0.0f, 0.0f, up), za));
    else
        xa = normalize(cross(mk(0.0f, up, 0.0f), za));
    v3 ya = cross(za, xa);
    s->mx = mk(xa.x, ya.x, za.x);
    s->my = mk(xa.y, ya.y, za.y);
    s->mz = mk(xa.z, ya.z, za.z);
}

void orc_set_background(orc_scene *s, const float rgb[3]) { s->background = ld3(rgb); }

int orc_add_medium(orc_scene *s, int type, const float sa[3], const float ss[3], float g) {
    GROW(s->meds, s->nmeds, s->cmeds, 1, medium);
    medium m = {type, ld3(sa), ld3(ss), g};
    s->meds[s->nmeds] = m;
    return s->nmeds++;
}

/* Medium ctor (materials/media/medium.h:19-23): sigma_a = -log(color) / distance;
 * IsotropicScatteringMedium (isotropic_scattering_medium.h:22-25): sigma_s = 1 / distance */
int orc_add_medium_ref(orc_scene *s, int type, const float color[3], float at_distance,
                       float scattering_distance) {
    float sa[3], ss[3];
    for (int c = 0; c < 3; ++c) {
        sa[c] = -logf(color[c]) / at_distance;
        ss[c] = type == ORC_MED_ISOTROPIC ? 1 / scattering_distance : 0.0f;
    }
    return orc_add_medium(s, type, sa, ss, 0.0f);
}

int orc_add_material(orc_scene *s, int bsdf, const float albedo[3], float ior, int med) {
    GROW(s->mats, s->nmats, s->cmats, 1, material);
    material m = {bsdf, ld3(albedo), ior, med, -1};
    s->mats[s->nmats] = m;
    return s->nmats++;
}

/* CalculateBoundingSphere, scene.cpp:49-80 */
static void bounding_sphere(const float *p, uint32_t n, float out[4]) {
    v3 c = ld3(p);
    float r = 0.0001f;
    for (int pass = 0; pass < 2; ++pass) {
        for (uint32_t j = 0; j < n; ++j) {
            v3 pos = ld3(p + 3 * j);
            v3 d = sub(pos, c);
            float len = length(d);
            if (len > r) {
                float a = len / r;
                float a2 = a * a;
                r = 0.5f * (a + 1 / a) * r;
                c = muls(add(muls(c, 1 + 1 / a2), muls(pos, 1 - 1 / a2)), 0.5f);
            }
        }
    }
    for (uint32_t j = 0; j < n; ++j) {
        v3 pos = ld3(p + 3 * j);
        v3 d = sub(pos, c);
        float len = length(d);
        if (len > r) {
            r = (r + len) / 2.0f;
            c = add(c, muls(d, (len - r) / len));
        }
    }
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = r;
}

int orc_add_mesh(orc_scene *s, const float *pos, uint32_t nv, const float *nrm,
                 const uint32_t *idx, uint32_t nt, int mat, const float *em, float power) {
    GROW(s->geoms, s->ngeoms, s->cgeoms, 1, geom);
    int gid = s->ngeoms++;
    geom *g = &s->geoms[gid];
    g->tri_begin = s->ntris;
    g->tri_count = nt;
    g->material = mat;
    g->light = -1;
    g->has_normals = nrm != NULL;
    g->has_texcoords = 0;

    uint32_t vbase = s->nverts;
    g->vbase = vbase;
    g->nverts = nv;
    s->vnormal = (float *)realloc(s->vnormal, (size_t)(s->nverts + nv) * 3 * sizeof(float));
    s->vtex = (float *)realloc(s->vtex, (size_t)(s->nverts + nv) * 2 * sizeof(float));
    for (uint32_t i = 0; i < nv; ++i) {
        for (int c = 0; c < 3; ++c) s->vnormal[3 * (vbase + i) + c] = nrm ? nrm[3 * i + c] : 0.0f;
        s->vtex[2 * (vbase + i)] = s->vtex[2 * (vbase + i) + 1] = 0.0f;
    }
    s->nverts += nv;

    size_t T = (size_t)s->ntris + nt;
    s->tri = (float *)realloc(s->tri, T * 9 * sizeof(float));
    s->tri_geom = (uint32_t *)realloc(s->tri_geom, T * sizeof(uint32_t));
    s->tri_vidx = (uint32_t *)realloc(s->tri_vidx, T * 3 * sizeof(uint32_t));
    float area = 0.0f;
    for (uint32_t t = 0; t < nt; ++t) {
        v3 a = ld3(pos + 3 * idx[3 * t]);
        v3 b = ld3(pos + 3 * idx[3 * t + 1]);
        v3 c = ld3(pos + 3 * idx[3 * t + 2]);
        size_t k = s->ntris + t;
        v3 e1 = sub(a, b), e2 = sub(c, a);
        float *d = s->tri + 9 * k;
        d[0] = a.x; d[1] = a.y; d[2] = a.z;
        d[3] = e1.x; d[4] = e1.y; d[5] = e1.z;
        d[6] = e2.x; d[7] = e2.y; d[8] = e2.z;
        s->tri_geom[k] = (uint32_t)gid;
        for (int j = 0; j < 3; ++j) s->tri_vidx[3 * k + j] = vbase + idx[3 * t + j];
        /* scene.cpp:465-471 */
        area += 0.5f * length(cross(sub(a, b), sub(a, c)));
    }
    s->ntris += nt;

    if (em) {
        GROW(s->lights, s->nlights, s->clights, 1, light);
        light *L = &s->lights[s->nlights];
        L->geom = gid;
        L->area = area;
        bounding_sphere(pos, nv, L->sphere);
        /* AreaLight ctor: color * radiantPower * (float)M_1_PI / area */
        L->radiance = divs(muls(muls(ld3(em), power), INV_PI_F), area);
        g->light = s->nlights++;
    }
    return gid;
}

void orc_light_info(const orc_scene *s, int i, float *area, float sphere[4], float rad[3]) {
    const light *L = &s->lights[i];
    *area = L->area;
    memcpy(sphere, L->sphere, 4 * sizeof(float));
    rad[0] = L->radiance.x; rad[1] = L->radiance.y; rad[2] = L->radiance.z;
}

uint32_t orc_num_triangles(const orc_scene *s) { return s->ntris; }

/* ------------------------------------------------------------------ BVH2 build */
/* Binned SAH (32 bins over centroids), at most 4 triangles per leaf. */
typedef struct { float lo[3], hi[3]; } aabb;

static inline void bb_empty(aabb *b) {
    for (int c = 0; c < 3; ++c) { b->lo[c] = INFINITY; b->hi[c] = -INFINITY; }
}
static inline void bb_grow(aabb *b, const aabb *o) {
    for (int c = 0; c < 3; ++c) {
        if (o->lo[c] < b->lo[c]) b->lo[c] = o->lo[c];
        if (o->hi[c] > b->hi[c]) b->hi[c] = o->hi[c];
    }
}
static inline float bb_area(const aabb *b) {
    float dx = b->hi[0] - b->lo[0], dy = b->hi[1] - b->lo[1], dz = b->hi[2] - b->lo[2];
    if (dx < 0) return 0.0f;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

typedef struct { aabb *tb; float *cen; uint32_t *idx; bnode *nodes; uint32_t nnodes, cnodes; } builder;

static uint32_t new_node(builder *B) {
    if (B->nnodes == B->cnodes) {
        B->cnodes = B->cnodes ? B->cnodes * 2 : 1024;
        B->nodes = (bnode *)realloc(B->nodes, B->cnodes * sizeof(bnode));
    }
    return B->nnodes++;
}

static void build_rec(builder *B, uint32_t ni, uint32_t begin, uint32_t end) {
    aabb nb, cb;
    bb_empty(&nb);
    bb_empty(&cb);
    for (uint32_t i = begin; i < end; ++i) {
        uint32_t t = B->idx[i];
        bb_grow(&nb, &B->tb[t]);
        aabb c;
        for (int k = 0; k < 3; ++k) c.lo[k] = c.hi[k] = B->cen[3 * t + k];
        bb_grow(&cb, &c);
    }
    bnode *n = &B->nodes[ni];
    memcpy(n->lo, nb.lo, sizeof nb.lo);
    memcpy(n->hi, nb.hi, sizeof nb.hi);
    uint32_t count = end - begin;
    if (count <= 4) {
        n->left = n->right = -1;
        n->first = begin;
        n->count = count;
        return;
    }
    int best_axis = -1, best_bin = -1;
    float best_cost = INFINITY;
    for (int ax = 0; ax < 3; ++ax) {
        float lo = cb.lo[ax], ext = cb.hi[ax] - cb.lo[ax];
        if (!(ext > 0.0f)) continue;
        aabb bins[NBINS];
        uint32_t cnt[NBINS];
        for (int b = 0; b < NBINS; ++b) { bb_empty(&bins[b]); cnt[b] = 0; }
        float k = (float)NBINS / ext;
        for (uint32_t i = begin; i < end; ++i) {
            uint32_t t = B->idx[i];
            int b = (int)((B->cen[3 * t + ax] - lo) * k);
            if (b >= NBINS) b = NBINS - 1;
            if (b < 0) b = 0;
            bb_grow(&bins[b], &B->tb[t]);
            cnt[b]++;
        }
        float rarea[NBINS];
        uint32_t rcnt[NBINS];
        aabb acc;
        bb_empty(&acc);
        uint32_t c = 0;
        for (int b = NBINS - 1; b > 0; --b) {
            bb_grow(&acc, &bins[b]);
            c += cnt[b];
            rarea[b] = bb_area(&acc);
            rcnt[b] = c;
        }
        bb_empty(&acc);
        c = 0;
        for (int b = 0; b < NBINS - 1; ++b) {
            bb_grow(&acc, &bins[b]);
            c += cnt[b];
            if (c == 0 || rcnt[b + 1] == 0) continue;
            float cost = bb_area(&acc) * (float)c + rarea[b + 1] * (float)rcnt[b + 1];
            if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = b; }
        }
    }
    uint32_t mid;
    if (best_axis < 0) {
        mid = begin + count / 2;
    } else {
        float lo = cb.lo[best_axis], ext = cb.hi[best_axis] - cb.lo[best_axis];
        float k = (float)NBINS / ext;
        uint32_t i = begin, j = end;
        while (i < j) {
            uint32_t t = B->idx[i];
            int b = (int)((B->cen[3 * t + best_axis] - lo) * k);
            if (b >= NBINS) b = NBINS - 1;
            if (b < 0) b = 0;
            if (b <= best_bin) {
                ++i;
            } else {
                --j;
                uint32_t tmp = B->idx[i];
                B->idx[i] = B->idx[j];
                B->idx[j] = tmp;
            }
        }
        mid = i;
        if (mid == begin || mid == end) mid = begin + count / 2;
    }
    uint32_t l = new_node(B);
    uint32_t r = new_node(B);
    n = &B->nodes[ni];
    n->left = (int32_t)l;
    n->right = (int32_t)r;
    n->first = 0;
    n->count = 0;
    build_rec(B, l, begin, mid);
    build_rec(B, r, mid, end);
}

int orc_scene_commit(orc_scene *s) {
    free(s->nodes);
    free(s->order);
    s->nodes = NULL;
    s->order = NULL;
    s->nnodes = 0;
    if (s->ntris == 0) return 0;
    builder B;
    memset(&B, 0, sizeof B);
    B.tb = (aabb *)malloc(s->ntris * sizeof(aabb));
    B.cen = (float *)malloc((size_t)s->ntris * 3 * sizeof(float));
    B.idx = (uint32_t *)malloc(s->ntris * sizeof(uint32_t));
    for (uint32_t t = 0; t < s->ntris; ++t) {
        const float *d = s->tri + 9 * (size_t)t;
        v3 a = ld3(d), e1 = ld3(d + 3), e2 = ld3(d + 6);
        v3 b = sub(a, e1), c = add(a, e2);
        v3 p[3] = {a, b, c};
        bb_empty(&B.tb[t]);
        for (int j = 0; j < 3; ++j) {
            aabb q;
            q.lo[0] = q.hi[0] = p[j].x;
            q.lo[1] = q.hi[1] = p[j].y;
            q.lo[2] = q.hi[2] = p[j].z;
            bb_grow(&B.tb[t], &q);
        }
        for (int k = 0; k < 3; ++k) B.cen[3 * t + k] = 0.5f * (B.tb[t].lo[k] + B.tb[t].hi[k]);
        B.idx[t] = t;
    }
    uint32_t root = new_node(&B);
    build_rec(&B, root, 0, s->ntris);
    s->nodes = B.nodes;
    s->nnodes = B.nnodes;
    s->order = B.idx;
    free(B.tb);
    free(B.cen);
    return 0;
}

/* ------------------------------------------------------------------ intersection */
/* Moeller-Trumbore as Embree 3.5 evaluates it for one triangle
 * (kernels/geometry/triangle_intersector_moeller.h:75-112, intersectEdge :117-124):
 * Ng = cross(e2, e1); C = v0 - O; R = cross(C, D); den = dot(Ng, D);
 * U = dot(R, e2) ^ sign(den); V = dot(R, e1) ^ sign(den); accept iff den != 0,
 * U >= 0, V >= 0, U + V <= |den|, |den|*tnear < T <= |den|*tfar with
 * T = dot(Ng, C) ^ sign(den). Embree's vector dot is x*x + (y*y + z*z) and no
 * FMA is used (SSE2 build). t, u, v are T, U, V / |den| by exact division; Embree
 * multiplies by an approximate reciprocal (finalize, :42-47), hence the 1e-5
 * relative tolerance on t against Embree itself. */
static inline float edot(v3 a, v3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
static inline float xorsign(float a, uint32_t s) {
    uint32_t u;
    memcpy(&u, &a, 4);
    u ^= s;
    memcpy(&a, &u, 4);
    return a;
}

static inline int tri_test(const float *d, v3 O, v3 D, float tnear, float tfar, float *ot, float *ou,
                           float *ov) {
    v3 v0 = ld3(d), e1 = ld3(d + 3), e2 = ld3(d + 6);
    v3 Ng = cross(e2, e1);
    v3 C = sub(v0, O);
    v3 R = cross(C, D);
    float den = edot(Ng, D);
    float absden = fabsf(den);
    uint32_t sgn;
    memcpy(&sgn, &den, 4);
    sgn &= 0x80000000u;
    float U = xorsign(edot(R, e2), sgn);
    float V = xorsign(edot(R, e1), sgn);
    if (!(den != 0.0f && U >= 0.0f && V >= 0.0f && U + V <= absden)) return 0;
    float T = xorsign(edot(Ng, C), sgn);
    if (!(absden * tnear < T && T <= absden * tfar)) return 0;
    *ot = T / absden;
    *ou = U / absden;
    *ov = V / absden;
    return 1;
}

typedef struct { float t, u, v; uint32_t prim; } hitrec;

static inline float safe_inv(float d) { return 1.0f / (fabsf(d) > 1e-30f ? d : copysignf(1e-30f, d)); }

/* Conservative slab test: the far distance is widened by 2*gamma(3) so that a
 * triangle hit inside the box is never culled by rounding. */
static inline int box_test(const bnode *n, v3 O, v3 inv, float tnear, float tfar, float *tentry) {
    float tx0 = (n->lo[0] - O.x) * inv.x, tx1 = (n->hi[0] - O.x) * inv.x;
    float ty0 = (n->lo[1] - O.y) * inv.y, ty1 = (n->hi[1] - O.y) * inv.y;
    float tz0 = (n->lo[2] - O.z) * inv.z, tz1 = (n->hi[2] - O.z) * inv.z;
    float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tnear));
    float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tfar));
    *tentry = tmin;
    return tmin <= tmax * 1.0000004f;
}

static void intersect1(const orc_scene *s, v3 O, v3 D, float tnear, float tfar, int use_bvh,
                       hitrec *h, uint32_t *cnt) {
    h->prim = 0xFFFFFFFFu;
    h->t = tfar;
    h->u = h->v = 0.0f;
    uint32_t nodes = 0, tests = 0;
    if (!use_bvh || !s->nodes) {
        for (uint32_t i = 0; i < s->ntris; ++i) {
            float t, u, v;
            if (tri_test(s->tri + 9 * (size_t)i, O, D, tnear, h->t, &t, &u, &v)) {
                h->t = t; h->u = u; h->v = v; h->prim = i;
            }
        }
        tests = s->ntris;
    } else {
        v3 inv = mk(safe_inv(D.x), safe_inv(D.y), safe_inv(D.z));
        uint32_t stack[128];
        float stt[128];
        int sp = 0;
        float te;
        nodes++;
        if (box_test(&s->nodes[0], O, inv, tnear, h->t, &te)) {
            stack[sp] = 0;
            stt[sp++] = te;
        }
        while (sp > 0) {
            --sp;
            if (stt[sp] > h->t * 1.0000004f) continue;
            const bnode *n = &s->nodes[stack[sp]];
            if (n->left < 0) {
                for (uint32_t k = 0; k < n->count; ++k) {
                    uint32_t ti = s->order[n->first + k];
                    float t, u, v;
                    tests++;
                    if (tri_test(s->tri + 9 * (size_t)ti, O, D, tnear, h->t, &t, &u, &v)) {
                        h->t = t; h->u = u; h->v = v; h->prim = ti;
                    }
                }
                continue;
            }
            float tl, tr;
            nodes += 2;
            int hl = box_test(&s->nodes[n->left], O, inv, tnear, h->t, &tl);
            int hr = box_test(&s->nodes[n->right], O, inv, tnear, h->t, &tr);
            if (hl && hr) {
                if (tl <= tr) {
                    stack[sp] = (uint32_t)n->right; stt[sp++] = tr;
                    stack[sp] = (uint32_t)n->left; stt[sp++] = tl;
                } else {
                    stack[sp] = (uint32_t)n->left; stt[sp++] = tl;
                    stack[sp] = (uint32_t)n->right; stt[sp++] = tr;
                }
            } else if (hl) {
                stack[sp] = (uint32_t)n->left; stt[sp++] = tl;
            } else if (hr) {
                stack[sp] = (uint32_t)n->right; stt[sp++] = tr;
            }
        }
    }
    if (cnt) { cnt[0] = nodes; cnt[1] = tests; }
}

int orc_intersect1(const orc_scene *s, const float org[3], const float dir[3], float tnear, float tfar,
                   float *t, float *u, float *v, uint32_t *prim, uint32_t *geom_id, uint32_t *local_prim) {
    hitrec h;
    intersect1(s, ld3(org), ld3(dir), tnear, tfar, 1, &h, NULL);
    *prim = h.prim;
    if (h.prim == 0xFFFFFFFFu) return 0;
    *t = h.t; *u = h.u; *v = h.v;
    uint32_t g = s->tri_geom[h.prim];
    *geom_id = g;
    *local_prim = h.prim - s->geoms[g].tri_begin;
    return 1;
}

/* ------------------------------------------------------------------ thread pool */
typedef struct {
    void (*fn)(void *ctx, uint64_t item);
    void *ctx;
    uint64_t n;
    volatile uint64_t next;
} job;

static void *worker(void *arg) {
    job *j = (job *)arg;
    for (;;) {
        uint64_t i = __sync_fetch_and_add(&j->next, 1);
        if (i >= j->n) break;
        j->fn(j->ctx, i);
    }
    return NULL;
}

static void parallel_for(uint64_t n, int threads, void (*fn)(void *, uint64_t), void *ctx) {
    job j = {fn, ctx, n, 0};
    if (threads <= 1) {
        worker(&j);
        return;
    }
    pthread_t th[256];
    if (threads > 256) threads = 256;
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, worker, &j);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
}

typedef struct { const orc_scene *s; const float *rays; uint32_t *hits; int use_bvh; uint32_t *counters; uint64_t n; } isect_ctx;

static void isect_chunk(void *c, uint64_t chunk) {
    isect_ctx *x = (isect_ctx *)c;
    uint64_t b = chunk * 4096, e = b + 4096;
    if (e > x->n) e = x->n;
    for (uint64_t i = b; i < e; ++i) {
        const float *r = x->rays + 8 * i;
        hitrec h;
        intersect1(x->s, mk(r[0], r[1], r[2]), mk(r[4], r[5], r[6]), r[3], r[7], x->use_bvh, &h,
                   x->counters ? x->counters + 2 * i : NULL);
        memcpy(&x->hits[4 * i + 0], &h.t, 4);
        memcpy(&x->hits[4 * i + 1], &h.u, 4);
        memcpy(&x->hits[4 * i + 2], &h.v, 4);
        x->hits[4 * i + 3] = h.prim;
    }
}

void orc_intersect(const orc_scene *s, const float *rays, uint32_t *hits, uint64_t n, int use_bvh,
                   uint32_t *counters, int threads) {
    isect_ctx c = {s, rays, hits, use_bvh, counters, n};
    parallel_for((n + 4095) / 4096, threads, isect_chunk, &c);
}

/* ------------------------------------------------------------------ shading helpers */
/* RotateToWorld, math/vector_math.cpp:12-33 */
static inline v3 rotate_to_world(float x, float y, float z, v3 n) {
    v3 major;
    if (fabsf(n.x) < 0.57735026919f) major = mk(1, 0, 0);
    else if (fabsf(n.y) < 0.57735026919f) major = mk(0, 1, 0);
    else major = mk(0, 0, 1);
    v3 u = normalize(cross(n, major));
    v3 v = cross(n, u);
    return add(add(muls(u, x), muls(v, y)), muls(n, z));
}

/* UniformSampleDisc, math/sampling.h:29-36 */
static inline void sample_disc(pcg *g, float radius, float *x, float *y) {
    float rnd = pcg_float(g);
    float r = sqrtf(rnd) * radius;
    float theta = pcg_float(g) * 2.0f * PI_F;
    *x = r * cosf(theta);
    *y = r * sinf(theta);
}

/* CosineSampleHemisphere, math/sampling.h:48-58 */
static inline v3 cosine_hemisphere(v3 n, pcg *g) {
    float x, y;
    sample_disc(g, 1.0f, &x, &y);
    float z = sqrtf(1.0f - x * x - y * y);
    return normalize(rotate_to_world(x, y, z, n));
}

/* UniformSampleSphere, math/sampling.h:72-84 */
static inline v3 uniform_sphere(pcg *g) {
    float cphi = 2.0f * pcg_float(g) - 1.0f;
    float sphi = sqrtf(1.0f - cphi * cphi);
    float theta = 2 * PI_F * pcg_float(g);
    return mk(sphi * sinf(theta), cphi, sphi * cosf(theta));
}

/* Henyey-Greenstein phase sampling (extension, no reference counterpart):
 * cos(theta) between the continuing direction and the incoming one, inverted
 * from the HG CDF; g == 0 falls back to the reference's uniform sphere so the
 * reference-expressible medium is reproduced exactly. */
static inline v3 hg_sample(pcg *g, v3 dir, float gg) {
    if (gg == 0.0f) return uniform_sphere(g);
    float u1 = pcg_float(g), u2 = pcg_float(g);
    float sq = (1.0f - gg * gg) / (1.0f - gg + 2.0f * gg * u1);
    float cost = (1.0f + gg * gg - sq * sq) / (2.0f * gg);
    if (cost < -1.0f) cost = -1.0f;
    if (cost > 1.0f) cost = 1.0f;
    float sint = sqrtf(fmaxf(0.0f, 1.0f - cost * cost));
    float phi = 2.0f * PI_F * u2;
    return normalize(rotate_to_world(sint * cosf(phi), sint * sinf(phi), cost, dir));
}

static inline float power_heuristic(float f, float g) {
    float a = 1.0f * f, b = 1.0f * g;
    return (a * a) / (a * a + b * b);
}

enum { LOBE_NULL = 0, LOBE_SREFL = 1, LOBE_STRANS = 2, LOBE_DIFFUSE = 4, LOBE_SPECULAR = 3 };

/* SurfaceInteraction, integrator/surface_interaction.h:14-30 */
typedef struct { v3 P, N, wi, wo; int lobe; float iori, ioro; v3 albedo; } inter;

/* BSDF Sample / Eval / Pdf, materials/bsdfs/{lambert_bsdf.h:26-38, mirror_bsdf.h:27-38,
 * ideal_specular_dielectric.h:31-68} */
static inline void bsdf_sample(const material *m, inter *it, pcg *g) {
    if (m->bsdf == ORC_BSDF_LAMBERT) {
        it->wi = cosine_hemisphere(it->N, g);
        it->lobe = LOBE_DIFFUSE;
    } else if (m->bsdf == ORC_BSDF_MIRROR) {
        it->wi = sub(muls(it->N, 2.0f * dot(it->wo, it->N)), it->wo);
        it->lobe = LOBE_SREFL;
    } else {
        float vdn = dot(it->wo, it->N);
        float ioro = m->ior;
        if (vdn < 0.0f) {
            ioro = 1.0f;
            it->N = neg(it->N);
            vdn = -vdn;
        }
        float eta = it->iori / ioro;
        float s2 = eta * eta * (1 - vdn * vdn);
        float F;
        if (s2 > 1.0f) {
            F = 1.0f;
        } else {
            float ct = sqrtf(1.0f - s2);
            float rperp = (it->iori * vdn - ioro * ct) / (it->iori * vdn + ioro * ct);
            float rpar = (ioro * vdn - it->iori * ct) / (ioro * vdn + it->iori * ct);
            F = 0.5f * (rperp * rperp + rpar * rpar);
        }
        float rnd = pcg_float(g);
        if (rnd <= F) {
            it->wi = sub(muls(it->N, 2.0f * dot(it->wo, it->N)), it->wo);
            it->lobe = LOBE_SREFL;
            it->ioro = it->iori;
        } else {
            it->wi = sub(muls(it->N, eta * vdn - sqrtf(1.0f - s2)), muls(it->wo, eta));
            it->lobe = LOBE_STRANS;
            it->ioro = ioro;
        }
    }
}

static inline v3 bsdf_eval(const material *m, const inter *it) {
    if (m->bsdf == ORC_BSDF_LAMBERT) return muls(muls(it->albedo, INV_PI_F), dot(it->wi, it->N));
    return it->albedo;
}
static inline float bsdf_pdf(const material *m, const inter *it) {
    if (m->bsdf == ORC_BSDF_LAMBERT) return dot(it->wi, it->N) * INV_PI_F;
    return 1.0f;
}

/* Scene::InterpolateNormal via rtcInterpolate1 (scene.cpp:123-132): the
 * barycentric blend (1-u-v)*n0 + u*n1 + v*n2, as the project rtc shim defines it */
static inline v3 interp_normal(const orc_scene *s, uint32_t prim, float u, float v) {
    const uint32_t *vi = s->tri_vidx + 3 * (size_t)prim;
    v3 n0 = ld3(s->vnormal + 3 * (size_t)vi[0]);
    v3 n1 = ld3(s->vnormal + 3 * (size_t)vi[1]);
    v3 n2 = ld3(s->vnormal + 3 * (size_t)vi[2]);
    float w = 1.0f - u - v;
    return add(add(muls(n0, w), muls(n1, u)), muls(n2, v));
}

/* The albedo texture at a hit. ConstantTexture; UVTexture (uv_texture.h:16-18):
 * (u, v, 0) of the texture coordinate rtcInterpolate1 gives on slot 1
 * (scene.cpp:134-143; (0, 0) without texture coordinates, integrator.cpp:184-188);
 * ImageTexture (image_texture.h:32-39) flips v and ImageCache::SampleImage
 * (image_cache.cpp:33-62) takes texel (round(u*W), round(v*H)), index
 * (y*W + x)*channels, value/256. The index is kept inside the image. */
static inline v3 material_albedo(const orc_scene *s, const material *m, const geom *G, uint32_t prim, float u,
                                 float v) {
    if (m->tex == -1) return m->albedo;
    float tu = 0.0f, tv = 0.0f;
    if (G->has_texcoords) {
        const uint32_t *vi = s->tri_vidx + 3 * (size_t)prim;
        float w = 1.0f - u - v;
        tu = s->vtex[2 * (size_t)vi[0]] * w + s->vtex[2 * (size_t)vi[1]] * u + s->vtex[2 * (size_t)vi[2]] * v;
        tv = s->vtex[2 * (size_t)vi[0] + 1] * w + s->vtex[2 * (size_t)vi[1] + 1] * u +
             s->vtex[2 * (size_t)vi[2] + 1] * v;
    }
    if (m->tex == -2) return mk(tu, tv, 0.0f);
    const image *I = &s->images[m->tex];
    tv = 1.0f - tv;
    float fx = fminf(fmaxf(roundf(tu * (float)I->w), 0.0f), 65536.0f);
    float fy = fminf(fmaxf(roundf(tv * (float)I->h), 0.0f), 65536.0f);
    uint64_t texel = (uint64_t)fy * I->w + (uint64_t)fx, last = (uint64_t)I->w * I->h - 1;
    if (texel > last) texel = last;
    const uint8_t *t = I->texels + texel * I->ch;
    float r = (float)t[0] / 256.0f;
    if (I->ch == 1) return mk(r, r, r);
    float gg = (float)t[1] / 256.0f;
    if (I->ch == 2) return mk(r, gg, 0.0f);
    return mk(r, gg, (float)t[2] / 256.0f);
}

int orc_add_image(orc_scene *s, const uint8_t *texels, uint32_t w, uint32_t h, uint32_t ch) {
    GROW(s->images, s->nimages, s->cimages, 1, image);
    image *I = &s->images[s->nimages];
    I->w = w;
    I->h = h;
    I->ch = ch;
    I->texels = (uint8_t *)malloc((size_t)w * h * ch);
    memcpy(I->texels, texels, (size_t)w * h * ch);
    return s->nimages++;
}

void orc_set_material_texture(orc_scene *s, int mat, int tex) { s->mats[mat].tex = tex; }

void orc_set_mesh_texcoords(orc_scene *s, int geom_id, const float *tc) {
    geom *g = &s->geoms[geom_id];
    memcpy(s->vtex + 2 * (size_t)g->vbase, tc, (size_t)g->nverts * 2 * sizeof(float));
    g->has_texcoords = 1;
}

typedef struct { uint64_t main, light, mis; } raystat;

/* AreaLight::SampleLi, scene/area_light.cpp:18-72 */
static v3 light_sample_li(const orc_scene *s, const light *L, pcg *g, inter *it, float *pdf,
                          raystat *rs) {
    float x, y;
    sample_disc(g, L->sphere[3], &x, &y);
    v3 cdir = sub(mk(L->sphere[0], L->sphere[1], L->sphere[2]), it->P);
    float dist = length(cdir);
    v3 cn = normalize(cdir);
    v3 point = rotate_to_world(x, y, dist - L->sphere[3], cn);
    v3 dir = normalize(point);
    it->wi = dir;
    if (dot(dir, it->N) <= 0.0f) {
        *pdf = 0.0f;
        return mk(0, 0, 0);
    }
    hitrec h;
    rs->light++;
    intersect1(s, it->P, dir, 0.001f, INFINITY, 1, &h, NULL);
    if (h.prim == 0xFFFFFFFFu || s->tri_geom[h.prim] != (uint32_t)L->geom) {
        *pdf = 0.0f;
        return mk(0, 0, 0);
    }
    v3 ip = add(it->P, muls(normalize(dir), h.t));
    v3 dd = sub(ip, it->P);
    float d2 = dot(dd, dd);
    *pdf = d2 / (fabsf(dot(normalize(interp_normal(s, h.prim, h.u, h.v)), neg(dir))) * L->area);
    return L->radiance;
}

/* AreaLight::PdfLi, area_light.cpp:74-110 */
static float light_pdf_li(const orc_scene *s, const light *L, const inter *it, raystat *rs) {
    if (dot(it->wi, it->N) <= 0.0f) return 0.0f;
    hitrec h;
    rs->mis++;
    intersect1(s, it->P, it->wi, 0.001f, INFINITY, 1, &h, NULL);
    if (h.prim == 0xFFFFFFFFu || s->tri_geom[h.prim] != (uint32_t)L->geom) return 0.0f;
    v3 ip = add(it->P, muls(normalize(it->wi), h.t));
    v3 dd = sub(ip, it->P);
    float d2 = dot(dd, dd);
    return d2 / (fabsf(dot(normalize(interp_normal(s, h.prim, h.u, h.v)), it->wi)) * L->area);
}

/* Integrator::EstimateDirect, integrator.cpp:273-315 */
static v3 estimate_direct(const orc_scene *s, const light *L, pcg *g, inter *it, const material *m,
                          raystat *rs) {
    v3 direct = mk(0, 0, 0);
    if (m->bsdf == ORC_BSDF_LAMBERT) { /* SupportedLobes & ~Specular */
        float lpdf;
        v3 Li = light_sample_li(s, L, g, it, &lpdf, rs);
        if (lpdf != 0.0f && !all_zero(Li)) {
            v3 f = bsdf_eval(m, it);
            float spdf = bsdf_pdf(m, it);
            if (spdf != 0.0f && !all_zero(f)) {
                float w = power_heuristic(lpdf, spdf);
                direct = add(direct, divs(muls(mul(f, Li), w), lpdf));
            }
        }
    }
    bsdf_sample(m, it, g);
    v3 f = bsdf_eval(m, it);
    float spdf = bsdf_pdf(m, it);
    if (spdf != 0.0f && !all_zero(f)) {
        float lpdf = light_pdf_li(s, L, it, rs);
        if (lpdf == 0.0f) return direct;
        float w = power_heuristic(spdf, lpdf);
        direct = add(direct, divs(muls(mul(f, L->radiance), w), spdf));
    }
    return direct;
}

/* Integrator::SampleOneLight + Scene::RandomOneLight, integrator.cpp:252-271,
 * scene.cpp:105-114. `it` is passed by value in the reference. */
static v3 sample_one_light(const orc_scene *s, pcg *g, inter it, const material *m, int hit_light,
                           raystat *rs) {
    uint32_t n = (uint32_t)s->nlights;
    if (n == 0 || (n == 1 && hit_light >= 0)) return mk(0, 0, 0);
    int li;
    do {
        li = (int)pcg_discrete(g, n);
    } while (li == hit_light);
    return muls(estimate_direct(s, &s->lights[li], g, &it, m, rs), (float)n);
}

/* Integrator::RenderPixel, integrator.cpp:98-250, with the two constants of the
 * loop (maxBounces at :114, the Russian-roulette threshold at :235) as options. */
static void render_pixel(const orc_scene *s, const orc_render_opts *o, uint32_t x, uint32_t y, pcg *g,
                         v3 *out_color, uint32_t *out_bounces, raystat *rs) {
    /* PinholeCamera::CalculateRayFromPixel, pinhole_camera.cpp:88-113 */
    v3 org = s->origin;
    float u = orc_filter_sample(pcg_float(g));
    float v = orc_filter_sample(pcg_float(g));
    v3 view = mk((((float)x + 0.5f + u) / (float)s->width * 2.0f - 1.0f) * s->tanx,
                 -(((float)y + 0.5f + v) / (float)s->height * 2.0f - 1.0f) * s->tany, -1.0f);
    v3 dir = mk(dot(view, s->mx), dot(view, s->my), dot(view, s->mz));
    float tnear = 0.0f;

    v3 color = mk(0, 0, 0), T = mk(1, 1, 1);
    inter it;
    memset(&it, 0, sizeof it);
    it.lobe = LOBE_NULL;
    it.iori = 1.0f;
    int med = -1;
    uint32_t bounces = 0;
    for (; bounces < o->max_depth; ++bounces) {
        hitrec h;
        rs->main++;
        intersect1(s, org, dir, tnear, INFINITY, 1, &h, NULL);
        if (h.prim == 0xFFFFFFFFu) {
            color = add(color, mul(T, s->background));
            break;
        }
        v3 origin = org;
        v3 direction = normalize(dir);
        int hit_surface = 1;
        if (med >= 0) {
            const medium *M = &s->meds[med];
            float dist;
            v3 trans;
            if (M->type == ORC_MED_NON_SCATTERING) {
                /* non_scattering_medium.h:20-39 */
                dist = h.t;
                trans = mk(expf(-M->sigma_a.x * dist), expf(-M->sigma_a.y * dist), expf(-M->sigma_a.z * dist));
                T = mul(muls(T, 1.0f), trans);
            } else if (M->type == ORC_MED_ISOTROPIC) {
                /* isotropic_scattering_medium.h:31-51: d = -ln(u)/sigma_s (scalar) */
                dist = -logf(pcg_float(g)) / M->sigma_s.x;
                if (dist >= h.t) dist = h.t;
                trans = mk(expf(-M->sigma_a.x * dist), expf(-M->sigma_a.y * dist), expf(-M->sigma_a.z * dist));
                T = mul(muls(T, 1.0f), trans);
            } else {
                /* RGB sigma_s extension: d sampled with the mean sigma_s; the
                 * per-channel ratio of transmittance (times sigma_s on scatter)
                 * to that pdf. Reduces to the isotropic medium for grey sigma_s. */
                float sbar = (M->sigma_s.x + M->sigma_s.y + M->sigma_s.z) / 3.0f;
                dist = -logf(pcg_float(g)) / sbar;
                int scat = dist < h.t;
                if (!scat) dist = h.t;
                v3 w;
                w.x = expf(-(M->sigma_a.x + M->sigma_s.x - sbar) * dist);
                w.y = expf(-(M->sigma_a.y + M->sigma_s.y - sbar) * dist);
                w.z = expf(-(M->sigma_a.z + M->sigma_s.z - sbar) * dist);
                if (scat) w = mul(w, divs(M->sigma_s, sbar));
                T = mul(T, w);
            }
            if (dist < h.t) {
                hit_surface = 0;
                org = add(origin, muls(direction, dist));
                dir = M->type == ORC_MED_HG ? hg_sample(g, direction, M->g) : uniform_sphere(g);
                tnear = 0.001f;
            }
        }
        if (hit_surface) {
            uint32_t gi = s->tri_geom[h.prim];
            const geom *G = &s->geoms[gi];
            const material *m = &s->mats[G->material];
            if ((bounces == 0 || (it.lobe & LOBE_SPECULAR) != 0) && G->light >= 0)
                color = add(color, mul(T, s->lights[G->light].radiance));
            it.P = add(origin, muls(direction, h.t));
            if (G->has_normals) it.N = normalize(interp_normal(s, h.prim, h.u, h.v));
            else it.N = normalize(mk(0, 0, 0));
            it.albedo = material_albedo(s, m, G, h.prim, h.u, h.v);
            it.wo = neg(direction);
            it.ioro = 0.0f;
            color = add(color, mul(T, sample_one_light(s, g, it, m, G->light, rs)));
            bsdf_sample(m, &it, g);
            float pdf = bsdf_pdf(m, &it);
            T = divs(mul(T, bsdf_eval(m, &it)), pdf);
            if (it.lobe == LOBE_STRANS) {
                it.iori = it.ioro;
                med = m->medium;
            }
            org = it.P;
            dir = it.wi;
            tnear = 0.001f;
        }
        if (bounces > o->rr_depth) {
            float p = fmaxf(T.x, fmaxf(T.y, T.z));
            if (pcg_float(g) > p) break;
            T = muls(T, 1 / p);
        }
    }
    *out_color = color;
    *out_bounces = bounces;
}

typedef struct {
    const orc_scene *s;
    const orc_render_opts *o;
    uint32_t frame;
    uint32_t tiles_x;
    float *rgb;
    uint32_t *bounces, *counts;
    raystat *stats; /* per work item */
} frame_ctx;

static void tile_job(void *c, uint64_t tile) {
    frame_ctx *f = (frame_ctx *)c;
    const orc_scene *s = f->s;
    uint32_t ty = (uint32_t)tile / f->tiles_x, tx = (uint32_t)tile - ty * f->tiles_x;
    uint32_t x0 = tx * 8, y0 = ty * 8;
    uint32_t x1 = x0 + 8 < s->width ? x0 + 8 : s->width;
    uint32_t y1 = y0 + 8 < s->height ? y0 + 8 : s->height;
    pcg g;
    pcg_init(&g, orc_tile_seed((uint32_t)tile, f->frame), f->frame);
    raystat rs = {0, 0, 0};
    for (uint32_t y = y0; y < y1; ++y)
        for (uint32_t x = x0; x < x1; ++x) {
            v3 c3;
            uint32_t b;
            render_pixel(s, f->o, x, y, &g, &c3, &b, &rs);
            size_t i = (size_t)y * s->width + x;
            f->rgb[3 * i] += c3.x;
            f->rgb[3 * i + 1] += c3.y;
            f->rgb[3 * i + 2] += c3.z;
            f->bounces[i] += b;
            f->counts[i] += 1u;
        }
    f->stats[tile] = rs;
}

/* pixel keying: seed = MurmurHash3(pixel index, frame), sequence = frame */
static void row_job(void *c, uint64_t row) {
    frame_ctx *f = (frame_ctx *)c;
    const orc_scene *s = f->s;
    raystat rs = {0, 0, 0};
    for (uint32_t x = 0; x < s->width; ++x) {
        uint32_t pix = (uint32_t)row * s->width + x;
        pcg g;
        pcg_init(&g, orc_tile_seed(pix, f->frame), f->frame);
        v3 c3;
        uint32_t b;
        render_pixel(s, f->o, x, (uint32_t)row, &g, &c3, &b, &rs);
        f->rgb[3 * (size_t)pix] += c3.x;
        f->rgb[3 * (size_t)pix + 1] += c3.y;
        f->rgb[3 * (size_t)pix + 2] += c3.z;
        f->bounces[pix] += b;
        f->counts[pix] += 1u;
    }
    f->stats[row] = rs;
}

void orc_render(const orc_scene *s, const orc_render_opts *o, uint32_t first, uint32_t nframes,
                float *rgb_a, uint32_t *b_a, uint32_t *c_a, float *rgb_b, uint32_t *b_b, uint32_t *c_b,
                uint64_t *ray_counts) {
    uint32_t tiles_x = (s->width + 7) / 8, tiles_y = (s->height + 7) / 8;
    uint64_t items = o->keying == LT_KEY_TILE ? (uint64_t)tiles_x * tiles_y : s->height;
    raystat *st = (raystat *)calloc(items, sizeof(raystat));
    if (ray_counts) ray_counts[0] = ray_counts[1] = ray_counts[2] = 0;
    for (uint32_t k = 0; k < nframes; ++k) {
        uint32_t frame = first + k;
        frame_ctx f = {s, o, frame, tiles_x, rgb_a, b_a, c_a, st};
        if (rgb_b && (k % 2 == 0)) { /* the first frame lands in the swap film */
            f.rgb = rgb_b; f.bounces = b_b; f.counts = c_b;
        }
        parallel_for(items, (int)o->threads, o->keying == LT_KEY_TILE ? tile_job : row_job, &f);
        if (ray_counts)
            for (uint64_t i = 0; i < items; ++i) {
                ray_counts[0] += st[i].main;
                ray_counts[1] += st[i].light;
                ray_counts[2] += st[i].mis;
            }
    }
    free(st);
}

void orc_render_path(const orc_scene *s, const orc_render_opts *o, uint32_t x, uint32_t y,
                     uint32_t frame, float color[3], uint32_t *bounces) {
    pcg g;
    pcg_init(&g, orc_tile_seed(y * s->width + x, frame), frame);
    raystat rs = {0, 0, 0};
    v3 c;
    render_pixel(s, o, x, y, &g, &c, bounces, &rs);
    color[0] = c.x; color[1] = c.y; color[2] = c.z;
}

void orc_camera_ray(const orc_scene *s, uint32_t x, uint32_t y, float u, float v, float out_dir[3],
                    float out_org[3]) {
    v3 view = mk((((float)x + 0.5f + u) / (float)s->width * 2.0f - 1.0f) * s->tanx,
                 -(((float)y + 0.5f + v) / (float)s->height * 2.0f - 1.0f) * s->tany, -1.0f);
    out_dir[0] = dot(view, s->mx);
    out_dir[1] = dot(view, s->my);
    out_dir[2] = dot(view, s->mz);
    out_org[0] = s->origin.x; out_org[1] = s->origin.y; out_org[2] = s->origin.z;
}

/* ------------------------------------------------------------------ accessors */
/* Read-only views of the loaded scene for the differentiable reference
 * (oracle/lt_diff_ref.cpp). */
void orc_camera_info(const orc_scene *s, float cam[14], uint32_t *w, uint32_t *h) {
    const v3 *v[4] = {&s->origin, &s->mx, &s->my, &s->mz};
    for (int i = 0; i < 4; ++i) {
        cam[3 * i] = v[i]->x; cam[3 * i + 1] = v[i]->y; cam[3 * i + 2] = v[i]->z;
    }
    cam[12] = s->tanx;
    cam[13] = s->tany;
    *w = s->width;
    *h = s->height;
}
void orc_background_info(const orc_scene *s, float rgb[3]) {
    rgb[0] = s->background.x; rgb[1] = s->background.y; rgb[2] = s->background.z;
}
int orc_num_lights(const orc_scene *s) { return s->nlights; }
int orc_num_media(const orc_scene *s) { return s->nmeds; }
int orc_light_geom(const orc_scene *s, int i) { return s->lights[i].geom; }
uint32_t orc_tri_geom(const orc_scene *s, uint32_t prim) { return s->tri_geom[prim]; }
void orc_geom_info(const orc_scene *s, uint32_t g, int *material, int *light, int *has_normals) {
    *material = s->geoms[g].material;
    *light = s->geoms[g].light;
    *has_normals = s->geoms[g].has_normals;
}
void orc_material_info(const orc_scene *s, int m, int *bsdf, float albedo[3], float *ior, int *medium) {
    const material *M = &s->mats[m];
    *bsdf = M->bsdf;
    albedo[0] = M->albedo.x; albedo[1] = M->albedo.y; albedo[2] = M->albedo.z;
    *ior = M->ior;
    *medium = M->medium;
}
void orc_medium_info(const orc_scene *s, int m, int *type, float sa[3], float ss[3], float *g) {
    const medium *M = &s->meds[m];
    *type = M->type;
    sa[0] = M->sigma_a.x; sa[1] = M->sigma_a.y; sa[2] = M->sigma_a.z;
    ss[0] = M->sigma_s.x; ss[1] = M->sigma_s.y; ss[2] = M->sigma_s.z;
    *g = M->g;
}
void orc_tri_normals(const orc_scene *s, uint32_t prim, float n[9]) {
    for (int j = 0; j < 3; ++j) {
        const float *p = s->vnormal + 3 * (size_t)s->tri_vidx[3 * (size_t)prim + j];
        n[3 * j] = p[0]; n[3 * j + 1] = p[1]; n[3 * j + 2] = p[2];
    }
}

/* ---------------------------------------------------------------- resolve */
/* visualizer.cpp:352-364 divides the colour sum by the count; the shader
 * (final_resolve_ps.glsl:24-43) scales by the exposure constant exp2f(stops)
 * (visualizer.cpp:1308) and tone maps. GLSL clamp(x, 0, 1) = min(max(x, 0), 1). */
static float clamp01f(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

static float filmicf(float c) {
    float x = fmaxf(0.0f, c - 0.004f);
    return clamp01f((x * (6.2f * x + 0.5f)) / (x * (6.2f * x + 1.7f) + 0.06f));
}

void orc_resolve(const float *rgb, const uint32_t *counts, uint64_t npix, int tonemap, float exposure_stops,
                 float *rgba, uint8_t *rgba8, uint32_t spp_minmax[2], uint64_t *spp_sum) {
    const float e = exp2f(exposure_stops);
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    uint64_t sum = 0;
    for (uint64_t i = 0; i < npix; ++i) {
        const float n = (float)counts[i];
        float c[4] = {e * (rgb[3 * i] / n), e * (rgb[3 * i + 1] / n), e * (rgb[3 * i + 2] / n), e * 1.0f};
        for (int k = 0; k < 4; ++k) c[k] = tonemap == 1 ? (k == 3 ? 1.0f : filmicf(c[k])) : clamp01f(c[k]);
        for (int k = 0; k < 4; ++k) {
            if (rgba) rgba[4 * i + k] = c[k];
            if (rgba8) rgba8[4 * i + k] = (uint8_t)lrintf(c[k] * 255.0f);
        }
        if (counts[i] < lo) lo = counts[i];
        if (counts[i] > hi) hi = counts[i];
        sum += counts[i];
    }
    if (spp_minmax) {
        spp_minmax[0] = lo;
        spp_minmax[1] = hi;
    }
    if (spp_sum) *spp_sum = sum;
}
