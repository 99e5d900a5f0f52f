// lt_kernels.cu -- sm_103a kernels of the wavefront path tracer.
//
// Stages per wavefront iteration (one path segment for every live path):
//   trace    closest hit of every queued path ray (rtcIntersect1, scene.cpp:116-121),
//            and in the same persistent launch the connection rays that the
//            previous shade emitted: occlusion query, area-light pdf and MIS
//            weight of SampleLi/PdfLi (area_light.cpp:18-110), film add
//   shade    one bounce of RenderPixel (integrator.cpp:116-243): background, medium
//            free flight, emission, light choice, BSDF sampling, roulette;
//            emits up to two connection rays; finished paths are added to the
//            film and their slot starts the next (pixel, frame) sample
//
// Queues are compacted with warp ballots and reserved once per block (one
// atomic per counter per block). Work items start in groups of one pixel's
// samples (sample_of_item), and each shade block writes its continuing paths
// grouped by the octant of their next direction, so that a trace warp holds
// rays that walk the same nodes. Every random number is drawn in shade, in the
// reference's order, so that a path's decisions do not depend on when its
// connection rays are traced. The differentiable estimator and its adjoint run
// on the same two stages (k_trace and k_dshade instantiated for their sources).
#include <cuda_runtime.h>

#include "lt_device.h"

namespace lt {

namespace {

constexpr int kStack = 64;
constexpr uint32_t kLobeNull = 0, kLobeSRefl = 1, kLobeSTrans = 2, kLobeDiffuse = 4, kLobeSpecular = 3;
constexpr uint32_t kConnectBsdf = 0x80000000u;
// Lights with at most this many triangles are tested triangle by triangle
// before a connection ray is traced.
constexpr uint32_t kLightBrute = 16;

__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

// The wavefront queues (path state, rays, hits, connection records) are read
// once by the next kernel and stream through L2 in far larger volume than it
// holds. Their loads and stores carry the streaming hint (evict first) so that
// the scene the traversal gathers from (nodes, triangles, normals) keeps its
// place in L2 from one kernel to the next.
template <class T>
__device__ __forceinline__ T ld_s(const T *p) { return __ldcs(p); }
template <class T>
__device__ __forceinline__ void st_s(T *p, T v) { __stcs(p, v); }

// ------------------------------------------------------------------ bound checks
// Compiled with -DLT_CHECKS=1 (liblantern_gpu_checked.so), the wavefront
// kernels check the indices they form against their arrays before each access:
// a failed check records its kind and the index in the wave counters (the
// first failure of a render wins), the access is skipped, and the render's
// later kernels return at once; the host reports LT_ERR_CHECK. Without
// LT_CHECKS, LT_CHECK is `true` and its condition is not compiled, so the plain
// kernels are unchanged. The kinds (CheckKind) and their names are in lt_device.h.
#ifndef LT_CHECKS
#define LT_CHECKS 0
#endif
#if LT_CHECKS
__device__ __noinline__ void check_failed(WaveCounters *wc, uint32_t kind, uint32_t value) {
    if (wc && atomicCAS(&wc->check, 0u, kind) == 0u) wc->check_value = value;
}
#define LT_CHECK(wc, cond, kind, value) ((cond) ? true : (check_failed((wc), (kind), (uint32_t)(value)), false))
// A whole block leaves a kernel of a render whose check failed (thread 0 reads
// the flag for the block, so that every thread takes the same branch).
#define LT_STOP_IF_FAILED(wc)                                                  \
    do {                                                                        \
        __shared__ uint32_t lt_stop_;                                           \
        if (threadIdx.x == 0) lt_stop_ = *(volatile uint32_t *)&(wc)->check;    \
        __syncthreads();                                                        \
        if (lt_stop_) return;                                                   \
    } while (0)
// a film pixel index: below the film's size, or below the test limit
// Wavefront::check_pixels when that is set and lower
#define LT_PIXEL_OK(W, pixel, npix)                                                                            \
    LT_CHECK((W).counters, (pixel) < ((W).check_pixels && (W).check_pixels < (npix) ? (W).check_pixels : (npix)), \
             kChkPixel, (pixel))
#else
#define LT_CHECK(wc, cond, kind, value) (sizeof(cond) > 0)  // not evaluated
#define LT_PIXEL_OK(W, pixel, npix) true
#define LT_STOP_IF_FAILED(wc) \
    do {                      \
    } while (0)
#endif

__device__ __forceinline__ float safe_inv(float d) {
    return 1.0f / (fabsf(d) > 1e-30f ? d : copysignf(1e-30f, d));
}

// Embree's dot for the triangle test: x*x + (y*y + z*z)
__device__ __forceinline__ float edot(v3 a, v3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }

__device__ __forceinline__ float xorsign(float a, uint32_t s) { return __uint_as_float(__float_as_uint(a) ^ s); }

struct Hit {
    float t, u, v;
    uint32_t prim;
};

// Moeller-Trumbore with Embree 3.5's acceptance rule
// (kernels/geometry/triangle_intersector_moeller.h:75-112): Ng = cross(e2, e1),
// |den| * tnear < T <= |den| * tfar; t, u, v by exact division.
__device__ __forceinline__ void tri_test(const float4 *tri, v3 O, v3 D, float tnear, Hit &h) {
    float4 a = ldg4(tri), b = ldg4(tri + 1), c = ldg4(tri + 2);
    v3 v0 = mk(a.x, a.y, a.z), e1 = mk(b.x, b.y, b.z), e2 = mk(c.x, c.y, c.z);
    v3 Ng = cross(e2, e1);
    v3 C = v0 - O;
    v3 R = cross(C, D);
    float den = edot(Ng, D);
    float absden = fabsf(den);
    uint32_t sgn = __float_as_uint(den) & 0x80000000u;
    float U = xorsign(edot(R, e2), sgn);
    float V = xorsign(edot(R, e1), sgn);
    if (den != 0.0f && U >= 0.0f && V >= 0.0f && U + V <= absden) {
        float T = xorsign(edot(Ng, C), sgn);
        if (absden * tnear < T && T <= absden * h.t) {
            h.t = __fdiv_rn(T, absden);
            h.u = __fdiv_rn(U, absden);
            h.v = __fdiv_rn(V, absden);
            h.prim = __float_as_uint(a.w);
        }
    }
}

// Conservative slab test of one child box (far distance widened by 2*gamma(3)).
__device__ __forceinline__ bool slab(float lox, float hix, float loy, float hiy, float loz, float hiz, v3 O,
                                     v3 inv, float tnear, float tfar, float &tentry) {
    float tx0 = (lox - O.x) * inv.x, tx1 = (hix - O.x) * inv.x;
    float ty0 = (loy - O.y) * inv.y, ty1 = (hiy - O.y) * inv.y;
    float tz0 = (loz - O.z) * inv.z, tz1 = (hiz - O.z) * inv.z;
    float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tnear));
    float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tfar));
    tentry = tmin;
    return tmin <= tmax * 1.0000004f;
}

// ------------------------------------------------------------------ traversal
// Persistent "while-while" traversal (Aila & Laine, "Understanding the
// efficiency of ray traversal on GPUs", HPG 2009): a warp walks inner nodes
// until every lane holds a leaf (one leaf per lane is postponed so that lanes
// keep descending), then all lanes test triangles together. A lane whose ray is
// done fetches the next one from a global counter; a warp leaves the loop early
// when fewer than kFetchThreshold lanes are still working so that idle lanes
// refill. Stack entries are node refs (inner >= 0, leaf < 0); the bottom entry
// is kSentinel. Box tests widen the far distance by 2*gamma(3) so no hit is lost.
constexpr int kSentinel = 0x76543210;
constexpr int kFetchThreshold = 20;

struct Trav {
    v3 O, D, inv;
    float tnear;
    Hit h;
    int node, leaf, sp;
    bool any;                // occlusion query: stop at the first hit not on `skip_geom`
    uint32_t skip_geom;
};

// Traversal stacks. LocalStack: a per-thread array (local memory). SharedStack:
// the first kSharedStack entries of every thread in the block's dynamic shared
// memory (column-interleaved, entry i of thread t at [i * blockDim + t], so a
// warp's accesses to one depth fall in distinct banks), deeper entries local.
#ifndef LT_SHARED_STACK
#define LT_SHARED_STACK 0
#endif
constexpr int kSharedStack = LT_SHARED_STACK;
extern __shared__ int lt_dyn_smem[];

struct LocalStack {
    int *a;
    __device__ __forceinline__ int get(int i) const { return a[i]; }
    __device__ __forceinline__ void set(int i, int v) { a[i] = v; }
};

struct SharedStack {
    int *loc;  // entries kSharedStack.. (local memory)
    __device__ __forceinline__ int get(int i) const {
        return i < kSharedStack ? lt_dyn_smem[i * blockDim.x + threadIdx.x] : loc[i - kSharedStack];
    }
    __device__ __forceinline__ void set(int i, int v) {
        if (i < kSharedStack) lt_dyn_smem[i * blockDim.x + threadIdx.x] = v;
        else loc[i - kSharedStack] = v;
    }
};

template <class St>
__device__ __forceinline__ void trav_start(Trav &r, St stack, v3 O, v3 D, float tnear, float tfar, bool any,
                                           uint32_t skip_geom) {
    r.O = O;
    r.D = D;
    r.inv = mk(safe_inv(D.x), safe_inv(D.y), safe_inv(D.z));
    r.tnear = tnear;
    r.h.t = tfar;
    r.h.u = r.h.v = 0.0f;
    r.h.prim = kMiss;
    r.node = 0;
    r.leaf = 0;
    r.sp = 0;
    stack.set(0, kSentinel);
    r.any = any;
    r.skip_geom = skip_geom;
}

// The arrays one traversal reads: nodes, leaf-ordered triangles, triangle -> mesh.
struct Geo {
    const float4 *nodes, *tris;
    const uint32_t *tri_geom;
    uint32_t num_nodes, num_tris;  // bounds of the node and triangle indices
#if LT_CHECKS
    WaveCounters *chk = nullptr;  // where a failed bound check is recorded
#endif
};

__device__ __forceinline__ Geo geo_of(const DevScene &S) {
    return Geo{S.nodes, S.tris, S.tri_geom, S.num_nodes, S.num_tris};
}

#if LT_CHECKS
#define LT_GEO_CHK(g) ((g).chk)
#define LT_SET_GEO_CHK(g, wc) ((g).chk = (wc))
#else
#define LT_GEO_CHK(g) nullptr
#define LT_SET_GEO_CHK(g, wc) ((void)0)
#endif

// Checked stack pop of the BVH2 / 4-wide traversals: a failed check ends the ray.
#define LT_TRAV_POP(S, r, stack)                                               \
    do {                                                                        \
        if (LT_CHECK(LT_GEO_CHK(S), (r).sp >= 0, kChkStack, (r).sp)) {          \
            (r).node = (stack).get((r).sp--);                                   \
        } else {                                                                \
            (r).node = kSentinel;                                               \
            (r).leaf = 0;                                                       \
        }                                                                       \
    } while (0)

// Advances the ray until it is finished (r.node == kSentinel) or the warp
// should refill idle lanes.
template <class St>
__device__ __forceinline__ void traverse(const Geo &S, Trav &r, St stack) {
    while (r.node != kSentinel) {
        while ((unsigned)r.node < (unsigned)kSentinel) {
            if (!LT_CHECK(LT_GEO_CHK(S), (uint32_t)r.node < S.num_nodes, kChkNode, r.node)) {
                r.node = kSentinel;
                r.leaf = 0;
                return;
            }
            const float4 *n = S.nodes + 4 * r.node;
            float4 n0 = ldg4(n), n1 = ldg4(n + 1), n2 = ldg4(n + 2), n3 = ldg4(n + 3);
            float t0, t1;
            bool h0 = slab(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, r.O, r.inv, r.tnear, r.h.t, t0);
            bool h1 = slab(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, r.O, r.inv, r.tnear, r.h.t, t1);
            int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
            if (!h0 && !h1) {
                LT_TRAV_POP(S, r, stack);
            } else {
                r.node = h0 ? c0 : c1;
                if (h0 && h1) {
                    int far = c1;
                    if (t1 < t0) { far = c0; r.node = c1; }
                    if (LT_CHECK(LT_GEO_CHK(S), r.sp + 1 < kStack, kChkStack, r.sp + 1)) {
                        stack.set(++r.sp, far);
                    } else {
                        r.node = kSentinel;
                        r.leaf = 0;
                        return;
                    }
                }
            }
            if (r.node < 0 && r.leaf >= 0) {  // postpone the first leaf, keep descending
                r.leaf = r.node;
                LT_TRAV_POP(S, r, stack);
            }
            if (!__any_sync(__activemask(), r.leaf >= 0)) break;
        }
        while (r.leaf < 0) {
            uint32_t code = ~(uint32_t)r.leaf;
            uint32_t first = code >> kLeafBits, count = code & ((1u << kLeafBits) - 1u);
            if (!LT_CHECK(LT_GEO_CHK(S), first + count <= S.num_tris, kChkLeaf, first)) {
                r.node = kSentinel;
                r.leaf = 0;
                return;
            }
            for (uint32_t k = 0; k < count; ++k) {
                const float4 *tri = S.tris + 3 * (first + k);
                if (!r.any) {
                    tri_test(tri, r.O, r.D, r.tnear, r.h);
                } else {
                    Hit c = r.h;
                    tri_test(tri, r.O, r.D, r.tnear, c);
                    if (c.prim != kMiss && !LT_CHECK(LT_GEO_CHK(S), c.prim < S.num_tris, kChkPrim, c.prim)) {
                        r.node = kSentinel;
                        r.leaf = 0;
                        return;
                    }
                    if (c.prim != kMiss && __ldg(S.tri_geom + c.prim) != r.skip_geom) {
                        r.h.prim = c.prim;  // occluded
                        r.node = kSentinel;
                        r.leaf = 0;
                        return;
                    }
                }
            }
            r.leaf = r.node;
            if (r.node < 0) LT_TRAV_POP(S, r, stack);
        }
        if (__popc(__activemask()) < kFetchThreshold) return;
    }
}

// ------------------------------------------------------------------ 4-wide traversal
// 4-wide BVH (Bvh4Node, lt_scene.h: the children of a BVH2 node with its inner
// children opened), traversed by the while-while loop above: a node's child
// boxes are tested together, the children hit are taken nearest first (the
// others stacked, farthest deepest), leaves are the BVH2's.
__device__ __forceinline__ void cswap(float &ta, int &ca, float &tb, int &cb) {
    if (tb < ta) {
        const float t = ta;
        ta = tb;
        tb = t;
        const int c = ca;
        ca = cb;
        cb = c;
    }
}

template <class St>
__device__ __forceinline__ void traverse4(const Geo &S, Trav &r, St stack) {
    const float kInf = __int_as_float(0x7f800000);
    while (r.node != kSentinel) {
        while ((unsigned)r.node < (unsigned)kSentinel) {
            if (!LT_CHECK(LT_GEO_CHK(S), (uint32_t)r.node < S.num_nodes, kChkNode, r.node)) {
                r.node = kSentinel;
                r.leaf = 0;
                return;
            }
            const float4 *n = S.nodes + 8 * (size_t)r.node;
            const float4 lx = ldg4(n), hx = ldg4(n + 1), ly = ldg4(n + 2), hy = ldg4(n + 3), lz = ldg4(n + 4),
                         hz = ldg4(n + 5), rf = ldg4(n + 6);
            int c0 = __float_as_int(rf.x), c1 = __float_as_int(rf.y), c2 = __float_as_int(rf.z),
                c3 = __float_as_int(rf.w);
            float t0, t1, t2, t3;
            const bool b0 = slab(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, r.O, r.inv, r.tnear, r.h.t, t0) && c0 != kEmptyRef4;
            const bool b1 = slab(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, r.O, r.inv, r.tnear, r.h.t, t1) && c1 != kEmptyRef4;
            const bool b2 = slab(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, r.O, r.inv, r.tnear, r.h.t, t2) && c2 != kEmptyRef4;
            const bool b3 = slab(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, r.O, r.inv, r.tnear, r.h.t, t3) && c3 != kEmptyRef4;
            const int nh = (int)b0 + (int)b1 + (int)b2 + (int)b3;
            if (nh == 0) {
                LT_TRAV_POP(S, r, stack);
            } else {
                if (!b0) t0 = kInf;
                if (!b1) t1 = kInf;
                if (!b2) t2 = kInf;
                if (!b3) t3 = kInf;
                cswap(t0, c0, t1, c1);  // sorting network, nearest first
                cswap(t2, c2, t3, c3);
                cswap(t0, c0, t2, c2);
                cswap(t1, c1, t3, c3);
                cswap(t1, c1, t2, c2);
                if (!LT_CHECK(LT_GEO_CHK(S), r.sp + nh - 1 < kStack, kChkStack, r.sp + nh - 1)) {
                    r.node = kSentinel;
                    r.leaf = 0;
                    return;
                }
                if (nh > 3) stack.set(++r.sp, c3);
                if (nh > 2) stack.set(++r.sp, c2);
                if (nh > 1) stack.set(++r.sp, c1);
                r.node = c0;
            }
            if (r.node < 0 && r.leaf >= 0) {  // postpone the first leaf, keep descending
                r.leaf = r.node;
                LT_TRAV_POP(S, r, stack);
            }
            if (!__any_sync(__activemask(), r.leaf >= 0)) break;
        }
        while (r.leaf < 0) {
            const uint32_t code = ~(uint32_t)r.leaf;
            const uint32_t first = code >> kLeafBits, count = code & ((1u << kLeafBits) - 1u);
            if (!LT_CHECK(LT_GEO_CHK(S), first + count <= S.num_tris, kChkLeaf, first)) {
                r.node = kSentinel;
                r.leaf = 0;
                return;
            }
            for (uint32_t k = 0; k < count; ++k) {
                const float4 *tri = S.tris + 3 * (first + k);
                if (!r.any) {
                    tri_test(tri, r.O, r.D, r.tnear, r.h);
                } else {
                    Hit c = r.h;
                    tri_test(tri, r.O, r.D, r.tnear, c);
                    if (c.prim != kMiss && !LT_CHECK(LT_GEO_CHK(S), c.prim < S.num_tris, kChkPrim, c.prim)) {
                        r.node = kSentinel;
                        r.leaf = 0;
                        return;
                    }
                    if (c.prim != kMiss && __ldg(S.tri_geom + c.prim) != r.skip_geom) {
                        r.h.prim = c.prim;  // occluded
                        r.node = kSentinel;
                        r.leaf = 0;
                        return;
                    }
                }
            }
            r.leaf = r.node;
            if (r.node < 0) LT_TRAV_POP(S, r, stack);
        }
        if (__popc(__activemask()) < kFetchThreshold) return;
    }
}

// ------------------------------------------------------------------ 8-wide traversal
// Compressed 8-wide BVH (Bvh8Node, lt_scene.h), traversed as in Ylitie,
// Karras and Laine (HPG 2017): the ray keeps a node group -- the children of
// one visited node that its box tests hit, as a base index and a hit mask --
// and a triangle group (base triangle index, 24-bit hit mask); the rest waits
// on a stack of such groups. Inner-child hits sit in bits 24-31 at position
// 24 + (slot ^ octant), so taking the highest bit first visits the children
// roughly front to back. Triangle groups are postponed (pushed) while fewer
// than a fifth of the warp's active lanes have triangles to test and the lane
// still has nodes to visit. Box planes are p + q * cell, the float expression
// the builder checked to enclose each child.
constexpr int kStack8 = 64;  // groups; the builder keeps 2 * depth + 2 within it

struct Trav8 {
    v3 O, D, inv;
    float tnear;
    Hit h;
    bool any;
    uint32_t skip_geom;
    uint32_t oct;    // bit c: D[c] < 0
    uint2 ngroup;    // (base child, hits << 24 | imask)
    uint2 tgroup;    // (base triangle, hits in bits 0-23)
    int sp;
    bool done;
};

__device__ __forceinline__ void trav8_start(Trav8 &r, v3 O, v3 D, float tnear, float tfar, bool any,
                                            uint32_t skip_geom) {
    r.O = O;
    r.D = D;
    r.inv = mk(safe_inv(D.x), safe_inv(D.y), safe_inv(D.z));
    r.tnear = tnear;
    r.h.t = tfar;
    r.h.u = r.h.v = 0.0f;
    r.h.prim = kMiss;
    r.any = any;
    r.skip_geom = skip_geom;
    r.oct = (D.x < 0.0f ? 1u : 0u) | (D.y < 0.0f ? 2u : 0u) | (D.z < 0.0f ? 4u : 0u);
    r.ngroup = make_uint2(0u, (1u << (24u + r.oct)) | 1u);  // the root: node 0 in slot 0
    r.tgroup = make_uint2(0u, 0u);
    r.sp = 0;
    r.done = false;
}

// float(byte k of w), exactly: the byte placed under the exponent of 2^23 by
// one byte permute, minus 2^23 (avoids the slower integer-to-float conversion).
__device__ __forceinline__ float byte_f(uint32_t w, uint32_t k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | k)) - 8388608.0f;
}

// Box tests of the 8 children of node `idx`; returns the hit mask (inner
// children in bits 24-31, leaf triangles in bits 0-23) and the node's bases.
__device__ __forceinline__ uint32_t node8_hits(const float4 *nodes, uint32_t idx, const Trav8 &r,
                                               uint32_t &base_child, uint32_t &base_tri, uint32_t &imask) {
    const float4 *n = nodes + 5 * (size_t)idx;
    const float4 w0 = ldg4(n), w1 = ldg4(n + 1), w2 = ldg4(n + 2), w3 = ldg4(n + 3), w4 = ldg4(n + 4);
    const uint32_t eb = __float_as_uint(w0.w);
    imask = eb >> 24;
    base_child = __float_as_uint(w1.x);
    base_tri = __float_as_uint(w1.y);
    const float cx = __uint_as_float((eb & 0xFFu) << 23), cy = __uint_as_float(((eb >> 8) & 0xFFu) << 23),
                cz = __uint_as_float(((eb >> 16) & 0xFFu) << 23);
    // t of plane p + q * cell along each axis: q * (cell * inv) + (p - O) * inv
    const float sx = cx * r.inv.x, sy = cy * r.inv.y, sz = cz * r.inv.z;
    const float ox = (w0.x - r.O.x) * r.inv.x, oy = (w0.y - r.O.y) * r.inv.y, oz = (w0.z - r.O.z) * r.inv.z;
    // near / far plane words per axis from the direction signs
    const bool nx = r.inv.x < 0.0f, ny = r.inv.y < 0.0f, nz = r.inv.z < 0.0f;
    const uint32_t lx0 = __float_as_uint(w2.x), lx1 = __float_as_uint(w2.y), ly0 = __float_as_uint(w2.z),
                   ly1 = __float_as_uint(w2.w), lz0 = __float_as_uint(w3.x), lz1 = __float_as_uint(w3.y),
                   hx0 = __float_as_uint(w3.z), hx1 = __float_as_uint(w3.w), hy0 = __float_as_uint(w4.x),
                   hy1 = __float_as_uint(w4.y), hz0 = __float_as_uint(w4.z), hz1 = __float_as_uint(w4.w);
    const uint32_t nx0 = nx ? hx0 : lx0, nx1 = nx ? hx1 : lx1, fx0 = nx ? lx0 : hx0, fx1 = nx ? lx1 : hx1;
    const uint32_t ny0 = ny ? hy0 : ly0, ny1 = ny ? hy1 : ly1, fy0 = ny ? ly0 : hy0, fy1 = ny ? ly1 : hy1;
    const uint32_t nz0 = nz ? hz0 : lz0, nz1 = nz ? hz1 : lz1, fz0 = nz ? lz0 : hz0, fz1 = nz ? lz1 : hz1;
    const uint32_t meta0 = __float_as_uint(w1.z), meta1 = __float_as_uint(w1.w);
    uint32_t hits = 0;
#pragma unroll
    for (uint32_t s = 0; s < 8; ++s) {
        const uint32_t k = s & 3u;
        const uint32_t meta = ((s < 4 ? meta0 : meta1) >> (8u * k)) & 0xFFu;
        const float tx0 = fmaf(byte_f(s < 4 ? nx0 : nx1, k), sx, ox), tx1 = fmaf(byte_f(s < 4 ? fx0 : fx1, k), sx, ox);
        const float ty0 = fmaf(byte_f(s < 4 ? ny0 : ny1, k), sy, oy), ty1 = fmaf(byte_f(s < 4 ? fy0 : fy1, k), sy, oy);
        const float tz0 = fmaf(byte_f(s < 4 ? nz0 : nz1, k), sz, oz), tz1 = fmaf(byte_f(s < 4 ? fz0 : fz1, k), sz, oz);
        const float tmin = fmaxf(fmaxf(tx0, ty0), fmaxf(tz0, r.tnear));
        const float tmax = fminf(fminf(tx1, ty1), fminf(tz1, r.h.t));
        if (meta != 0u && tmin <= tmax * 1.0000004f) {
            if (imask & (1u << s)) hits |= 1u << (24u + (s ^ r.oct));
            else hits |= (meta >> 5) << (meta & 31u);
        }
    }
    return hits;
}

__device__ __forceinline__ void traverse8(const Geo &g, Trav8 &r, uint2 *stack) {
    while (!r.done) {
        if (r.ngroup.y > 0x00FFFFFFu) {
            // next inner child of the node group
            const uint32_t b = 31u - __clz(r.ngroup.y);
            const uint32_t slot = (b - 24u) ^ r.oct;
            const uint32_t imask = r.ngroup.y & 0xFFu;
            const uint32_t idx = r.ngroup.x + __popc(imask & ((1u << slot) - 1u));
            r.ngroup.y &= ~(1u << b);
            if (r.ngroup.y > 0x00FFFFFFu && r.sp < kStack8) stack[r.sp++] = r.ngroup;
            if (idx < g.num_nodes) {
                uint32_t bc, bt, im;
                const uint32_t hits = node8_hits(g.nodes, idx, r, bc, bt, im);
                r.ngroup = make_uint2(bc, (hits & 0xFF000000u) | im);
                r.tgroup = make_uint2(bt, hits & 0x00FFFFFFu);
            } else {  // malformed tree: skip the subtree rather than read out of bounds
                r.ngroup = make_uint2(0u, 0u);
                r.tgroup = make_uint2(0u, 0u);
            }
        } else {
            r.tgroup = r.ngroup;  // a triangle group from the stack (or nothing)
            r.ngroup = make_uint2(0u, 0u);
        }
        // triangles, unless too few lanes have some and this lane can visit nodes instead
        {
            const unsigned act = __activemask();
            const unsigned want = __ballot_sync(act, r.tgroup.y != 0u);
            if (r.tgroup.y != 0u && r.ngroup.y > 0x00FFFFFFu && 5 * __popc(want) < __popc(act) &&
                r.sp < kStack8) {
                stack[r.sp++] = r.tgroup;
                r.tgroup.y = 0u;
            }
        }
        while (r.tgroup.y != 0u) {
            const uint32_t t = __ffs(r.tgroup.y) - 1u;
            r.tgroup.y &= r.tgroup.y - 1u;
            if (r.tgroup.x + t >= g.num_tris) continue;
            const float4 *tri = g.tris + 3 * (size_t)(r.tgroup.x + t);
            if (!r.any) {
                tri_test(tri, r.O, r.D, r.tnear, r.h);
            } else {
                Hit c = r.h;
                tri_test(tri, r.O, r.D, r.tnear, c);
                if (c.prim != kMiss && __ldg(g.tri_geom + c.prim) != r.skip_geom) {
                    r.h.prim = c.prim;  // occluded
                    r.done = true;
                    return;
                }
            }
        }
        if (r.ngroup.y <= 0x00FFFFFFu) {
            if (r.sp == 0) {
                r.done = true;
                return;
            }
            r.ngroup = stack[--r.sp];
        }
        if (__popc(__activemask()) < kFetchThreshold) return;
    }
}

// Traversal policies: the BVH2 (while-while, Trav) and the compressed 8-wide BVH (Trav8).
struct Bvh2 {
    using State = Trav;
    using Entry = int;
    static constexpr int kDepth = kStack - kSharedStack;  // local entries
    static constexpr int kSharedBytesPerThread = 4 * kSharedStack;
    // k_trace<OneScene> register budget: 5 x 256 threads per SM (at most 51
    // registers), measured 1.3% faster than the compiler's own choice of 51
    // (the batched instantiation keeps the compiler's choice: it spilled)
    static constexpr int kMinBlocks256 = 5;
    __device__ static Geo geo(const DevScene &S) { return geo_of(S); }
    __device__ static void start(State &r, Entry *st, v3 O, v3 D, float tnear, float tfar, bool any, uint32_t skip) {
        if (kSharedStack) trav_start(r, SharedStack{st}, O, D, tnear, tfar, any, skip);
        else trav_start(r, LocalStack{st}, O, D, tnear, tfar, any, skip);
    }
    __device__ static void run(const Geo &g, State &r, Entry *st) {
        if (kSharedStack) traverse(g, r, SharedStack{st});
        else traverse(g, r, LocalStack{st});
    }
    __device__ static bool done(const State &r) { return r.node == kSentinel; }
    __device__ static void idle(State &r) { r.node = kSentinel; }
};

struct Bvh4 {
    using State = Trav;
    using Entry = int;
    static constexpr int kDepth = kStack;
    static constexpr int kSharedBytesPerThread = 0;
    static constexpr int kMinBlocks256 = 0;  // k_trace register budget: compiler's choice
    __device__ static Geo geo(const DevScene &S) { return Geo{S.nodes4, S.tris, S.tri_geom, S.num_nodes4, S.num_tris}; }
    __device__ static void start(State &r, Entry *st, v3 O, v3 D, float tnear, float tfar, bool any, uint32_t skip) {
        trav_start(r, LocalStack{st}, O, D, tnear, tfar, any, skip);
    }
    __device__ static void run(const Geo &g, State &r, Entry *st) { traverse4(g, r, LocalStack{st}); }
    __device__ static bool done(const State &r) { return r.node == kSentinel; }
    __device__ static void idle(State &r) { r.node = kSentinel; }
};

struct Bvh8 {
    using State = Trav8;
    using Entry = uint2;
    static constexpr int kDepth = kStack8;
    static constexpr int kSharedBytesPerThread = 0;
    static constexpr int kMinBlocks256 = 0;  // k_trace register budget: 0 = no minimum (compiler's choice)
    __device__ static Geo geo(const DevScene &S) {
        return Geo{S.nodes8, S.tris8, S.tri_geom, S.num_nodes8, S.num_tris};
    }
    __device__ static void start(State &r, Entry *, v3 O, v3 D, float tnear, float tfar, bool any, uint32_t skip) {
        trav8_start(r, O, D, tnear, tfar, any, skip);
    }
    __device__ static void run(const Geo &g, State &r, Entry *st) { traverse8(g, r, st); }
    __device__ static bool done(const State &r) { return r.done; }
    __device__ static void idle(State &r) { r.done = true; }
};

// Warp-aggregated fetch of the next work index for the lanes that ask.
__device__ __forceinline__ uint32_t fetch_next(uint32_t *counter) {
    unsigned m = __activemask();
    int leader = __ffs(m) - 1;
    uint32_t lane = threadIdx.x & 31u, base = 0;
    if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ v3 interp_normal(const DevScene &S, uint32_t prim, float u, float v) {
    uint32_t i0 = __ldg(S.tri_vidx + 3 * prim), i1 = __ldg(S.tri_vidx + 3 * prim + 1),
             i2 = __ldg(S.tri_vidx + 3 * prim + 2);
    v3 n0 = mk(__ldg(S.vnormal + 3 * i0), __ldg(S.vnormal + 3 * i0 + 1), __ldg(S.vnormal + 3 * i0 + 2));
    v3 n1 = mk(__ldg(S.vnormal + 3 * i1), __ldg(S.vnormal + 3 * i1 + 1), __ldg(S.vnormal + 3 * i1 + 2));
    v3 n2 = mk(__ldg(S.vnormal + 3 * i2), __ldg(S.vnormal + 3 * i2 + 1), __ldg(S.vnormal + 3 * i2 + 2));
    float w = 1.0f - u - v;
    return (n0 * w + n1 * u) + n2 * v;
}

// Albedo texture at a hit (BSDF::Eval's m_albedoTexture->Sample): constant;
// UVTexture (uv_texture.h:16-18): (u, v, 0) of the interpolated texture
// coordinate; ImageTexture (image_texture.h:32-39, image_cache.cpp:33-62): v
// flipped, nearest texel at (round(u * W), round(v * H)), 8-bit value / 256,
// grey -> (g, g, g), two channels -> (r, g, 0). The texel index is
// (y * W + x) * channels as the reference computes it (x == W reads the next
// row's first texel), kept inside the image. A mesh without texture
// coordinates samples (0, 0) (integrator.cpp:184-188).
__device__ __forceinline__ v3 material_albedo(const DevScene &S, const MaterialInfo &m, const GeomInfo &G,
                                              uint32_t prim, float u, float v) {
    if (m.tex == kAlbedoConstant) return mk(m.albedo[0], m.albedo[1], m.albedo[2]);
    float tu = 0.0f, tv = 0.0f;
    if (G.has_texcoords) {
        const uint32_t i0 = __ldg(S.tri_vidx + 3 * prim), i1 = __ldg(S.tri_vidx + 3 * prim + 1),
                       i2 = __ldg(S.tri_vidx + 3 * prim + 2);
        const float w = 1.0f - u - v;
        tu = (__ldg(S.vtex + 2 * i0) * w + __ldg(S.vtex + 2 * i1) * u) + __ldg(S.vtex + 2 * i2) * v;
        tv = (__ldg(S.vtex + 2 * i0 + 1) * w + __ldg(S.vtex + 2 * i1 + 1) * u) + __ldg(S.vtex + 2 * i2 + 1) * v;
    }
    if (m.tex == kAlbedoUV) return mk(tu, tv, 0.0f);
    const ImageInfo I = S.images[m.tex];
    tv = 1.0f - tv;
    const float fx = fminf(fmaxf(roundf(tu * (float)I.width), 0.0f), 65536.0f);
    const float fy = fminf(fmaxf(roundf(tv * (float)I.height), 0.0f), 65536.0f);
    uint64_t texel = (uint64_t)fy * I.width + (uint64_t)fx;
    const uint64_t last = (uint64_t)I.width * I.height - 1;
    if (texel > last) texel = last;
    const uint8_t *t = S.texels + I.offset + texel * I.channels;
    const float r = (float)__ldg(t) / 256.0f;
    if (I.channels == 1) return mk(r, r, r);
    const float g = (float)__ldg(t + 1) / 256.0f;
    if (I.channels == 2) return mk(r, g, 0.0f);
    return mk(r, g, (float)__ldg(t + 2) / 256.0f);
}

// Distance to the closest of the light's own triangles along (org, dir), t in
// (0.001, inf): 0 when the ray misses the light, -1 when the light has more
// than kLightBrute triangles and was not tested. `out` (optional) gets the hit.
__device__ __forceinline__ float light_distance(const DevScene &S, const LightInfo &L, v3 org, v3 dir, Hit *out) {
    if (L.tri_count > kLightBrute) return -1.0f;
    Hit lh;
    lh.t = __int_as_float(0x7f800000);
    lh.u = lh.v = 0.0f;
    lh.prim = kMiss;
    for (uint32_t k = 0; k < L.tri_count; ++k) tri_test(S.light_tris + 3 * (L.tri_first + k), org, dir, 0.001f, lh);
    if (out) *out = lh;
    return lh.prim == kMiss ? 0.0f : lh.t;
}

// A path queue holds the paths that continue (entries 0 .. n_push - 1, in the
// order their warps enqueued them) and, apart from them at the top of the
// arrays, the paths that start with a camera ray (slots cap - n_cam .. cap - 1),
// so that camera rays of the same pixel fill warps of their own. Entry q of
// the queue lives in slot:
__device__ __forceinline__ uint32_t queue_slot(uint32_t q, uint32_t n_push, uint32_t n_cam, uint32_t cap) {
    return q < n_push ? q : cap - n_cam + (q - n_push);
}

struct Path {
    Pcg rng;
    uint32_t pixel, frame;
    v3 T;
    uint32_t bounces, lobe;
    int medium;
    float iori;
    uint32_t scene;  // slot of a batched render, 0 otherwise
};

// Path flags: bits 0-7 sampled lobe, 8-20 medium index + 1, 21-31 scene slot.
constexpr uint32_t kFlagMediumShift = 8, kFlagMediumMask = 0x1FFFu, kFlagSceneShift = 21;
// A path that starts with its camera ray: throughput 1, no bounce, IOR 1, no
// lobe, no medium; only its sampler, pixel, frame and flags are stored.
constexpr uint32_t kFlagFresh = 0x80u;
// Connection record word: bits 0-19 light index, 20-30 scene slot, bit 31 BSDF sample.
constexpr uint32_t kConnLightMask = 0xFFFFFu, kConnSceneShift = 20, kConnSceneMask = 0x7FFu;
static_assert(kMaxBatchScenes <= kConnSceneMask + 1 && kMaxBatchScenes <= (1u << (32 - kFlagSceneShift)),
              "scene slot field too narrow");
static_assert(kMaxLights <= kConnLightMask + 1 && kMaxMedia < kFlagMediumMask, "light / medium field too narrow");

// Start sample `item`: PinholeCamera::CalculateRayFromPixel (pinhole_camera.cpp:88-113)
// with the sampler of (pixel, frame).
__device__ __forceinline__ void start_path(const DevScene &S, const RenderArgs &a, unsigned long long item, Path &p,
                                           v3 &org, v3 &dir, float &tnear) {
    const uint32_t npix = a.width * a.height;
    uint32_t fo;
    if (item >> 32 == 0) {  // 32-bit division when the item index fits (the same quotient)
        fo = (uint32_t)item / npix;
        p.pixel = (uint32_t)item - fo * npix;
    } else {
        fo = (uint32_t)(item / npix);
        p.pixel = (uint32_t)(item - (unsigned long long)fo * npix);
    }
    p.frame = a.first_frame + fo;
    const uint32_t y = p.pixel / a.width, x = p.pixel - y * a.width;
    p.rng = sampler_for(p.pixel, p.frame);
    float u = tent_sample(S.filter, p.rng.next_float());
    float v = tent_sample(S.filter, p.rng.next_float());
    dir = camera_dir(S.cam, x, y, u, v);
    org = S.cam.origin;
    tnear = 0.0f;
    p.T = mk(1.0f, 1.0f, 1.0f);
    p.bounces = 0;
    p.lobe = kLobeNull;
    p.medium = -1;
    p.iori = 1.0f;
    p.scene = 0;
}

__device__ __forceinline__ void store_path(const PathState &ps, uint32_t cap, uint32_t slot, const Path &p) {
    st_s(ps.rng + slot, (uint64_t)p.rng.state);
    st_s(ps.pixel + slot, p.pixel);
    st_s(ps.frame + slot, p.frame);
    st_s(ps.T + slot, p.T.x);
    st_s(ps.T + cap + slot, p.T.y);
    st_s(ps.T + 2 * cap + slot, p.T.z);
    st_s(ps.bounces + slot, p.bounces);
    st_s(ps.flags + slot, p.lobe | ((uint32_t)(p.medium + 1) << kFlagMediumShift) | (p.scene << kFlagSceneShift));
    st_s(ps.iori + slot, p.iori);
}

// A fresh path (a camera ray's): the state start_path gives, with only the
// sampler, pixel, frame and flags stored.
__device__ __forceinline__ void store_fresh_path(const PathState &ps, uint32_t slot, const Path &p) {
    st_s(ps.rng + slot, (uint64_t)p.rng.state);
    st_s(ps.pixel + slot, p.pixel);
    st_s(ps.frame + slot, p.frame);
    st_s(ps.flags + slot, kLobeNull | kFlagFresh | (p.scene << kFlagSceneShift));
}

__device__ __forceinline__ void load_path(const PathState &ps, uint32_t cap, uint32_t slot, Path &p) {
    p.rng.state = ld_s(ps.rng + slot);
    p.pixel = ld_s(ps.pixel + slot);
    p.frame = ld_s(ps.frame + slot);
    p.rng.inc = (uint64_t)p.frame | 1u;
    const uint32_t fl = ld_s(ps.flags + slot);
    p.scene = fl >> kFlagSceneShift;
    if (fl & kFlagFresh) {
        p.T = mk(1.0f, 1.0f, 1.0f);
        p.bounces = 0;
        p.lobe = kLobeNull;
        p.medium = -1;
        p.iori = 1.0f;
    } else {
        p.T = mk(ld_s(ps.T + slot), ld_s(ps.T + cap + slot), ld_s(ps.T + 2 * cap + slot));
        p.bounces = ld_s(ps.bounces + slot);
        p.lobe = fl & 0xFFu;
        p.medium = (int)((fl >> kFlagMediumShift) & kFlagMediumMask) - 1;
        p.iori = ld_s(ps.iori + slot);
    }
}

__device__ __forceinline__ void write_ray(float4 *rays, uint32_t i, v3 o, float tnear, v3 d) {
    st_s(rays + 2 * i, make_float4(o.x, o.y, o.z, tnear));
    st_s(rays + 2 * i + 1, make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000)));
}

// SurfaceInteraction (integrator/surface_interaction.h:14-30)
struct Inter {
    v3 P, N, wi, wo;
    uint32_t lobe;
    float iori, ioro;
};

// BSDF Sample (lambert_bsdf.h:34-37, mirror_bsdf.h:31-34, ideal_specular_dielectric.h:35-64)
__device__ __forceinline__ void bsdf_sample(const MaterialInfo &m, Inter &it, Pcg &g) {
    if (m.bsdf == LT_BSDF_LAMBERT) {
        it.wi = cosine_hemisphere(it.N, g);
        it.lobe = kLobeDiffuse;
    } else if (m.bsdf == LT_BSDF_MIRROR) {
        it.wi = it.N * (2.0f * dot(it.wo, it.N)) - it.wo;
        it.lobe = kLobeSRefl;
    } else {
        float vdn = dot(it.wo, it.N);
        float ioro = m.ior;
        if (vdn < 0.0f) {
            ioro = 1.0f;
            it.N = -it.N;
            vdn = -vdn;
        }
        float eta = it.iori / ioro;
        float s2 = eta * eta * (1 - vdn * vdn);
        float F;
        if (s2 > 1.0f) {
            F = 1.0f;
        } else {
            float ct = sqrtf(1.0f - s2);
            float rperp = (it.iori * vdn - ioro * ct) / (it.iori * vdn + ioro * ct);
            float rpar = (ioro * vdn - it.iori * ct) / (ioro * vdn + it.iori * ct);
            F = 0.5f * (rperp * rperp + rpar * rpar);
        }
        float rnd = g.next_float();
        if (rnd <= F) {
            it.wi = it.N * (2.0f * dot(it.wo, it.N)) - it.wo;
            it.lobe = kLobeSRefl;
            it.ioro = it.iori;
        } else {
            it.wi = it.N * (eta * vdn - sqrtf(1.0f - s2)) - it.wo * eta;
            it.lobe = kLobeSTrans;
            it.ioro = ioro;
        }
    }
}

__device__ __forceinline__ v3 bsdf_eval(const MaterialInfo &m, v3 alb, const Inter &it) {
    if (m.bsdf == LT_BSDF_LAMBERT) return (alb * kInvPi) * dot(it.wi, it.N);
    return alb;
}

__device__ __forceinline__ float bsdf_pdf(const MaterialInfo &m, const Inter &it) {
    if (m.bsdf == LT_BSDF_LAMBERT) return dot(it.wi, it.N) * kInvPi;
    return 1.0f;
}

__device__ __forceinline__ void film_add(const FilmPtrs &f, uint32_t pixel, v3 c) {
    if (c.x != 0.0f) atomicAdd(f.rgb + 3 * (size_t)pixel, c.x);
    if (c.y != 0.0f) atomicAdd(f.rgb + 3 * (size_t)pixel + 1, c.y);
    if (c.z != 0.0f) atomicAdd(f.rgb + 3 * (size_t)pixel + 2, c.z);
}

// One radiance contribution of a path to its pixel, counted when a channel is
// not finite.
__device__ __forceinline__ void film_contribute(WaveCounters *counters, const FilmPtrs &f, uint32_t pixel, v3 c) {
    if (!(isfinite(c.x) && isfinite(c.y) && isfinite(c.z))) atomicAdd(&counters->nonfinite, 1ull);
    film_add(f, pixel, c);
}

// Work item -> sample index (frame offset * pixels + pixel, as start_path reads
// it) of a render of npix pixels x spp samples. Work items run in groups of G
// consecutive samples of one pixel, G the largest power of two up to
// min(spp, 64): a warp's camera rays then start in the same pixel and walk the
// same BVH nodes (icosphere render 1,641 -> 1,801 Msamples/s with G = 32, and
// 1,856 -> 1,871 with G = 64 once the shade groups continuing paths by
// octant: a block's paths come from fewer pixels). The spp % G samples left of
// every pixel follow as groups of spp % G. A bijection on [0, npix * spp): the
// same samples in another order.
__device__ __forceinline__ unsigned long long sample_of_item(unsigned long long item, unsigned long long npix,
                                                             uint32_t spp) {
    const uint32_t g = spp >= 64u ? 64u : 1u << (31 - __clz(spp | 1u));
    const uint32_t sh = __ffs(g) - 1, rem = spp & (g - 1u);
    const unsigned long long full = npix * (spp - rem);
    unsigned long long fo, pixel;
    if (item < full) {
        const unsigned long long q = item >> sh;
        const unsigned long long hi = (q | npix) >> 32 == 0 ? (uint32_t)q / (uint32_t)npix : q / npix;
        pixel = q - hi * npix;
        fo = (hi << sh) + (item & (g - 1u));
    } else {  // the last rem samples of every pixel
        const unsigned long long t = item - full;
        pixel = t / rem;
        fo = (spp - rem) + (t - pixel * rem);
    }
    return fo * npix + pixel;
}

// ------------------------------------------------------------------ scene sources
// The wavefront kernels are instantiated for two sources of scene data.
// OneScene keeps the scene, its render arguments and its film in the kernel
// parameters (lt_render). ManyScenes reads them per path from a batch's scene
// table in device memory (lt_render_batch): the work items of all scenes form
// one sequence, slot i owning [begin[i], begin[i] + slots[i].a.total), and every
// path carries its slot in its flags and connection records.
struct OneScene {
    static constexpr bool kMany = false, kDiff = false, kAdj = false;
    DevScene s;
    RenderArgs a;
    FilmPtrs f;
    __device__ __forceinline__ const DevScene &scene(uint32_t) const { return s; }
    __device__ __forceinline__ const RenderArgs &args(uint32_t) const { return a; }
    __device__ __forceinline__ const FilmPtrs &film(uint32_t) const { return f; }
    __device__ __forceinline__ unsigned long long total() const { return a.total; }
    __device__ __forceinline__ uint32_t locate(unsigned long long item, unsigned long long &local) const {
        const unsigned long long npix = (unsigned long long)a.width * a.height;
        local = sample_of_item(item, npix, (uint32_t)(a.total / npix));
        return 0;
    }
    __device__ __forceinline__ bool valid(uint32_t sid) const { return sid == 0; }
};

struct ManyScenes {
    static constexpr bool kMany = true, kDiff = false, kAdj = false;
    const SceneTable *t;
    __device__ __forceinline__ const DevScene &scene(uint32_t i) const { return t->slots[i].s; }
    __device__ __forceinline__ const RenderArgs &args(uint32_t i) const { return t->slots[i].a; }
    __device__ __forceinline__ const FilmPtrs &film(uint32_t i) const { return t->slots[i].f; }
    __device__ __forceinline__ unsigned long long total() const { return t->total; }
    // the slot that owns work item `item`: the last i with begin[i] <= item;
    // within the slot, work items in sample_of_item's order
    __device__ __forceinline__ uint32_t locate(unsigned long long item, unsigned long long &local) const {
        uint32_t lo = 0, hi = t->count;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (t->begin[mid] <= item) lo = mid;
            else hi = mid;
        }
        const RenderArgs &a = t->slots[lo].a;
        const unsigned long long npix = (unsigned long long)a.width * a.height;
        local = sample_of_item(item - t->begin[lo], npix, (uint32_t)(a.total / npix));
        return lo;
    }
    __device__ __forceinline__ bool valid(uint32_t sid) const { return sid < t->count; }
};

// The differentiable forward (lt_render_diff) as a third source: one scene,
// plus the estimator's parameters and the path extras of DiffWave. Its trace
// stage writes each connection record's contribution into d.res instead of
// the film.
struct DiffOne {
    static constexpr bool kMany = false, kDiff = true, kAdj = false;
    DevScene s;
    RenderArgs a;
    FilmPtrs f;
    DiffParams p;
    DiffWave d;
    __device__ __forceinline__ const DevScene &scene(uint32_t) const { return s; }
    __device__ __forceinline__ const RenderArgs &args(uint32_t) const { return a; }
    __device__ __forceinline__ const FilmPtrs &film(uint32_t) const { return f; }
    __device__ __forceinline__ const DiffParams &params(uint32_t) const { return p; }
    __device__ __forceinline__ float *samples(uint32_t) const { return d.sample_I; }
    __device__ __forceinline__ unsigned long long total() const { return a.total; }
    __device__ __forceinline__ uint32_t locate(unsigned long long item, unsigned long long &local) const {
        const unsigned long long npix = (unsigned long long)a.width * a.height;
        local = sample_of_item(item, npix, (uint32_t)(a.total / npix));
        return 0;
    }
    __device__ __forceinline__ bool valid(uint32_t sid) const { return sid == 0; }
};

// The batched differentiable forward (lt_render_diff_batch): the scenes of a
// batch's table, each with its parameters and per-sample radiance
// (SceneTable::diff), on one wavefront whose path extras are `d`.
struct DiffMany {
    static constexpr bool kMany = true, kDiff = true, kAdj = false;
    const SceneTable *t;
    DiffWave d;
    __device__ __forceinline__ const DevScene &scene(uint32_t i) const { return t->slots[i].s; }
    __device__ __forceinline__ const RenderArgs &args(uint32_t i) const { return t->slots[i].a; }
    __device__ __forceinline__ const FilmPtrs &film(uint32_t i) const { return t->slots[i].f; }
    __device__ __forceinline__ const DiffParams &params(uint32_t i) const { return t->diff[i].p; }
    __device__ __forceinline__ float *samples(uint32_t i) const { return t->diff[i].sample_I; }
    __device__ __forceinline__ unsigned long long total() const { return t->total; }
    __device__ __forceinline__ uint32_t locate(unsigned long long item, unsigned long long &local) const {
        uint32_t lo = 0, hi = t->count;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (t->begin[mid] <= item) lo = mid;
            else hi = mid;
        }
        const RenderArgs &a = t->slots[lo].a;
        const unsigned long long npix = (unsigned long long)a.width * a.height;
        local = sample_of_item(item - t->begin[lo], npix, (uint32_t)(a.total / npix));
        return lo;
    }
    __device__ __forceinline__ bool valid(uint32_t sid) const { return sid < t->count; }
};

// The adjoint (lt_render_adjoint with the forward's per-sample radiance) as a
// fourth source: DiffOne's paths replayed from their seeds over the samples of
// a crop, with the loss gradient and the gradient arrays of g. The work items
// are the crop's samples (a.total counts them), in sample_of_item's order over
// the crop's pixels. The adjoint leaves the film alone.
struct AdjOne {
    static constexpr bool kMany = false, kDiff = true, kAdj = true;
    DevScene s;
    RenderArgs a;
    DiffParams p;
    DiffWave d;
    DiffGrads g;
    __device__ __forceinline__ const DevScene &scene(uint32_t) const { return s; }
    __device__ __forceinline__ const RenderArgs &args(uint32_t) const { return a; }
    __device__ __forceinline__ const DiffParams &params(uint32_t) const { return p; }
    __device__ __forceinline__ const DiffGrads &grads(uint32_t) const { return g; }
    __device__ __forceinline__ unsigned long long total() const { return a.total; }
    __device__ __forceinline__ uint32_t locate(unsigned long long item, unsigned long long &local) const {
        const uint32_t cw = g.x1 - g.x0, ch = g.y1 - g.y0;
        const uint32_t ncrop = cw * ch;
        // sample * crop pixels + crop pixel, in sample_of_item's order
        const unsigned long long sc = sample_of_item(item, ncrop, (uint32_t)(a.total / ncrop));
        if (cw == a.width && ch == a.height) {
            local = sc;
            return 0;
        }
        const unsigned long long smp = sc / ncrop;
        const uint32_t k = (uint32_t)(sc - smp * ncrop), y = k / cw;
        local = smp * ((unsigned long long)a.width * a.height) + (unsigned long long)(g.y0 + y) * a.width + g.x0 +
                (k - y * cw);
        return 0;
    }
    __device__ __forceinline__ bool valid(uint32_t sid) const { return sid == 0; }
};

// The batched adjoint (lt_render_adjoint_batch, every job with its per-sample
// radiance): the whole films of a batch's table on one wavefront, work items
// as DiffMany's.
struct AdjMany {
    static constexpr bool kMany = true, kDiff = true, kAdj = true;
    const SceneTable *t;
    DiffWave d;
    __device__ __forceinline__ const DevScene &scene(uint32_t i) const { return t->slots[i].s; }
    __device__ __forceinline__ const RenderArgs &args(uint32_t i) const { return t->slots[i].a; }
    __device__ __forceinline__ const DiffParams &params(uint32_t i) const { return t->diff[i].p; }
    __device__ __forceinline__ const DiffGrads &grads(uint32_t i) const { return t->diff[i].g; }
    __device__ __forceinline__ unsigned long long total() const { return t->total; }
    __device__ __forceinline__ uint32_t locate(unsigned long long item, unsigned long long &local) const {
        uint32_t lo = 0, hi = t->count;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (t->begin[mid] <= item) lo = mid;
            else hi = mid;
        }
        const RenderArgs &a = t->slots[lo].a;
        const unsigned long long npix = (unsigned long long)a.width * a.height;
        local = sample_of_item(item - t->begin[lo], npix, (uint32_t)(a.total / npix));
        return lo;
    }
    __device__ __forceinline__ bool valid(uint32_t sid) const { return sid < t->count; }
};

__device__ __forceinline__ v3 ld3_planes(const float *p, uint32_t cap, uint32_t slot) {
    return mk(ld_s(p + slot), ld_s(p + cap + slot), ld_s(p + 2 * cap + slot));
}
__device__ __forceinline__ void st3_planes(float *p, uint32_t cap, uint32_t slot, v3 v) {
    st_s(p + slot, v.x);
    st_s(p + cap + slot, v.y);
    st_s(p + 2 * cap + slot, v.z);
}

// ------------------------------------------------------------------ kernels
// Closest hits of n rays (lt_intersect). Persistent: rays are fetched from *fetch.
template <class B>
__global__ void __launch_bounds__(128) k_intersect(DevScene S, const float4 *__restrict__ rays,
                                                   float4 *__restrict__ hits, uint32_t n, uint32_t *fetch) {
    const Geo g = B::geo(S);
    typename B::State r;
    typename B::Entry stack[B::kDepth];
    B::idle(r);
    uint32_t idx = 0;
    for (;;) {
        if (B::done(r)) {
            idx = fetch_next(fetch);
            if (idx >= n) break;
            float4 a = ld_s(rays + 2 * idx), b = ld_s(rays + 2 * idx + 1);
            B::start(r, stack, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w, false, 0);
        }
        B::run(g, r, stack);
        if (B::done(r)) st_s(hits + idx, make_float4(r.h.t, r.h.u, r.h.v, __uint_as_float(r.h.prim)));
    }
}

// Fill up to `capacity` slots with camera rays of the first work items.
template <class Src>
__global__ void __launch_bounds__(256) k_raygen(Src src, Wavefront W) {
    const unsigned long long total = src.total();
    unsigned long long first = total < W.capacity ? total : W.capacity;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < first; i += gridDim.x * blockDim.x) {
        Path p;
        v3 o, d;
        float tn;
        unsigned long long local;
        const uint32_t sid = src.locate(i, local);
        start_path(src.scene(sid), src.args(sid), local, p, o, d, tn);
        p.scene = sid;
        store_fresh_path(W.p[0], i, p);
        write_ray(W.ray[0], i, o, tn, d);
        if constexpr (Src::kDiff) {
            st3_planes(src.d.C[0], W.capacity, i, mk(0.0f, 0.0f, 0.0f));
            st3_planes(src.d.Ts[0], W.capacity, i, p.T);
            st_s(src.d.rec[0] + i, make_uint2(kNoRecord, kNoRecord));
        }
        if constexpr (Src::kAdj) st_s(src.d.pend[0] + i, kMiss);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counters->count[0] = (uint32_t)first;
        W.counters->count[1] = 0;
        W.counters->rcount[0] = W.counters->rcount[1] = 0;
        W.counters->ccount[0] = W.counters->ccount[1] = 0;
        W.counters->work_next = first;
        W.counters->fcount[0] = W.counters->fcount[1] = 0;
        W.counters->trace_fetch = 0;
    }
}

// Queue slots of one warp of a shade kernel: first connection record, first
// continuing-path entry, first finishing entry, first camera-ray entry and how
// many of the warp's finished paths start a camera ray, first work item.
struct Slots {
    uint32_t c, q, f, r, n_regen;
    unsigned long long w;
    uint32_t flag;  // the block's flag word as it stood once every warp had staged its counts
    uint32_t qpos;  // with octant keys: the lane's continuing-path entry
};

// The block's slots, reserved by one thread with one atomic per counter: each
// warp's lane 0 stages the warp's counts (connection records, continuing
// paths, finishing entries, finished paths) in shared memory, thread 0
// reserves the block's records, queue entries, finishing entries and work
// items and hands every warp its share (warps in order), then the camera-ray
// entries, whose number depends on how many work items were left. Every
// thread of the block calls it (block-uniform loops), at most 512 threads.
// `flag` (shared, optional): a word that the block's threads set before the
// call; every thread gets its value in Slots::flag (the same for all) and the
// word is cleared for the next round.
// kOct: the continuing paths take the block's entries grouped by `okey`, the
// octant of their next direction (0-7; 8 for a lane that does not continue),
// octants in order. A warp of the next trace then holds rays of a few
// neighbouring pixels that leave in the same octant. Each warp counts its
// octants into one of two per-block buffers of 8 counters (a shared atomic per
// octant present, `it` = the caller's iteration, whose parity picks the
// buffer; the first call zeroes both), thread 0 turns the counts into offsets
// and zeroes the other buffer, so no barrier is added after the first call.
template <bool kOct = false>
__device__ __forceinline__ Slots reserve_block(WaveCounters *wc, int cur, uint32_t nc, uint32_t np, uint32_t nf,
                                               uint32_t nd, unsigned long long total, uint32_t *flag = nullptr,
                                               uint32_t okey = 8u, uint32_t it = 0u) {
    const int nxt = cur ^ 1;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __shared__ uint32_t s_cnt[4][16];
    __shared__ uint32_t s_base[5][16];
    __shared__ unsigned long long s_wbase[16];
    __shared__ uint32_t s_flag;
    __shared__ uint32_t s_oct[2][8];  // kOct: continuing paths per octant, then their offsets (by parity)
    uint32_t orank = 0;               // kOct: the lane's place within its octant's entries
    const uint32_t ob = it & 1u;
    if constexpr (kOct) {
        if (it == 0u) {  // block-uniform
            if (threadIdx.x < 16u) s_oct[threadIdx.x >> 3][threadIdx.x & 7u] = 0u;
            __syncthreads();
        }
        const unsigned same = __match_any_sync(0xFFFFFFFFu, okey);
        const int leader = __ffs(same) - 1;
        uint32_t b = 0;
        if (okey < 8u && (int)lane == leader) b = atomicAdd(&s_oct[ob][okey], (uint32_t)__popc(same));
        orank = __shfl_sync(0xFFFFFFFFu, b, leader) + __popc(same & ((1u << lane) - 1u));
    }
    if (lane == 0) {
        s_cnt[0][warp] = nc;
        s_cnt[1][warp] = np;
        s_cnt[2][warp] = nf;
        s_cnt[3][warp] = nd;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (flag) {
            s_flag = *flag;
            *flag = 0u;
        }
        const uint32_t nw = blockDim.x >> 5;
        uint32_t tc = 0, tp = 0, tf = 0, td = 0;
        for (uint32_t w = 0; w < nw; ++w) {
            tc += s_cnt[0][w];
            tp += s_cnt[1][w];
            tf += s_cnt[2][w];
            td += s_cnt[3][w];
        }
        const uint32_t c0 = tc ? atomicAdd(&wc->ccount[cur], tc) : 0u;
        const uint32_t q0 = tp ? atomicAdd(&wc->count[nxt], tp) : 0u;
        const uint32_t f0 = tf ? atomicAdd(&wc->fcount[nxt], tf) : 0u;
        const unsigned long long w0 = td ? atomicAdd(&wc->work_next, (unsigned long long)td) : 0ull;
        const unsigned long long left = w0 < total ? total - w0 : 0ull;
        const uint32_t nreg = left < (unsigned long long)td ? (uint32_t)left : td;
        const uint32_t r0 = nreg ? atomicAdd(&wc->rcount[nxt], nreg) : 0u;
        if constexpr (kOct) {  // octant offsets; the other buffer is zeroed for the next call
            uint32_t a = 0;
#pragma unroll
            for (uint32_t k = 0; k < 8u; ++k) {
                const uint32_t v = s_oct[ob][k];
                s_oct[ob][k] = a;
                a += v;
                s_oct[ob ^ 1u][k] = 0u;
            }
        }
        uint32_t pc = 0, pp = 0, pf = 0, pd = 0;
        for (uint32_t w = 0; w < nw; ++w) {
            s_base[0][w] = c0 + pc;
            s_base[1][w] = q0 + pp;
            s_base[2][w] = f0 + pf;
            s_wbase[w] = w0 + pd;
            const uint32_t before = pd < nreg ? pd : nreg;  // camera rays of the warps before
            s_base[3][w] = r0 + before;
            s_base[4][w] = nreg - before < s_cnt[3][w] ? nreg - before : s_cnt[3][w];
            pc += s_cnt[0][w];
            pp += s_cnt[1][w];
            pf += s_cnt[2][w];
            pd += s_cnt[3][w];
        }
    }
    __syncthreads();
    Slots r;
    r.c = s_base[0][warp];
    r.q = s_base[1][warp];
    r.f = s_base[2][warp];
    r.r = s_base[3][warp];
    r.n_regen = s_base[4][warp];
    r.w = s_wbase[warp];
    r.flag = flag ? s_flag : 0u;
    r.qpos = 0u;
    if constexpr (kOct) {
        if (okey < 8u) r.qpos = s_base[1][0] + s_oct[ob][okey] + orank;
    }
    return r;
}

// k_shade's checks of a surface hit (LT_CHECKS builds): the triangle's mesh,
// the mesh's material and its light.
__device__ __forceinline__ bool surface_ok(const DevScene &S, WaveCounters *wc, uint32_t prim) {
#if LT_CHECKS
    const uint32_t gid = __ldg(S.tri_geom + prim);
    if (!LT_CHECK(wc, gid < S.num_geoms, kChkGeom, gid)) return false;
    const GeomInfo &G = S.geoms[gid];
    if (!LT_CHECK(wc, (uint32_t)G.material < S.num_mats, kChkMaterial, G.material)) return false;
    if (!LT_CHECK(wc, G.light < 0 || (uint32_t)G.light < S.num_lights, kChkLight, G.light)) return false;
#endif
    return true;
}

// One iteration of the bounce loop of Integrator::RenderPixel (integrator.cpp:115-243).
// Register budget: 1024 threads per SM (64 registers, a few spilled) for the
// single-scene instantiation, measured 1.1% faster than 768 threads (76
// registers) with the whole render in flight; the batched one keeps 768.
template <class Src>
__global__ void __launch_bounds__(Src::kMany ? 256 : 512, Src::kMany ? 3 : 2) k_shade(Src src, Wavefront W, int cur) {
    const uint32_t n_push = W.counters->count[cur], n_cam = W.counters->rcount[cur];
    const uint32_t n = n_push + n_cam;
    const uint32_t cap = W.capacity;
    const int nxt = cur ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counters->trace_fetch = 0;  // for the next k_trace
    LT_STOP_IF_FAILED(W.counters);
    uint32_t n_ref_rays = 0, n_ref_rays_b = 0;  // connection rays the reference would trace
    uint32_t it = 0;                            // this block's iteration of the loop below
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t q = base + threadIdx.x;
        const uint32_t slot = q < n ? queue_slot(q, n_push, n_cam, cap) : 0u;
        const bool active = q < n && LT_CHECK(W.counters, slot < cap, kChkSlot, slot);
        Path p;
        bool done = false, push = false;
        v3 norg = mk(0, 0, 0), ndir = mk(0, 0, 0);
        float ntnear = 0.0f;
        // connection records (light sample, BSDF-MIS sample)
        bool emit_l = false, emit_b = false;
        v3 l_dir = mk(0, 0, 0), b_dir = mk(0, 0, 0), l_f = mk(0, 0, 0), b_f = mk(0, 0, 0), conn_org = mk(0, 0, 0);
        float l_pdf = 0.0f, b_pdf = 0.0f, l_tl = 0.0f, b_tl = 0.0f;
        uint32_t conn_light = 0;
        v3 conn_T = mk(0, 0, 0);
        if (active) load_path(W.p[cur], cap, slot, p);
        if (active && LT_CHECK(W.counters, src.valid(p.scene), kChkScene, p.scene)) {
            const DevScene &S = src.scene(p.scene);
            const RenderArgs &A = src.args(p.scene);
            float4 hv = ld_s(W.hits + slot);
            float4 r0 = ld_s(W.ray[cur] + 2 * slot), r1 = ld_s(W.ray[cur] + 2 * slot + 1);
            uint32_t prim = __float_as_uint(hv.w);
            float t = hv.x;
            if (prim == kMiss) {
                if (LT_PIXEL_OK(W, p.pixel, A.width * A.height))
                    film_contribute(W.counters, src.film(p.scene), p.pixel, p.T * S.background);
                done = true;
            } else if (!LT_CHECK(W.counters, prim < S.num_tris, kChkPrim, prim)) {
                done = true;
            } else {
                v3 origin = mk(r0.x, r0.y, r0.z);
                v3 direction = normalize(mk(r1.x, r1.y, r1.z));
                bool hit_surface = true;
                if (p.medium >= 0 && !LT_CHECK(W.counters, (uint32_t)p.medium < S.num_media, kChkMedium, p.medium)) {
                    done = true;
                    hit_surface = false;
                    p.medium = -1;
                }
                if (hit_surface && !surface_ok(S, W.counters, prim)) {
                    done = true;
                    hit_surface = false;
                }
                if (p.medium >= 0) {
                    const MediumInfo M = S.meds[p.medium];
                    float dist;
                    if (M.type == LT_MEDIUM_NON_SCATTERING) {
                        // non_scattering_medium.h:20-39
                        dist = t;
                        v3 tr = mk(expf(-M.sigma_a[0] * dist), expf(-M.sigma_a[1] * dist), expf(-M.sigma_a[2] * dist));
                        p.T = (p.T * 1.0f) * tr;
                    } else if (M.type == LT_MEDIUM_ISOTROPIC) {
                        // isotropic_scattering_medium.h:31-51
                        dist = -logf(p.rng.next_float()) / M.sigma_s[0];
                        if (dist >= t) dist = t;
                        v3 tr = mk(expf(-M.sigma_a[0] * dist), expf(-M.sigma_a[1] * dist), expf(-M.sigma_a[2] * dist));
                        p.T = (p.T * 1.0f) * tr;
                    } else {
                        // RGB sigma_s (extension): distance from the mean sigma_s,
                        // weight = transmittance (x sigma_s on scatter) / pdf
                        float sbar = M.sigma_s_mean;
                        dist = -logf(p.rng.next_float()) / sbar;
                        bool scat = dist < t;
                        if (!scat) dist = t;
                        v3 w = mk(expf(-(M.sigma_a[0] + M.sigma_s[0] - sbar) * dist),
                                  expf(-(M.sigma_a[1] + M.sigma_s[1] - sbar) * dist),
                                  expf(-(M.sigma_a[2] + M.sigma_s[2] - sbar) * dist));
                        if (scat) w = w * (mk(M.sigma_s[0], M.sigma_s[1], M.sigma_s[2]) / sbar);
                        p.T = p.T * w;
                    }
                    if (dist < t) {
                        hit_surface = false;
                        norg = origin + direction * dist;
                        ndir = M.type == LT_MEDIUM_HG ? hg_sample(p.rng, direction, M.g) : uniform_sphere(p.rng);
                        ntnear = 0.001f;
                    }
                }
                if (hit_surface) {
                    const GeomInfo G = S.geoms[__ldg(S.tri_geom + prim)];
                    const MaterialInfo m = S.mats[G.material];
                    if ((p.bounces == 0 || (p.lobe & kLobeSpecular) != 0) && G.light >= 0 &&
                        LT_PIXEL_OK(W, p.pixel, A.width * A.height)) {
                        const LightInfo &L = S.lights[G.light];
                        film_contribute(W.counters, src.film(p.scene), p.pixel,
                                        p.T * mk(L.radiance[0], L.radiance[1], L.radiance[2]));
                    }
                    Inter it;
                    it.P = origin + direction * t;
                    it.N = G.has_normals ? normalize(interp_normal(S, prim, hv.y, hv.z)) : normalize(mk(0, 0, 0));
                    const v3 alb = material_albedo(S, m, G, prim, hv.y, hv.z);
                    it.wo = -direction;
                    it.ioro = 0.0f;
                    it.iori = p.iori;
                    it.lobe = p.lobe;
                    it.wi = mk(0, 0, 0);
                    // SampleOneLight (integrator.cpp:252-271), interaction by value
                    uint32_t nl = S.num_lights;
                    if (!(nl == 0 || (nl == 1 && G.light >= 0))) {
                        int li;
                        int guard = 0;
                        do {
                            li = (int)p.rng.next_discrete(nl);
                        } while (li == G.light && ++guard < 1 << 20);
                        const LightInfo &L = S.lights[li];
                        v3 Le = mk(L.radiance[0], L.radiance[1], L.radiance[2]);
                        Inter c = it;
                        conn_org = it.P;
                        conn_light = (uint32_t)li;
                        conn_T = p.T;
                        // EstimateDirect (integrator.cpp:273-315)
                        if (m.bsdf == LT_BSDF_LAMBERT) {
                            // AreaLight::SampleLi (area_light.cpp:18-36)
                            float x, y;
                            sample_disc(p.rng, L.sphere[3], x, y);
                            v3 cdir = mk(L.sphere[0], L.sphere[1], L.sphere[2]) - c.P;
                            float dist = length(cdir);
                            v3 cn = normalize(cdir);
                            v3 point = rotate_to_world(x, y, dist - L.sphere[3], cn);
                            v3 ldir = normalize(point);
                            c.wi = ldir;
                            if (dot(ldir, c.N) > 0.0f) {
                                n_ref_rays++;  // the reference traces this ray (area_light.cpp:58)
                                v3 f = bsdf_eval(m, alb, c);
                                float spdf = bsdf_pdf(m, c);
                                if (!is_black(Le) && spdf != 0.0f && !is_black(f)) {
                                    // a ray that misses the light's own triangles cannot contribute
                                    float tl = light_distance(S, L, c.P, ldir, nullptr);
                                    if (tl != 0.0f) {
                                        emit_l = true;
                                        l_dir = ldir;
                                        l_f = f;
                                        l_pdf = spdf;
                                        l_tl = tl;
                                    }
                                }
                            }
                        }
                        bsdf_sample(m, c, p.rng);
                        v3 f = bsdf_eval(m, alb, c);
                        float spdf = bsdf_pdf(m, c);
                        // AreaLight::PdfLi horizon test (area_light.cpp:76-78)
                        if (spdf != 0.0f && !is_black(f) && dot(c.wi, c.N) > 0.0f) {
                            n_ref_rays_b++;  // the reference traces this ray (area_light.cpp:100)
                            float tl = light_distance(S, L, c.P, c.wi, nullptr);
                            if (tl != 0.0f) {
                                emit_b = true;
                                b_dir = c.wi;
                                b_f = f;
                                b_pdf = spdf;
                                b_tl = tl;
                            }
                        }
                    }
                    // main path BSDF sample (integrator.cpp:199-209)
                    bsdf_sample(m, it, p.rng);
                    float pdf = bsdf_pdf(m, it);
                    p.T = (p.T * bsdf_eval(m, alb, it)) / pdf;
                    if (it.lobe == kLobeSTrans) {
                        it.iori = it.ioro;
                        p.medium = m.medium;
                    }
                    p.iori = it.iori;
                    p.lobe = it.lobe;
                    norg = it.P;
                    ndir = it.wi;
                    ntnear = 0.001f;
                }
                // Russian roulette (integrator.cpp:235-242)
                if (p.bounces > A.rr_depth) {
                    float pr = fmaxf(p.T.x, fmaxf(p.T.y, p.T.z));
                    if (p.rng.next_float() > pr) done = true;
                    else p.T = p.T * (1 / pr);
                }
            }
            if (!done) {
                p.bounces++;
                if (p.bounces >= A.max_depth) done = true;
                else push = true;
            }
        }
        const uint32_t lane = threadIdx.x & 31u;
        const unsigned below = (1u << lane) - 1u;
        const unsigned m_l = __ballot_sync(0xFFFFFFFFu, emit_l), m_b = __ballot_sync(0xFFFFFFFFu, emit_b);
        const unsigned m_d = __ballot_sync(0xFFFFFFFFu, done), m_p = __ballot_sync(0xFFFFFFFFu, push);
        const uint32_t okey =
            push ? (ndir.x < 0.0f ? 1u : 0u) | (ndir.y < 0.0f ? 2u : 0u) | (ndir.z < 0.0f ? 4u : 0u) : 8u;
        const Slots sl = reserve_block<true>(W.counters, cur, __popc(m_l) + __popc(m_b), __popc(m_p), 0u, __popc(m_d),
                                             src.total(), nullptr, okey, it++);
        const uint32_t c_base = sl.c, r_base = sl.r, n_regen = sl.n_regen;
        const unsigned long long w_base = sl.w;
        // connection records: the warp's light samples, then its BSDF samples
        {
            conn_light |= p.scene << kConnSceneShift;
            uint32_t idx = c_base + __popc(m_l & below);
            if (emit_l && LT_CHECK(W.counters, idx < 2u * cap, kChkRecord, idx)) {
                st_s(W.cray + 2 * idx, make_float4(conn_org.x, conn_org.y, conn_org.z, __uint_as_float(conn_light)));
                st_s(W.cray + 2 * idx + 1, make_float4(l_dir.x, l_dir.y, l_dir.z, l_tl));
                st_s(W.crec + 2 * idx, make_float4(l_f.x, l_f.y, l_f.z, l_pdf));
                st_s(W.crec + 2 * idx + 1, make_float4(conn_T.x, conn_T.y, conn_T.z, __uint_as_float(p.pixel)));
            }
            idx = c_base + __popc(m_l) + __popc(m_b & below);
            if (emit_b && LT_CHECK(W.counters, idx < 2u * cap, kChkRecord, idx)) {
                st_s(W.cray + 2 * idx,
                     make_float4(conn_org.x, conn_org.y, conn_org.z, __uint_as_float(conn_light | kConnectBsdf)));
                st_s(W.cray + 2 * idx + 1, make_float4(b_dir.x, b_dir.y, b_dir.z, b_tl));
                st_s(W.crec + 2 * idx, make_float4(b_f.x, b_f.y, b_f.z, b_pdf));
                st_s(W.crec + 2 * idx + 1, make_float4(conn_T.x, conn_T.y, conn_T.z, __uint_as_float(p.pixel)));
            }
        }
        // finished paths: film write (integrator.cpp:245-249; the radiance went to
        // the film as it was found); the thread then starts the next work item
        // in their place
        bool regen = false;
        if (done && LT_PIXEL_OK(W, p.pixel, src.args(p.scene).width * src.args(p.scene).height)) {
            const FilmPtrs &F = src.film(p.scene);
            atomicAdd(F.bounces + p.pixel, p.bounces);
            atomicAdd(F.counts + p.pixel, 1u);
        }
        // work items go to the finished lanes in lane order
        const uint32_t rank_d = __popc(m_d & below);
        if (done && rank_d < n_regen) {
            unsigned long long local;
            const uint32_t sid = src.locate(w_base + rank_d, local);
            start_path(src.scene(sid), src.args(sid), local, p, norg, ndir, ntnear);
            p.scene = sid;
            regen = true;
        }
        if (push || regen) {
            const uint32_t qi = push ? sl.qpos : cap - 1u - (r_base + rank_d);
            if (LT_CHECK(W.counters, qi < cap, kChkOutSlot, qi)) {
                write_ray(W.ray[nxt], qi, norg, ntnear, ndir);
                if (push) store_path(W.p[nxt], cap, qi, p);
                else store_fresh_path(W.p[nxt], qi, p);
            }
        }
    }
    // ray tallies in the reference's terms (every SampleLi / PdfLi trace), one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        n_ref_rays += __shfl_xor_sync(0xFFFFFFFFu, n_ref_rays, o);
        n_ref_rays_b += __shfl_xor_sync(0xFFFFFFFFu, n_ref_rays_b, o);
    }
    if ((threadIdx.x & 31u) == 0 && (n_ref_rays | n_ref_rays_b)) {
        atomicAdd(&W.counters->light_rays, (unsigned long long)n_ref_rays);
        atomicAdd(&W.counters->bsdf_rays, (unsigned long long)n_ref_rays_b);
    }
}

__device__ __forceinline__ void add3(float *g, v3 v) {
    if (v.x != 0.0f) atomicAdd(g, v.x);
    if (v.y != 0.0f) atomicAdd(g + 1, v.y);
    if (v.z != 0.0f) atomicAdd(g + 2, v.z);
}

// Per-block sums of the adjoint's gradient terms in shared memory, keyed by
// the address of the gradient triple they add to: direct mapped by a
// multiplicative hash of the address, a slot is claimed by the first key that
// lands on it and kept until the kernel ends (or, in the batched shade, until
// the table moves to a new scene). Most terms fall on a few triangles (a
// ground quad, a light's triangles) and on the media, whose sums then stay in
// shared memory instead of queueing at one L2 address; a term whose slot holds
// another key goes straight to the gradient array. Every block adds its sums
// to the gradient arrays once, at its end. 2^kBits slots: the fewer, the more
// L1 the kernel keeps (measured: 256 slots 2% faster than 512 on the whole
// adjoint, 1024 slower still).
template <int kBits>
struct GradTable {
    static constexpr int kSlots = 1 << kBits;
    unsigned long long key[kSlots];
    float val[3 * kSlots];
    uint32_t scene;  // batched adjoint: the scene slot the table was last given to
    uint32_t other;  // 1 + a scene slot seen since the last round, or 0 (plain stores by
                     // any thread: which of the values written wins does not matter)

    // Every thread of the block calls it; a barrier follows before the first add.
    __device__ __forceinline__ void init() {
        for (int i = threadIdx.x; i < kSlots; i += blockDim.x) {
            key[i] = 0ull;
            val[3 * i] = val[3 * i + 1] = val[3 * i + 2] = 0.0f;
        }
        if (threadIdx.x == 0) {
            scene = kMiss;
            other = 0u;
        }
    }

    __device__ __forceinline__ void add(float *g, v3 v) {
        if (v.x == 0.0f && v.y == 0.0f && v.z == 0.0f) return;
        const unsigned long long k = (unsigned long long)g;
        const uint32_t s = (uint32_t)(((k >> 2) * 0x9E3779B97F4A7C15ull) >> (64 - kBits));
        unsigned long long held = *(volatile unsigned long long *)&key[s];
        if (held == 0ull) {
            held = atomicCAS(&key[s], 0ull, k);
            if (held == 0ull) held = k;
        }
        if (held == k) {
            float *vs = val + 3 * s;
            if (v.x != 0.0f) atomicAdd(vs, v.x);
            if (v.y != 0.0f) atomicAdd(vs + 1, v.y);
            if (v.z != 0.0f) atomicAdd(vs + 2, v.z);
        } else {
            add3(g, v);
        }
    }

    // Every thread of the block calls it, after a barrier that follows the last add.
    __device__ __forceinline__ void flush() {
        for (int i = threadIdx.x; i < kSlots; i += blockDim.x) {
            const unsigned long long k = key[i];
            if (k) add3((float *)k, mk(val[3 * i], val[3 * i + 1], val[3 * i + 2]));
        }
    }
};
constexpr int kTraceGradBits = 8, kShadeGradBits = 8;
using TraceGrads = GradTable<kTraceGradBits>;
using ShadeGrads = GradTable<kShadeGradBits>;

// The table of the calling kernel (one per adjoint kernel instantiation).
template <class Src, class T>
__device__ __forceinline__ T *grad_table() {
    __shared__ T t;
    return &t;
}

// The adjoint's inputs for sample (pixel, frame) of slot sid: the sample's
// radiance I from the forward and delta = d loss / d film colour sum.
template <class Src>
__device__ __forceinline__ void adj_inputs(const Src &src, uint32_t sid, uint32_t pixel, uint32_t frame, v3 &I,
                                           v3 &delta) {
    const RenderArgs &A = src.args(sid);
    const DiffGrads &G = src.grads(sid);
    const unsigned long long item =
        (unsigned long long)(frame - A.first_frame) * ((unsigned long long)A.width * A.height) + pixel;
    I = mk(ld_s(G.sample_I + 3 * item), ld_s(G.sample_I + 3 * item + 1), ld_s(G.sample_I + 3 * item + 2));
    delta = ld3(G.dI + 3 * (size_t)pixel);
}

// The albedo term of a surface bounce on triangle prim, delta * (I - C) *
// dlog(f)/d albedo (f is linear in the albedo), once C holds the bounce's
// connection contributions.
template <class Src>
__device__ __forceinline__ void albedo_term(ShadeGrads *t, const Src &src, uint32_t sid, uint32_t prim, v3 I, v3 delta,
                                            v3 C) {
    const v3 R = (I - C) * delta;
    const v3 alb = ld3(src.params(sid).albedo + 3 * prim);
    t->add(src.grads(sid).albedo + 3 * prim,
           mk(alb.x > 0.0f ? R.x / alb.x : 0.0f, alb.y > 0.0f ? R.y / alb.y : 0.0f, alb.z > 0.0f ? R.z / alb.z : 0.0f));
}

// One bounce of the differentiable estimator (diff_path below, one bounce of
// its loop) for every queued path, on the wavefront. It is k_shade with the
// estimator's arithmetic: per-triangle albedo and emission, the RGB medium form
// with the detached sigma_s for distances, roulette from the detached
// throughput Ts, and a path radiance C carried in the path state so that every
// sample's radiance is summed in the estimator's order. A surface bounce
// emits the same connection records as k_shade; k_trace writes their
// contributions into d.res, and the path's next shade adds them to C (light
// sample, then BSDF sample) before anything of its next bounce. A path that
// ends with records still to be traced becomes a finishing entry, completed by
// the next shade. Finished samples write their radiance to d.sample_I; film
// counts and path lengths are added here, the colour sums later in sample
// order (k_diff_film).
__device__ __forceinline__ v3 add_record(const DiffWave &d, uint32_t rec, v3 C) {
    if (rec == kNoRecord) return C;
    const float4 v = ld_s(d.res + rec);
    return v.w != 0.0f ? C + mk(v.x, v.y, v.z) : C;
}

// add_record for the batched adjoint: a contributing record also adds its
// gradient terms (d.gres, from the trace stage) to the albedo of the triangle
// it was sampled on (prim) and to the emission of the light triangle it reached.
__device__ __forceinline__ v3 add_record_adj(const DiffWave &d, uint32_t rec, v3 C, ShadeGrads *gt,
                                             const DiffGrads &G, uint32_t prim) {
    if (rec == kNoRecord) return C;
    const float4 v = ld_s(d.res + rec);
    if (v.w == 0.0f) return C;
    const float4 a = ld_s(d.gres + 2 * rec), e = ld_s(d.gres + 2 * rec + 1);
    gt->add(G.albedo + 3 * (size_t)prim, mk(a.x, a.y, a.z));
    gt->add(G.emission + 3 * (size_t)__float_as_uint(a.w), mk(e.x, e.y, e.z));
    return C + mk(v.x, v.y, v.z);
}

__device__ __forceinline__ void write_sample(float *sample_I, const RenderArgs &A, uint32_t pixel, uint32_t frame,
                                             v3 C) {
    const unsigned long long item =
        (unsigned long long)(frame - A.first_frame) * ((unsigned long long)A.width * A.height) + pixel;
    st_s(sample_I + 3 * item, C.x);
    st_s(sample_I + 3 * item + 1, C.y);
    st_s(sample_I + 3 * item + 2, C.z);
}

// Register budget: three 256-thread blocks per SM for the forward; four for
// the adjoint (64 registers, spilling), measured 0.5-1% faster on the whole
// adjoint than three (80 registers) and 15% faster than two (no spills).
template <class Src>
__global__ void __launch_bounds__(256, Src::kAdj ? 4 : 3) k_dshade(Src src, Wavefront W, int cur) {
    const DiffWave &D = src.d;
    const uint32_t n_push = W.counters->count[cur], n_cam = W.counters->rcount[cur];
    const uint32_t n = n_push + n_cam, nf = W.counters->fcount[cur];
    const uint32_t cap = W.capacity;
    const int nxt = cur ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) W.counters->trace_fetch = 0;  // for the next k_trace
    LT_STOP_IF_FAILED(W.counters);
    uint32_t n_ref_rays = 0, n_ref_rays_b = 0;
    ShadeGrads *gt = nullptr;
    if constexpr (Src::kAdj) {
        gt = grad_table<Src, ShadeGrads>();
        gt->init();
        __syncthreads();
    }
    uint32_t it = 0;  // this block's iteration of the loop below
    for (uint32_t base = blockIdx.x * blockDim.x; base < n + nf; base += gridDim.x * blockDim.x) {
        const uint32_t q = base + threadIdx.x;
        const uint32_t slot = q < n ? queue_slot(q, n_push, n_cam, cap) : 0u;
        const bool active = q < n && LT_CHECK(W.counters, slot < cap, kChkSlot, slot);
        if (q >= n && q < n + nf) {  // a finishing entry: its last records, then the sample is complete
            const uint32_t e = q - n;
            const uint4 id = ld_s(D.fin_id[cur] + e);  // pixel, frame, scene slot
            const float4 c4 = ld_s(D.fin_C[cur] + e);
            const uint2 rc = ld_s(D.fin_rec[cur] + e);
            if constexpr (Src::kAdj) {  // its records (and their terms), then its last bounce's albedo term
                const DiffGrads &Gr = src.grads(id.z);
                const v3 C4 = mk(c4.x, c4.y, c4.z);
                const v3 Cf = Src::kMany ? add_record_adj(D, rc.y, add_record_adj(D, rc.x, C4, gt, Gr, id.w), gt, Gr, id.w)
                                         : add_record(D, rc.y, add_record(D, rc.x, C4));
                if (Src::kMany && id.z != gt->scene) gt->other = id.z + 1u;
                if (id.w != kMiss) {
                    v3 I, delta;
                    adj_inputs(src, id.z, id.x, id.y, I, delta);
                    albedo_term(gt, src, id.z, id.w, I, delta, Cf);
                }
            } else {
                write_sample(src.samples(id.z), src.args(id.z), id.x, id.y,
                             add_record(D, rc.y, add_record(D, rc.x, mk(c4.x, c4.y, c4.z))));
            }
        }
        Path p;
        v3 C = mk(0, 0, 0), Ts = mk(0, 0, 0);
        bool done = false, push = false;
        v3 norg = mk(0, 0, 0), ndir = mk(0, 0, 0);
        float ntnear = 0.0f;
        bool emit_l = false, emit_b = false;
        v3 l_dir = mk(0, 0, 0), b_dir = mk(0, 0, 0), l_f = mk(0, 0, 0), b_f = mk(0, 0, 0), conn_org = mk(0, 0, 0);
        float l_pdf = 0.0f, b_pdf = 0.0f, l_tl = 0.0f, b_tl = 0.0f;
        uint32_t conn_light = 0;
        v3 conn_T = mk(0, 0, 0);
        // adjoint: the sample's radiance and loss gradient, the triangle whose
        // albedo term waits for this bounce's records, the BSDF sample's f / albedo
        v3 I = mk(0, 0, 0), delta = mk(0, 0, 0);
        uint32_t pend = kMiss, shade_prim = kMiss;
        float b_dfa = 0.0f;
        if (active) {
            load_path(W.p[cur], cap, slot, p);
            const DevScene &S = src.scene(p.scene);
            const RenderArgs &A = src.args(p.scene);
            const DiffParams &P = src.params(p.scene);
            C = ld3_planes(D.C[cur], cap, slot);
            Ts = ld3_planes(D.Ts[cur], cap, slot);
            const uint2 rc = ld_s(D.rec[cur] + slot);
            bool skip = false;
            if constexpr (Src::kAdj) {
                adj_inputs(src, p.scene, p.pixel, p.frame, I, delta);
                const uint32_t pp = ld_s(D.pend[cur] + slot);  // the previous bounce's triangle
                const DiffGrads &Gr = src.grads(p.scene);
                C = Src::kMany ? add_record_adj(D, rc.y, add_record_adj(D, rc.x, C, gt, Gr, pp), gt, Gr, pp)
                               : add_record(D, rc.y, add_record(D, rc.x, C));
                if (pp != kMiss) albedo_term(gt, src, p.scene, pp, I, delta, C);
                if (Src::kMany && p.scene != gt->scene) gt->other = p.scene + 1u;
                skip = is_black(delta);  // every term of the sample is 0
            } else {
                C = add_record(D, rc.y, add_record(D, rc.x, C));  // the previous bounce's light, then BSDF sample
            }
            const float4 hv = ld_s(W.hits + slot);
            const float4 r0 = ld_s(W.ray[cur] + 2 * slot), r1 = ld_s(W.ray[cur] + 2 * slot + 1);
            const uint32_t prim = __float_as_uint(hv.w);
            const float t = hv.x;
            if (skip) {
                done = true;
            } else if (prim == kMiss) {
                C = C + p.T * S.background;
                done = true;
            } else {
                const v3 origin = mk(r0.x, r0.y, r0.z);
                const v3 direction = normalize(mk(r1.x, r1.y, r1.z));
                bool hit_surface = true;
                if (p.medium >= 0) {
                    const int mi = p.medium;
                    const MediumInfo M = S.meds[mi];
                    const v3 sa = ld3(P.sigma_a + 3 * mi), ss = ld3(P.sigma_s + 3 * mi);
                    const v3 sa_d = ld3(P.sigma_a_s + 3 * mi), ss_d = ld3(P.sigma_s_s + 3 * mi);
                    float dist;
                    bool scat = false;
                    v3 w, ws;
                    if (M.type == LT_MEDIUM_NON_SCATTERING) {
                        dist = t;
                        w = mk(expf(-sa.x * dist), expf(-sa.y * dist), expf(-sa.z * dist));
                        ws = mk(expf(-sa_d.x * dist), expf(-sa_d.y * dist), expf(-sa_d.z * dist));
                    } else {
                        const float sbar = M.type == LT_MEDIUM_ISOTROPIC ? ss_d.x : (ss_d.x + ss_d.y + ss_d.z) / 3.0f;
                        dist = -logf(p.rng.next_float()) / sbar;
                        scat = dist < t;
                        if (!scat) dist = t;
                        w = mk(expf(-(sa.x + ss.x - sbar) * dist), expf(-(sa.y + ss.y - sbar) * dist),
                               expf(-(sa.z + ss.z - sbar) * dist));
                        ws = mk(expf(-(sa_d.x + ss_d.x - sbar) * dist), expf(-(sa_d.y + ss_d.y - sbar) * dist),
                                expf(-(sa_d.z + ss_d.z - sbar) * dist));
                        if (scat) {
                            w = w * (ss / sbar);
                            ws = ws * (ss_d / sbar);
                        }
                    }
                    if constexpr (Src::kAdj) {  // d log(w) / d sigma, with C before this segment's end
                        const v3 R = (I - C) * delta;
                        const v3 ga = R * (-dist);
                        v3 gs = mk(0, 0, 0);
                        if (M.type != LT_MEDIUM_NON_SCATTERING)
                            gs = mk(R.x * (-dist + (scat ? 1.0f / ss.x : 0.0f)),
                                    R.y * (-dist + (scat ? 1.0f / ss.y : 0.0f)),
                                    R.z * (-dist + (scat ? 1.0f / ss.z : 0.0f)));
                        gt->add(src.grads(p.scene).sigma_a + 3 * mi, ga);
                        gt->add(src.grads(p.scene).sigma_s + 3 * mi, gs);
                    }
                    p.T = p.T * w;
                    Ts = Ts * ws;
                    if (scat) {
                        hit_surface = false;
                        norg = origin + direction * dist;
                        ndir = M.type == LT_MEDIUM_HG ? hg_sample(p.rng, direction, M.g) : uniform_sphere(p.rng);
                        ntnear = 0.001f;
                    }
                }
                if (hit_surface) {
                    const GeomInfo G = S.geoms[__ldg(S.tri_geom + prim)];
                    const MaterialInfo m = S.mats[G.material];
                    const v3 alb = ld3(P.albedo + 3 * prim), alb_d = ld3(P.albedo_s + 3 * prim);
                    if ((p.bounces == 0 || (p.lobe & kLobeSpecular) != 0) && G.light >= 0) {
                        C = C + p.T * ld3(P.emission + 3 * prim);
                        if constexpr (Src::kAdj) gt->add(src.grads(p.scene).emission + 3 * prim, p.T * delta);
                    }
                    shade_prim = prim;
                    Inter it;
                    it.P = origin + direction * t;
                    it.N = G.has_normals ? normalize(interp_normal(S, prim, hv.y, hv.z)) : normalize(mk(0, 0, 0));
                    it.wo = -direction;
                    it.ioro = 0.0f;
                    it.iori = p.iori;
                    it.lobe = p.lobe;
                    it.wi = mk(0, 0, 0);
                    const uint32_t nl = S.num_lights;
                    if (!(nl == 0 || (nl == 1 && G.light >= 0))) {
                        int li;
                        int guard = 0;
                        do {
                            li = (int)p.rng.next_discrete(nl);
                        } while (li == G.light && ++guard < 1 << 20);
                        const LightInfo &L = S.lights[li];
                        Inter c = it;
                        conn_org = it.P;
                        conn_light = (uint32_t)li;
                        conn_T = p.T;
                        if (m.bsdf == LT_BSDF_LAMBERT) {
                            float x, y;
                            sample_disc(p.rng, L.sphere[3], x, y);
                            const v3 cdir = mk(L.sphere[0], L.sphere[1], L.sphere[2]) - c.P;
                            const float dl = length(cdir);
                            const v3 point = rotate_to_world(x, y, dl - L.sphere[3], normalize(cdir));
                            const v3 ldir = normalize(point);
                            c.wi = ldir;
                            const float cosl = dot(ldir, c.N);
                            if (cosl > 0.0f) {
                                n_ref_rays++;
                                const float tl = light_distance(S, L, c.P, ldir, nullptr);
                                if (tl != 0.0f) {
                                    emit_l = true;
                                    l_dir = ldir;
                                    l_f = (alb * kInvPi) * cosl;
                                    l_pdf = cosl * kInvPi;
                                    l_tl = tl;
                                }
                            }
                        }
                        bsdf_sample(m, c, p.rng);
                        const float spdf = bsdf_pdf(m, c);
                        const float cosb = dot(c.wi, c.N);
                        if (spdf != 0.0f && cosb > 0.0f) {
                            n_ref_rays_b++;
                            const float tl = light_distance(S, L, c.P, c.wi, nullptr);
                            if (tl != 0.0f) {
                                emit_b = true;
                                b_dir = c.wi;
                                b_f = m.bsdf == LT_BSDF_LAMBERT ? (alb * kInvPi) * cosb : alb;
                                b_dfa = m.bsdf == LT_BSDF_LAMBERT ? kInvPi * cosb : 1.0f;
                                b_pdf = spdf;
                                b_tl = tl;
                            }
                        }
                    }
                    bsdf_sample(m, it, p.rng);
                    const float pdf = bsdf_pdf(m, it);
                    const v3 f = m.bsdf == LT_BSDF_LAMBERT ? (alb * kInvPi) * dot(it.wi, it.N) : alb;
                    const v3 fs = m.bsdf == LT_BSDF_LAMBERT ? (alb_d * kInvPi) * dot(it.wi, it.N) : alb_d;
                    if constexpr (Src::kAdj) {
                        if (emit_l || emit_b) pend = prim;  // once this bounce's records are traced
                        else albedo_term(gt, src, p.scene, prim, I, delta, C);
                    }
                    p.T = (p.T * f) / pdf;
                    Ts = (Ts * fs) / pdf;
                    if (it.lobe == kLobeSTrans) {
                        it.iori = it.ioro;
                        p.medium = m.medium;
                    }
                    p.iori = it.iori;
                    p.lobe = it.lobe;
                    norg = it.P;
                    ndir = it.wi;
                    ntnear = 0.001f;
                }
                if (p.bounces > A.rr_depth) {  // roulette from the detached throughput
                    const float pr = fmaxf(Ts.x, fmaxf(Ts.y, Ts.z));
                    if (p.rng.next_float() > pr) {
                        done = true;
                    } else {
                        p.T = p.T * (1 / pr);
                        Ts = Ts * (1 / pr);
                    }
                }
            }
            if (!done) {
                p.bounces++;
                if (p.bounces >= A.max_depth) done = true;
                else push = true;
            }
        }
        // slots of this warp: records, queue entries, finishing entries, next
        // work items, then camera-ray entries (reserve_block)
        const uint32_t lane = threadIdx.x & 31u;
        const unsigned below = (1u << lane) - 1u;
        const bool fin = done && (emit_l || emit_b);
        const unsigned m_l = __ballot_sync(0xFFFFFFFFu, emit_l), m_b = __ballot_sync(0xFFFFFFFFu, emit_b);
        const unsigned m_d = __ballot_sync(0xFFFFFFFFu, done), m_p = __ballot_sync(0xFFFFFFFFu, push);
        const unsigned m_f = __ballot_sync(0xFFFFFFFFu, fin);
        const uint32_t okey =
            push ? (ndir.x < 0.0f ? 1u : 0u) | (ndir.y < 0.0f ? 2u : 0u) | (ndir.z < 0.0f ? 4u : 0u) : 8u;
        const Slots sl = reserve_block<true>(W.counters, cur, __popc(m_l) + __popc(m_b), __popc(m_p), __popc(m_f),
                                             __popc(m_d), src.total(), Src::kAdj && Src::kMany ? &gt->other : nullptr,
                                             okey, it++);
        if constexpr (Src::kAdj && Src::kMany) {
            // paths of another scene came: the table's sums go to the gradient
            // arrays and its slots to the new scene's triangles (a block-uniform
            // decision; every add of this round is done)
            if (sl.flag != 0u) {
                gt->flush();
                __syncthreads();
                gt->init();
                if (threadIdx.x == 0) gt->scene = sl.flag - 1u;
                __syncthreads();
            }
        }
        const uint32_t c_base = sl.c, f_base = sl.f, r_base = sl.r, n_regen = sl.n_regen;
        const unsigned long long w_base = sl.w;
        const uint32_t rec_l = emit_l ? c_base + __popc(m_l & below) : kNoRecord;
        const uint32_t rec_b = emit_b ? c_base + __popc(m_l) + __popc(m_b & below) : kNoRecord;
        conn_light |= p.scene << kConnSceneShift;
        if (emit_l && !LT_CHECK(W.counters, rec_l < 2u * cap, kChkRecord, rec_l)) emit_l = false;
        if (emit_b && !LT_CHECK(W.counters, rec_b < 2u * cap, kChkRecord, rec_b)) emit_b = false;
        if (emit_l) {
            st_s(W.cray + 2 * rec_l, make_float4(conn_org.x, conn_org.y, conn_org.z, __uint_as_float(conn_light)));
            st_s(W.cray + 2 * rec_l + 1, make_float4(l_dir.x, l_dir.y, l_dir.z, l_tl));
            st_s(W.crec + 2 * rec_l, make_float4(l_f.x, l_f.y, l_f.z, l_pdf));
            st_s(W.crec + 2 * rec_l + 1, make_float4(conn_T.x, conn_T.y, conn_T.z, __uint_as_float(p.pixel)));
        }
        if (emit_b) {
            st_s(W.cray + 2 * rec_b,
                 make_float4(conn_org.x, conn_org.y, conn_org.z, __uint_as_float(conn_light | kConnectBsdf)));
            st_s(W.cray + 2 * rec_b + 1, make_float4(b_dir.x, b_dir.y, b_dir.z, b_tl));
            st_s(W.crec + 2 * rec_b, make_float4(b_f.x, b_f.y, b_f.z, b_pdf));
            st_s(W.crec + 2 * rec_b + 1, make_float4(conn_T.x, conn_T.y, conn_T.z, __uint_as_float(p.pixel)));
        }
        if constexpr (Src::kAdj) {  // what the trace stage needs for the records' gradient terms
            if (emit_l) st_s(D.aux + rec_l, make_float2(__uint_as_float(shade_prim), l_pdf));  // f / albedo = cos / pi
            if (emit_b) st_s(D.aux + rec_b, make_float2(__uint_as_float(shade_prim), b_dfa));
        }
        bool regen = false;
        if (done) {
            if constexpr (!Src::kAdj) {
                const FilmPtrs &F = src.film(p.scene);
                atomicAdd(F.bounces + p.pixel, p.bounces);
                atomicAdd(F.counts + p.pixel, 1u);
            }
            if (fin) {
                const uint32_t e = f_base + __popc(m_f & below);
                if (!LT_CHECK(W.counters, e < cap, kChkOutSlot, e)) continue;
                st_s(D.fin_id[nxt] + e, make_uint4(p.pixel, p.frame, p.scene, Src::kAdj ? pend : 0u));
                st_s(D.fin_C[nxt] + e, make_float4(C.x, C.y, C.z, 0.0f));
                st_s(D.fin_rec[nxt] + e, make_uint2(rec_l, rec_b));
            } else {
                if constexpr (!Src::kAdj) write_sample(src.samples(p.scene), src.args(p.scene), p.pixel, p.frame, C);
            }
        }
        const uint32_t rank_d = __popc(m_d & below);
        if (done && rank_d < n_regen) {
            unsigned long long local;
            const uint32_t sid = src.locate(w_base + rank_d, local);
            start_path(src.scene(sid), src.args(sid), local, p, norg, ndir, ntnear);
            p.scene = sid;
            C = mk(0, 0, 0);
            Ts = p.T;
            regen = true;
        }
        if (push || regen) {
            const uint32_t qi = push ? sl.qpos : cap - 1u - (r_base + rank_d);
            if (!LT_CHECK(W.counters, qi < cap, kChkOutSlot, qi)) continue;
            write_ray(W.ray[nxt], qi, norg, ntnear, ndir);
            store_path(W.p[nxt], cap, qi, p);
            st3_planes(D.C[nxt], cap, qi, C);
            st3_planes(D.Ts[nxt], cap, qi, Ts);
            st_s(D.rec[nxt] + qi, push ? make_uint2(rec_l, rec_b) : make_uint2(kNoRecord, kNoRecord));
            if constexpr (Src::kAdj) st_s(D.pend[nxt] + qi, push ? pend : kMiss);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_ref_rays += __shfl_xor_sync(0xFFFFFFFFu, n_ref_rays, o);
        n_ref_rays_b += __shfl_xor_sync(0xFFFFFFFFu, n_ref_rays_b, o);
    }
    if ((threadIdx.x & 31u) == 0 && (n_ref_rays | n_ref_rays_b)) {
        atomicAdd(&W.counters->light_rays, (unsigned long long)n_ref_rays);
        atomicAdd(&W.counters->bsdf_rays, (unsigned long long)n_ref_rays_b);
    }
    if constexpr (Src::kAdj) {
        __syncthreads();
        gt->flush();
    }
}

// Film colour sums of the differentiable forward from its per-sample radiance:
// per pixel the samples in frame order, then one addition to the film, so
// the film does not depend on the order in which samples finished.
__global__ void __launch_bounds__(256) k_diff_film(const float *__restrict__ sample_I, RenderArgs A, FilmPtrs F) {
    const uint32_t npix = A.width * A.height;
    const uint32_t spp = (uint32_t)(A.total / npix);
    for (uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < npix; pixel += gridDim.x * blockDim.x) {
        v3 sum = mk(0, 0, 0);
        for (uint32_t s = 0; s < spp; ++s) {
            const size_t item = (size_t)s * npix + pixel;
            sum = sum + mk(ld_s(sample_I + 3 * item), ld_s(sample_I + 3 * item + 1), ld_s(sample_I + 3 * item + 2));
        }
        F.rgb[3 * (size_t)pixel] += sum.x;
        F.rgb[3 * (size_t)pixel + 1] += sum.y;
        F.rgb[3 * (size_t)pixel + 2] += sum.z;
    }
}

// k_diff_film over the pixels of all slots of a batch (slot i owns
// [pbegin[i], pbegin[i] + width * height) of the global pixel sequence).
__device__ __forceinline__ uint32_t locate_pixel(const SceneTable *t, unsigned long long gp, uint32_t &pixel);

__global__ void __launch_bounds__(256) k_diff_film_batch(const SceneTable *t, unsigned long long total_pixels) {
    for (unsigned long long gp = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; gp < total_pixels;
         gp += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t pixel;
        const uint32_t sid = locate_pixel(t, gp, pixel);
        const RenderArgs &A = t->slots[sid].a;
        const FilmPtrs &F = t->slots[sid].f;
        const float *sample_I = t->diff[sid].sample_I;
        const uint32_t npix = A.width * A.height;
        const uint32_t spp = (uint32_t)(A.total / npix);
        v3 sum = mk(0, 0, 0);
        for (uint32_t s = 0; s < spp; ++s) {
            const size_t item = (size_t)s * npix + pixel;
            sum = sum + mk(ld_s(sample_I + 3 * item), ld_s(sample_I + 3 * item + 1), ld_s(sample_I + 3 * item + 2));
        }
        F.rgb[3 * (size_t)pixel] += sum.x;
        F.rgb[3 * (size_t)pixel + 1] += sum.y;
        F.rgb[3 * (size_t)pixel + 2] += sum.z;
    }
}

// Connection rays and their MIS-weighted contributions (EstimateDirect,
// integrator.cpp:281-312; SampleLi/PdfLi, area_light.cpp:58-67,100-109).
//
// The reference takes the closest hit in the whole scene and keeps it if it
// lies on the chosen light. The same answer (up to exact distance ties between
// the light and an occluder) comes cheaper in two steps: k_shade finds the
// closest hit among the light's own triangles and emits only rays that reach
// the light, with that distance; here an occlusion query up to the distance,
// ignoring the light's own geometry, decides the rest. Lights with more than
// kLightBrute triangles (distance -1 in the record) use a full closest-hit query.
template <class State>
__device__ __forceinline__ void resolve_connection(const DevScene &S, const Wavefront &W, const FilmPtrs &F,
                                                   uint32_t idx, uint32_t kl, const State &r, uint32_t npix) {
    const bool is_bsdf = (kl & kConnectBsdf) != 0;
    const LightInfo &L = S.lights[kl & kConnLightMask];
    Hit h;
    if (r.any) {
        if (r.h.prim != kMiss) return;  // occluded
        light_distance(S, L, r.O, r.D, &h);  // the same light hit k_shade found
    } else {
        if (r.h.prim == kMiss) return;
        if (!LT_CHECK(W.counters, r.h.prim < S.num_tris, kChkPrim, r.h.prim)) return;
        if (__ldg(S.tri_geom + r.h.prim) != (uint32_t)L.geom) return;
        h = r.h;
    }
    v3 org = r.O, dir = r.D;
    v3 ip = org + normalize(dir) * h.t;
    v3 dd = ip - org;
    float d2 = dot(dd, dd);
    v3 nrm = normalize(interp_normal(S, h.prim, h.u, h.v));
    float cosl = is_bsdf ? dot(nrm, dir) : dot(nrm, -dir);
    float lpdf = d2 / (fabsf(cosl) * L.area);
    if (lpdf == 0.0f) return;
    float4 r0 = ld_s(W.crec + 2 * idx), r1 = ld_s(W.crec + 2 * idx + 1);
    const uint32_t pixel = __float_as_uint(r1.w);
    v3 f = mk(r0.x, r0.y, r0.z);
    float spdf = r0.w;
    v3 Le = mk(L.radiance[0], L.radiance[1], L.radiance[2]);
    v3 c;
    if (!is_bsdf) c = ((f * Le) * power_heuristic(lpdf, spdf)) / lpdf;
    else c = ((f * Le) * power_heuristic(spdf, lpdf)) / spdf;
    v3 T = mk(r1.x, r1.y, r1.z);
    if (!LT_PIXEL_OK(W, pixel, npix)) return;
    film_contribute(W.counters, F, pixel, T * (c * (float)S.num_lights));
}

// resolve_connection for the differentiable estimator (diff_path's light and
// BSDF samples): the emission is the hit light triangle's parameter, and the
// contribution T * ((f * Le * w) / pdf * numLights) goes to the record's result
// slot (w = 1) for the path's next shade to add in order; a record that does
// not contribute gets w = 0. For the adjoint, a contributing record also
// yields the contribution's derivatives: delta * T * Le * (numLights * (f /
// albedo) * w / pdf) for the shading triangle's albedo and delta * T * f *
// (numLights * w / pdf) for the emission of the light triangle hit. The
// single-scene adjoint adds them to its block's gradient table gt here; the
// batched one writes them to d.gres for the path's next shade to add (its
// table follows the scenes, which only the shade's block-uniform rounds allow).
template <class Src, class State>
__device__ __forceinline__ void resolve_connection_diff(const Src &src, const Wavefront &W, uint32_t idx,
                                                        uint32_t kl, const State &r, TraceGrads *gt) {
    const uint32_t sid = (kl >> kConnSceneShift) & kConnSceneMask;
    const DevScene &S = src.scene(sid);
    const bool is_bsdf = (kl & kConnectBsdf) != 0;
    const LightInfo &L = S.lights[kl & kConnLightMask];
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    Hit h;
    bool visible;
    if (r.any) {
        visible = r.h.prim == kMiss;
        if (visible) light_distance(S, L, r.O, r.D, &h);  // the same light hit k_dshade found
    } else {
        visible = r.h.prim != kMiss && __ldg(S.tri_geom + r.h.prim) == (uint32_t)L.geom;
        h = r.h;
    }
    if (visible) {
        const v3 org = r.O, dir = r.D;
        const v3 ip = org + normalize(dir) * h.t;
        const v3 dd = ip - org;
        const float d2 = dot(dd, dd);
        const v3 nrm = normalize(interp_normal(S, h.prim, h.u, h.v));
        const float cosl = is_bsdf ? dot(nrm, dir) : dot(nrm, -dir);
        const float lpdf = d2 / (fabsf(cosl) * L.area);
        const float4 r0 = ld_s(W.crec + 2 * idx), r1 = ld_s(W.crec + 2 * idx + 1);
        const float spdf = r0.w;
        if (lpdf != 0.0f && spdf != 0.0f) {
            const v3 f = mk(r0.x, r0.y, r0.z);
            const v3 Le = ld3(src.params(sid).emission + 3 * h.prim);
            const v3 T = mk(r1.x, r1.y, r1.z);
            const float fn = (float)S.num_lights;
            v3 c;
            if (!is_bsdf) c = T * ((((f * Le) * power_heuristic(lpdf, spdf)) / lpdf) * fn);
            else c = T * ((((f * Le) * power_heuristic(spdf, lpdf)) / spdf) * fn);
            out = make_float4(c.x, c.y, c.z, 1.0f);
            if constexpr (Src::kAdj) {
                const float2 aux = ld_s(src.d.aux + idx);  // shading triangle, f / albedo
                const uint32_t pixel = __float_as_uint(r1.w);
                const DiffGrads &G = src.grads(sid);
                const v3 Td = T * ld3(G.dI + 3 * (size_t)pixel);
                const float wgt = is_bsdf ? power_heuristic(spdf, lpdf) : power_heuristic(lpdf, spdf);
                const float pdf = is_bsdf ? spdf : lpdf;
                const v3 ga = Td * (Le * (fn * aux.y * wgt / pdf)), ge = Td * (f * (fn * wgt / pdf));
                if constexpr (Src::kMany) {
                    st_s(src.d.gres + 2 * idx, make_float4(ga.x, ga.y, ga.z, __uint_as_float(h.prim)));
                    st_s(src.d.gres + 2 * idx + 1, make_float4(ge.x, ge.y, ge.z, 0.0f));
                } else {
                    gt->add(G.albedo + 3 * (size_t)__float_as_uint(aux.x), ga);
                    gt->add(G.emission + 3 * (size_t)h.prim, ge);
                }
            }
        }
    }
    st_s(src.d.res + idx, out);
}

// Path rays of iteration `cur` (closest hit into W.hits) and, in the same
// persistent launch, the connection records that the previous k_shade wrote
// (parity cur ^ 1; occlusion query or closest hit, then resolve_connection).
// Both come from one launch of k_shade, so one traversal kernel serves them:
// items [0, n) are path rays (queue entries, placed by queue_slot), [n, n + nc)
// connection records, fetched from
// counters->trace_fetch (zeroed by the launch before). Path rays come first so
// that the short connection queries fill the tail.
template <class Src, class B>
__global__ void __launch_bounds__(256, Src::kMany ? 0 : B::kMinBlocks256)
    k_trace(Src src, Wavefront W, int cur, uint32_t coop_limit = 0) {
    const uint32_t n_push = W.counters->count[cur], n_cam = W.counters->rcount[cur];
    const uint32_t n = n_push + n_cam;
    const uint32_t nc = W.counters->ccount[cur ^ 1];
    const uint32_t total = n + nc;
    const uint32_t cap = W.capacity;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.counters->count[cur ^ 1] = 0;  // filled by the next k_shade
        W.counters->rcount[cur ^ 1] = 0;
        W.counters->ccount[cur] = 0;
        W.counters->fcount[cur ^ 1] = 0;  // filled by the next differentiable shade
        W.counters->main_rays += n;
        const uint32_t it = W.counters->trace_launches++;  // one launch per iteration, stream-ordered
        if (it < W.qtrace_cap) W.qtrace[it] = make_uint3(n_push, n_cam, nc);
    }
    if (total <= coop_limit) return;  // k_trace_tail traces this iteration
    LT_STOP_IF_FAILED(W.counters);
    TraceGrads *gt = nullptr;  // the single-scene adjoint's connection terms
    if constexpr (Src::kAdj && !Src::kMany) {
        gt = grad_table<Src, TraceGrads>();
        gt->init();
        __syncthreads();
    }
    const float4 *rays = W.ray[cur];
    Geo g = B::geo(src.scene(0));
    LT_SET_GEO_CHK(g, W.counters);
    typename B::State r;
    typename B::Entry stack[B::kDepth];
    B::idle(r);
    uint32_t idx = 0, kl = 0, n_trav = 0;
    bool bad = false;  // a bound check rejected the current item: nothing is written for it
    for (;;) {
        if (B::done(r)) {
            idx = fetch_next(&W.counters->trace_fetch);
            if (idx >= total) break;
            bad = false;
            if (idx < n) {
                const uint32_t s = queue_slot(idx, n_push, n_cam, cap);
                if (!LT_CHECK(W.counters, s < cap, kChkSlot, s)) {
                    bad = true;
                    continue;
                }
                if (Src::kMany) {
                    const uint32_t sid = ld_s(W.p[cur].flags + s) >> kFlagSceneShift;
                    if (!LT_CHECK(W.counters, src.valid(sid), kChkScene, sid)) {
                        bad = true;
                        continue;
                    }
                    g = B::geo(src.scene(sid));
                    LT_SET_GEO_CHK(g, W.counters);
                }
                float4 a = ld_s(rays + 2 * s), b = ld_s(rays + 2 * s + 1);
                B::start(r, stack, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w, false, 0);
            } else {
                const uint32_t c = idx - n;
                if (!LT_CHECK(W.counters, c < 2u * cap, kChkRecord, c)) {
                    bad = true;
                    continue;
                }
                float4 a = ld_s(W.cray + 2 * c), b = ld_s(W.cray + 2 * c + 1);
                const float tl = b.w;
                kl = __float_as_uint(a.w);
                const uint32_t sid = (kl >> kConnSceneShift) & kConnSceneMask;
                if (!LT_CHECK(W.counters, src.valid(sid), kChkScene, sid)) {
                    bad = true;
                    continue;
                }
                const DevScene &S = src.scene(sid);
                if (!LT_CHECK(W.counters, (kl & kConnLightMask) < S.num_lights, kChkLight, kl & kConnLightMask)) {
                    bad = true;
                    continue;
                }
                if (Src::kMany) {
                    g = B::geo(S);
                    LT_SET_GEO_CHK(g, W.counters);
                }
                const LightInfo &L = S.lights[kl & kConnLightMask];
                if (tl > 0.0f)
                    B::start(r, stack, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), 0.001f, tl, true, (uint32_t)L.geom);
                else
                    B::start(r, stack, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), 0.001f, __int_as_float(0x7f800000),
                             false, 0);
                n_trav++;
            }
        }
        B::run(g, r, stack);
        if (B::done(r) && !bad) {
            if (idx < n) {
                st_s(W.hits + queue_slot(idx, n_push, n_cam, cap),
                     make_float4(r.h.t, r.h.u, r.h.v, __uint_as_float(r.h.prim)));
            } else {
                const uint32_t sid = (kl >> kConnSceneShift) & kConnSceneMask;
                if constexpr (Src::kDiff) resolve_connection_diff(src, W, idx - n, kl, r, gt);
                else resolve_connection(src.scene(sid), W, src.film(sid), idx - n, kl, r,
                                        src.args(sid).width * src.args(sid).height);
            }
        }
    }
    if (n_trav) atomicAdd(&W.counters->light_traversals, (unsigned long long)n_trav);
    if constexpr (Src::kAdj && !Src::kMany) {
        __syncthreads();
        gt->flush();
    }
}

// ------------------------------------------------------------------ small iterations
// The last iterations of a render trace few rays (a 1-spp 1024x1024 frame:
// 50-7,000 paths from its sixth bounce on), and a launch then lasts as long as
// its slowest ray, one dependent node fetch after the other (about 180 us for
// a ray inside the 1.3M-triangle glass mesh). When an iteration has at most
// `coop_limit` rays, k_trace returns at once and k_trace_tail gives every ray
// a warp: each step the warp takes up to 32 entries off the ray's stack in
// shared memory, tests their child boxes (inner nodes) or triangles (leaves)
// in parallel with the closest distance found so far, and pushes the children
// hit; the warp's closest hit (or any occluder) is the ray's. The same
// triangles are tested with the same arithmetic, so the hit is the sequential
// traversal's up to the choice between hits at exactly the same distance.
constexpr int kCoopStack = 1024;     // stack entries per warp
constexpr int kCoopWarps = 8;        // warps per block (256 threads)
constexpr uint32_t kCoopRaysPerWarp = 8;

__device__ __forceinline__ Hit coop_traverse(const Geo &g, v3 O, v3 D, float tnear, float tfar, bool any,
                                             uint32_t skip_geom, int *st) {
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned full = 0xFFFFFFFFu;
    const v3 inv = mk(safe_inv(D.x), safe_inv(D.y), safe_inv(D.z));
    Hit best;
    best.t = tfar;
    best.u = best.v = 0.0f;
    best.prim = kMiss;
    if (lane == 0) st[0] = 0;  // the root (an inner node)
    int sp = 1;                // warp-uniform
    __syncwarp();
    while (sp > 0) {
        // at most 32 entries: each taken entry pushes at most two, so a step
        // grows the stack by at most 32 (to kCoopStack - 96 from at most
        // kCoopStack - 128); above that, one entry per step, depth first, which
        // adds at most the tree's depth (< 64, as the sequential stack holds)
        int m = sp < 32 ? sp : 32;
        if (sp > kCoopStack - 128) m = 1;
        const bool have = (int)lane < m;
        const int node = have ? st[sp - 1 - (int)lane] : 0;
        __syncwarp();
        sp -= m;
        const float tmax = best.t;
        int push0 = 0, push1 = 0, npush = 0;  // children to push, far one first
        Hit mine = best;
        bool occluded = false;
        const bool entry_ok =
            !have || (node >= 0 ? LT_CHECK(LT_GEO_CHK(g), (uint32_t)node < g.num_nodes, kChkNode, node)
                                : LT_CHECK(LT_GEO_CHK(g),
                                           (~(uint32_t)node >> kLeafBits) + (~(uint32_t)node & ((1u << kLeafBits) - 1u)) <=
                                               g.num_tris,
                                           kChkLeaf, ~(uint32_t)node >> kLeafBits));
        if (have && entry_ok && node >= 0) {
            const float4 *nd = g.nodes + 4 * node;
            const float4 n0 = ldg4(nd), n1 = ldg4(nd + 1), n2 = ldg4(nd + 2), n3 = ldg4(nd + 3);
            float t0, t1;
            const bool h0 = slab(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, O, inv, tnear, tmax, t0);
            const bool h1 = slab(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, O, inv, tnear, tmax, t1);
            const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
            if (h0 && h1) {
                npush = 2;
                if (t1 < t0) {
                    push0 = c0;
                    push1 = c1;
                } else {
                    push0 = c1;
                    push1 = c0;
                }
            } else if (h0 || h1) {
                npush = 1;
                push0 = h0 ? c0 : c1;
            }
        } else if (have && entry_ok) {
            const uint32_t code = ~(uint32_t)node;
            const uint32_t first = code >> kLeafBits, count = code & ((1u << kLeafBits) - 1u);
            for (uint32_t k = 0; k < count; ++k) {
                const float4 *tri = g.tris + 3 * (first + k);
                if (!any) {
                    tri_test(tri, O, D, tnear, mine);
                } else if (!occluded) {
                    Hit c = best;
                    tri_test(tri, O, D, tnear, c);
                    if (c.prim != kMiss && !LT_CHECK(LT_GEO_CHK(g), c.prim < g.num_tris, kChkPrim, c.prim)) break;
                    if (c.prim != kMiss && __ldg(g.tri_geom + c.prim) != skip_geom) {
                        occluded = true;
                        mine.prim = c.prim;
                    }
                }
            }
        }
        if (any) {
            const unsigned occ = __ballot_sync(full, occluded);
            if (occ) {
                best.prim = __shfl_sync(full, mine.prim, __ffs(occ) - 1);
                return best;
            }
        } else {
            float tmin = mine.t;
            for (int o = 16; o > 0; o >>= 1) tmin = fminf(tmin, __shfl_xor_sync(full, tmin, o));
            if (tmin < best.t) {  // the lowest lane holding the closest new hit
                const int src = __ffs(__ballot_sync(full, mine.prim != kMiss && mine.t == tmin)) - 1;
                best.t = tmin;
                best.u = __shfl_sync(full, mine.u, src);
                best.v = __shfl_sync(full, mine.v, src);
                best.prim = __shfl_sync(full, mine.prim, src);
            }
        }
        // push: the entries of higher lanes first, so that lane 0's (the top
        // entry's children) end on top
        const unsigned b1 = __ballot_sync(full, npush >= 1), b2 = __ballot_sync(full, npush == 2);
        if (!LT_CHECK(LT_GEO_CHK(g), sp + __popc(b1) + __popc(b2) <= kCoopStack, kChkStack,
                      sp + __popc(b1) + __popc(b2)))
            return best;  // warp-uniform: the ballots are the warp's
        const unsigned above = lane == 31u ? 0u : full << (lane + 1u);
        const int off = sp + __popc(b1 & above) + __popc(b2 & above);
        if (npush == 2) {
            st[off] = push0;
            st[off + 1] = push1;
        } else if (npush == 1) {
            st[off] = push0;
        }
        sp += __popc(b1) + __popc(b2);
        __syncwarp();
    }
    return best;
}

// The rays of an iteration with at most coop_limit of them (k_trace returned):
// one warp per path ray or connection record, fetched from trace_fetch.
template <class Src>
__global__ void __launch_bounds__(kCoopWarps * 32) k_trace_tail(Src src, Wavefront W, int cur, uint32_t coop_limit) {
    const uint32_t n_push = W.counters->count[cur], n_cam = W.counters->rcount[cur];
    const uint32_t n = n_push + n_cam;
    const uint32_t nc = W.counters->ccount[cur ^ 1];
    const uint32_t total = n + nc;
    if (total > coop_limit) return;  // k_trace traced them
    LT_STOP_IF_FAILED(W.counters);
    TraceGrads *gt = nullptr;  // the single-scene adjoint's connection terms
    if constexpr (Src::kAdj && !Src::kMany) {
        gt = grad_table<Src, TraceGrads>();
        gt->init();
        __syncthreads();
    }
    __shared__ int stacks[kCoopWarps][kCoopStack];
    const uint32_t lane = threadIdx.x & 31u;
    int *st = stacks[threadIdx.x >> 5];
    const uint32_t cap = W.capacity;
    uint32_t n_trav = 0;
    for (;;) {
        uint32_t idx = 0;
        if (lane == 0) idx = atomicAdd(&W.counters->trace_fetch, 1u);
        idx = __shfl_sync(0xFFFFFFFFu, idx, 0);
        if (idx >= total) break;
        Trav r;  // the ray and its result, in the form the resolve functions read
        uint32_t kl = 0, s = 0;
        Geo g;
        if (idx < n) {
            s = queue_slot(idx, n_push, n_cam, cap);
            if (!LT_CHECK(W.counters, s < cap, kChkSlot, s)) continue;  // warp-uniform: one item per warp
            const uint32_t sid = Src::kMany ? ld_s(W.p[cur].flags + s) >> kFlagSceneShift : 0u;
            if (!LT_CHECK(W.counters, src.valid(sid), kChkScene, sid)) continue;
            g = geo_of(src.scene(sid));
            LT_SET_GEO_CHK(g, W.counters);
            const float4 a = ld_s(W.ray[cur] + 2 * s), b = ld_s(W.ray[cur] + 2 * s + 1);
            r.O = mk(a.x, a.y, a.z);
            r.D = mk(b.x, b.y, b.z);
            r.any = false;
            r.h = coop_traverse(g, r.O, r.D, a.w, b.w, false, 0, st);
        } else {
            const uint32_t c = idx - n;
            if (!LT_CHECK(W.counters, c < 2u * cap, kChkRecord, c)) continue;
            const float4 a = ld_s(W.cray + 2 * c), b = ld_s(W.cray + 2 * c + 1);
            kl = __float_as_uint(a.w);
            const uint32_t sid = (kl >> kConnSceneShift) & kConnSceneMask;
            if (!LT_CHECK(W.counters, src.valid(sid), kChkScene, sid)) continue;
            const DevScene &S = src.scene(sid);
            if (!LT_CHECK(W.counters, (kl & kConnLightMask) < S.num_lights, kChkLight, kl & kConnLightMask)) continue;
            g = geo_of(S);
            LT_SET_GEO_CHK(g, W.counters);
            const LightInfo &L = S.lights[kl & kConnLightMask];
            r.O = mk(a.x, a.y, a.z);
            r.D = mk(b.x, b.y, b.z);
            r.any = b.w > 0.0f;
            r.h = coop_traverse(g, r.O, r.D, 0.001f, r.any ? b.w : __int_as_float(0x7f800000), r.any,
                                (uint32_t)L.geom, st);
            n_trav++;
        }
        if (lane == 0) {
            if (idx < n) {
                st_s(W.hits + s, make_float4(r.h.t, r.h.u, r.h.v, __uint_as_float(r.h.prim)));
            } else {
                const uint32_t sid = (kl >> kConnSceneShift) & kConnSceneMask;
                if constexpr (Src::kDiff) resolve_connection_diff(src, W, idx - n, kl, r, gt);
                else resolve_connection(src.scene(sid), W, src.film(sid), idx - n, kl, r,
                                        src.args(sid).width * src.args(sid).height);
            }
        }
        __syncwarp();
    }
    if (lane == 0 && n_trav) atomicAdd(&W.counters->light_traversals, (unsigned long long)n_trav);
    if constexpr (Src::kAdj && !Src::kMany) {
        __syncthreads();
        gt->flush();
    }
}

// While-node condition of a captured wavefront loop (one thread): continue
// while queue `cur` holds paths; give up with error 2 at the iteration limit.
__global__ void k_loop_condition(WaveCounters *c, const SceneTable *t, cudaGraphConditionalHandle h, int cur,
                                 uint32_t iters) {
    c->iterations += iters;
    unsigned int more = c->count[cur] != 0u || c->rcount[cur] != 0u || c->ccount[cur ^ 1] != 0u;
    if (LT_CHECKS && c->check != 0u) more = 0;  // a bound check failed: the host reports it
    if (more && c->iterations >= t->iteration_limit) {
        c->error = 2;
        more = 0;
    }
    cudaGraphSetConditional(h, more);
}

// counts += spp for every pixel (render with max_depth 0: the bounce loop never runs)
__global__ void k_add_counts(FilmPtrs F, uint32_t npix, uint32_t spp) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x)
        F.counts[i] += spp;
}

// ------------------------------------------------------------------ differentiable rendering
// Extension with no reference counterpart: gradients of an image loss with
// respect to per-triangle albedo, per-triangle emission and per-medium
// sigma_a / sigma_s, by path replay (Vicini, Speierer, Jakob, "Path Replay
// Backpropagation", SIGGRAPH 2021). The estimator is the render loop above with
// three changes that make it a smooth function of the parameters: albedo and
// emission come from per-triangle arrays, media use the RGB form (distance
// sampled with the mean of a detached sigma_s, weight = transmittance x sigma_s
// / pdf), and the roulette probability comes from a detached throughput Ts
// computed with the detached parameter copies. At the detached values the
// paths are the same as a plain render's; finite differences that keep the
// detached copies fixed differentiate the same function as the adjoint.
//
// One thread replays one (pixel, frame) sample from its seed: pass 1 collects
// the path's radiance I, pass 2 replays it again and, at every factor w that
// depends on a parameter, adds delta * (I - C) * dlog(w)/dtheta, where C is the
// radiance collected before w applies; every emission term e adds
// delta * T * de/dtheta.

constexpr int kMediaAcc = 4;  // media whose gradients are summed in registers

__device__ __forceinline__ Hit trace_all(const DevScene &S, v3 O, v3 D, float tnear, float tfar, bool any,
                                         uint32_t skip_geom) {
    const Geo g = geo_of(S);
    Trav r;
    int stack[kStack];
    trav_start(r, LocalStack{stack}, O, D, tnear, tfar, any, skip_geom);
    do {
        traverse(g, r, LocalStack{stack});
    } while (r.node != kSentinel);
    return r.h;
}

// Is the closest hit along (P, dir) on light L? On success h is the light hit.
__device__ __forceinline__ bool diff_light_visible(const DevScene &S, const LightInfo &L, v3 P, v3 dir, Hit &h) {
    float tl = light_distance(S, L, P, dir, &h);
    if (tl == 0.0f) return false;
    if (tl > 0.0f) return trace_all(S, P, dir, 0.001f, tl, true, (uint32_t)L.geom).prim == kMiss;
    h = trace_all(S, P, dir, 0.001f, __int_as_float(0x7f800000), false, 0);
    return h.prim != kMiss && __ldg(S.tri_geom + h.prim) == (uint32_t)L.geom;
}

// Per-thread sums of gradient terms keyed by triangle (direct mapped). A
// pixel's samples keep hitting the same few triangles, so most additions stay
// in the thread; the atomics happen when an entry is evicted and at the end.
template <int N> struct GradCache {
    uint32_t key[N];
    v3 val[N];
    __device__ __forceinline__ void init() {
        for (int i = 0; i < N; ++i) key[i] = kMiss;
    }
    __device__ __forceinline__ void add(float *base, uint32_t prim, v3 v) {
        int s = (int)(prim % N);
        if (key[s] == prim) {
            val[s] = val[s] + v;
            return;
        }
        if (key[s] != kMiss) add3(base + 3 * key[s], val[s]);
        key[s] = prim;
        val[s] = v;
    }
    __device__ __forceinline__ void flush(float *base) {
        for (int i = 0; i < N; ++i) {
            if (key[i] != kMiss) add3(base + 3 * key[i], val[i]);
            key[i] = kMiss;
        }
    }
};
using AlbedoCache = GradCache<4>;
using EmissionCache = GradCache<2>;

__device__ __forceinline__ void add_medium(const DiffGrads &G, float *acc, int mi, v3 ga, v3 gs) {
    if (mi < kMediaAcc) {
        acc[6 * mi] += ga.x; acc[6 * mi + 1] += ga.y; acc[6 * mi + 2] += ga.z;
        acc[6 * mi + 3] += gs.x; acc[6 * mi + 4] += gs.y; acc[6 * mi + 5] += gs.z;
    } else {
        add3(G.sigma_a + 3 * mi, ga);
        add3(G.sigma_s + 3 * mi, gs);
    }
}

template <bool kGrad>
__device__ v3 diff_path(const DevScene &S, const DiffParams &P, const DiffGrads &G, const RenderArgs &A,
                        unsigned long long item, v3 I, v3 delta, float *macc, AlbedoCache &ca, EmissionCache &ce,
                        uint32_t &bounces_out) {
    Path p;
    v3 org, dir;
    float tnear;
    start_path(S, A, item, p, org, dir, tnear);
    v3 Ts = p.T;
    v3 C = mk(0, 0, 0);
    const float inf = __int_as_float(0x7f800000);
    uint32_t bounces = 0;
    for (; bounces < A.max_depth; ++bounces) {
        Hit h = trace_all(S, org, dir, tnear, inf, false, 0);
        if (h.prim == kMiss) {
            C = C + p.T * S.background;
            break;
        }
        const uint32_t prim = h.prim;
        v3 origin = org, direction = normalize(dir);
        bool hit_surface = true;
        if (p.medium >= 0) {
            const int mi = p.medium;
            const MediumInfo M = S.meds[mi];
            v3 sa = ld3(P.sigma_a + 3 * mi), ss = ld3(P.sigma_s + 3 * mi);
            v3 sa_d = ld3(P.sigma_a_s + 3 * mi), ss_d = ld3(P.sigma_s_s + 3 * mi);
            float dist;
            bool scat = false;
            v3 w, ws;
            if (M.type == LT_MEDIUM_NON_SCATTERING) {
                dist = h.t;
                w = mk(expf(-sa.x * dist), expf(-sa.y * dist), expf(-sa.z * dist));
                ws = mk(expf(-sa_d.x * dist), expf(-sa_d.y * dist), expf(-sa_d.z * dist));
            } else {
                float sbar = M.type == LT_MEDIUM_ISOTROPIC ? ss_d.x : (ss_d.x + ss_d.y + ss_d.z) / 3.0f;
                dist = -logf(p.rng.next_float()) / sbar;
                scat = dist < h.t;
                if (!scat) dist = h.t;
                w = mk(expf(-(sa.x + ss.x - sbar) * dist), expf(-(sa.y + ss.y - sbar) * dist),
                       expf(-(sa.z + ss.z - sbar) * dist));
                ws = mk(expf(-(sa_d.x + ss_d.x - sbar) * dist), expf(-(sa_d.y + ss_d.y - sbar) * dist),
                        expf(-(sa_d.z + ss_d.z - sbar) * dist));
                if (scat) {
                    w = w * (ss / sbar);
                    ws = ws * (ss_d / sbar);
                }
            }
            if (kGrad) {
                v3 R = (I - C) * delta;
                v3 ga = R * (-dist);
                v3 gs = mk(0, 0, 0);
                if (M.type != LT_MEDIUM_NON_SCATTERING)
                    gs = mk(R.x * (-dist + (scat ? 1.0f / ss.x : 0.0f)), R.y * (-dist + (scat ? 1.0f / ss.y : 0.0f)),
                            R.z * (-dist + (scat ? 1.0f / ss.z : 0.0f)));
                add_medium(G, macc, mi, ga, gs);
            }
            p.T = p.T * w;
            Ts = Ts * ws;
            if (scat) {
                hit_surface = false;
                org = origin + direction * dist;
                dir = M.type == LT_MEDIUM_HG ? hg_sample(p.rng, direction, M.g) : uniform_sphere(p.rng);
                tnear = 0.001f;
            }
        }
        if (hit_surface) {
            const GeomInfo Gi = S.geoms[__ldg(S.tri_geom + prim)];
            const MaterialInfo m = S.mats[Gi.material];
            const v3 alb = ld3(P.albedo + 3 * prim), alb_d = ld3(P.albedo_s + 3 * prim);
            if ((bounces == 0 || (p.lobe & kLobeSpecular) != 0) && Gi.light >= 0) {
                C = C + p.T * ld3(P.emission + 3 * prim);
                if (kGrad) ce.add(G.emission, prim, p.T * delta);
            }
            Inter it;
            it.P = origin + direction * h.t;
            it.N = Gi.has_normals ? normalize(interp_normal(S, prim, h.u, h.v)) : normalize(mk(0, 0, 0));
            it.wo = -direction;
            it.ioro = 0.0f;
            it.iori = p.iori;
            it.lobe = p.lobe;
            it.wi = mk(0, 0, 0);
            const uint32_t nl = S.num_lights;
            if (!(nl == 0 || (nl == 1 && Gi.light >= 0))) {
                int li;
                int guard = 0;
                do {
                    li = (int)p.rng.next_discrete(nl);
                } while (li == Gi.light && ++guard < 1 << 20);
                const LightInfo &L = S.lights[li];
                const float fn = (float)nl;
                Inter c = it;
                if (m.bsdf == LT_BSDF_LAMBERT) {
                    float x, y;
                    sample_disc(p.rng, L.sphere[3], x, y);
                    v3 cdir = mk(L.sphere[0], L.sphere[1], L.sphere[2]) - c.P;
                    float dl = length(cdir);
                    v3 point = rotate_to_world(x, y, dl - L.sphere[3], normalize(cdir));
                    v3 ldir = normalize(point);
                    c.wi = ldir;
                    float cosl = dot(ldir, c.N);
                    Hit lh;
                    if (cosl > 0.0f && diff_light_visible(S, L, c.P, ldir, lh)) {
                        float spdf = cosl * kInvPi;
                        v3 ip = c.P + normalize(ldir) * lh.t;
                        v3 dd = ip - c.P;
                        float lpdf = dot(dd, dd) / (fabsf(dot(normalize(interp_normal(S, lh.prim, lh.u, lh.v)), -ldir)) * L.area);
                        if (lpdf != 0.0f && spdf != 0.0f) {
                            v3 Li = ld3(P.emission + 3 * lh.prim);
                            v3 f = (alb * kInvPi) * cosl;
                            float wgt = power_heuristic(lpdf, spdf);
                            C = C + p.T * ((((f * Li) * wgt) / lpdf) * fn);
                            if (kGrad) {
                                v3 Td = p.T * delta;
                                ca.add(G.albedo, prim, Td * (Li * (fn * (cosl * kInvPi) * wgt / lpdf)));
                                ce.add(G.emission, lh.prim, Td * (f * (fn * wgt / lpdf)));
                            }
                        }
                    }
                }
                bsdf_sample(m, c, p.rng);
                float spdf = bsdf_pdf(m, c);
                float cosb = dot(c.wi, c.N);
                Hit bh;
                if (spdf != 0.0f && cosb > 0.0f && diff_light_visible(S, L, c.P, c.wi, bh)) {
                    v3 ip = c.P + normalize(c.wi) * bh.t;
                    v3 dd = ip - c.P;
                    float lpdf = dot(dd, dd) / (fabsf(dot(normalize(interp_normal(S, bh.prim, bh.u, bh.v)), c.wi)) * L.area);
                    if (lpdf != 0.0f) {
                        v3 Le = ld3(P.emission + 3 * bh.prim);
                        float dfa = m.bsdf == LT_BSDF_LAMBERT ? kInvPi * cosb : 1.0f;  // f = albedo * dfa
                        v3 f = m.bsdf == LT_BSDF_LAMBERT ? (alb * kInvPi) * cosb : alb;
                        float wgt = power_heuristic(spdf, lpdf);
                        C = C + p.T * ((((f * Le) * wgt) / spdf) * fn);
                        if (kGrad) {
                            v3 Td = p.T * delta;
                            ca.add(G.albedo, prim, Td * (Le * (fn * dfa * wgt / spdf)));
                            ce.add(G.emission, bh.prim, Td * (f * (fn * wgt / spdf)));
                        }
                    }
                }
            }
            bsdf_sample(m, it, p.rng);
            float pdf = bsdf_pdf(m, it);
            v3 f = m.bsdf == LT_BSDF_LAMBERT ? (alb * kInvPi) * dot(it.wi, it.N) : alb;
            v3 fs = m.bsdf == LT_BSDF_LAMBERT ? (alb_d * kInvPi) * dot(it.wi, it.N) : alb_d;
            if (kGrad) {
                v3 R = (I - C) * delta;
                ca.add(G.albedo, prim, mk(alb.x > 0.0f ? R.x / alb.x : 0.0f, alb.y > 0.0f ? R.y / alb.y : 0.0f,
                                             alb.z > 0.0f ? R.z / alb.z : 0.0f));
            }
            p.T = (p.T * f) / pdf;
            Ts = (Ts * fs) / pdf;
            if (it.lobe == kLobeSTrans) {
                it.iori = it.ioro;
                p.medium = m.medium;
            }
            p.iori = it.iori;
            p.lobe = it.lobe;
            org = it.P;
            dir = it.wi;
            tnear = 0.001f;
        }
        if (bounces > A.rr_depth) {
            float pr = fmaxf(Ts.x, fmaxf(Ts.y, Ts.z));  // detached roulette probability
            if (p.rng.next_float() > pr) break;
            p.T = p.T * (1 / pr);
            Ts = Ts * (1 / pr);
        }
    }
    bounces_out = bounces;
    return C;
}

// Next 32 work items for the calling warp (all lanes call it together).
__device__ __forceinline__ unsigned long long fetch_chunk(unsigned long long *fetch);

// Gradient terms of samples [s0, s1) of one pixel.
__device__ __forceinline__ void diff_adjoint_samples(const DevScene &S, const DiffParams &P, const RenderArgs &A,
                                                     const DiffGrads &G, uint32_t pixel, uint32_t s0, uint32_t s1,
                                                     float *macc, AlbedoCache &ca, EmissionCache &ce) {
    const uint32_t npix = A.width * A.height;
    const v3 delta = ld3(G.dI + 3 * (size_t)pixel);
    if (is_black(delta)) return;
    for (uint32_t s = s0; s < s1; ++s) {
        const unsigned long long item = (unsigned long long)s * npix + pixel;
        uint32_t b = 0;
        const v3 I = G.sample_I ? ld3(G.sample_I + 3 * item)
                                : diff_path<false>(S, P, G, A, item, mk(0, 0, 0), mk(0, 0, 0), macc, ca, ce, b);
        diff_path<true>(S, P, G, A, item, I, delta, macc, ca, ce, b);
    }
}

// Work items of the adjoint: a pixel's samples in chunks of
// kAdjointChunkSamples, taken from a shared counter 32 at a time per warp, so
// that no thread is left with a whole pixel's worth of paths at the end; the
// consecutive samples of a chunk keep hitting the same triangles, which the
// per-thread gradient caches exploit.
constexpr uint32_t kAdjointChunk = kAdjointChunkSamples;

__global__ void __launch_bounds__(128) k_diff_adjoint(DevScene S, DiffParams P, RenderArgs A, DiffGrads G,
                                                     uint32_t num_media, unsigned long long *fetch) {
    float macc[6 * kMediaAcc];
    for (int k = 0; k < 6 * kMediaAcc; ++k) macc[k] = 0.0f;
    AlbedoCache ca;
    EmissionCache ce;
    ca.init();
    ce.init();
    const uint32_t npix = A.width * A.height;
    const uint32_t spp = (uint32_t)(A.total / npix);
    const uint32_t chunks = (spp + kAdjointChunk - 1) / kAdjointChunk;
    const uint32_t cw = G.x1 - G.x0, ch = G.y1 - G.y0;
    const unsigned long long items = (unsigned long long)cw * ch * chunks;
    for (;;) {
        const unsigned long long base = fetch_chunk(fetch);
        if (base >= items) break;
        const unsigned long long it = base + (threadIdx.x & 31u);
        if (it < items) {
            const uint32_t k = (uint32_t)(it / chunks), c = (uint32_t)(it - (unsigned long long)k * chunks);
            const uint32_t pixel = (G.y0 + k / cw) * A.width + G.x0 + k % cw;
            const uint32_t s0 = c * kAdjointChunk, s1 = s0 + kAdjointChunk < spp ? s0 + kAdjointChunk : spp;
            diff_adjoint_samples(S, P, A, G, pixel, s0, s1, macc, ca, ce);
        }
    }
    ca.flush(G.albedo);
    ce.flush(G.emission);
    // medium gradients: warp sums, one atomic per warp and component
    for (int k = 0; k < 6 * kMediaAcc; ++k) {
        if (k / 6 >= (int)num_media) break;
        float v = macc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if ((threadIdx.x & 31u) == 0 && v != 0.0f) {
            int mi = k / 6, c = k % 6;
            atomicAdd(c < 3 ? G.sigma_a + 3 * mi + c : G.sigma_s + 3 * mi + (c - 3), v);
        }
    }
}

// ---- batched differentiable rendering (lt_render_diff_batch / lt_render_adjoint_batch)
// The pixels of all slots form one sequence (slot i owns [pbegin[i],
// pbegin[i] + width * height)); warps take 32 consecutive pixels at a time
// from t->fetch, so scenes of any size and spp share one persistent launch.

// The slot that owns global pixel gp: the last i with pbegin[i] <= gp.
__device__ __forceinline__ uint32_t locate_pixel(const SceneTable *t, unsigned long long gp, uint32_t &pixel) {
    uint32_t lo = 0, hi = t->count;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (t->pbegin[mid] <= gp) lo = mid;
        else hi = mid;
    }
    pixel = (uint32_t)(gp - t->pbegin[lo]);
    return lo;
}

// Next 32-pixel chunk for the calling warp (all lanes call it together).
__device__ __forceinline__ unsigned long long fetch_chunk(unsigned long long *fetch) {
    unsigned long long base = 0;
    if ((threadIdx.x & 31u) == 0) base = atomicAdd(fetch, 32ull);
    return __shfl_sync(0xFFFFFFFFu, base, 0);
}

// Adds a thread's cached gradient terms to slot d's arrays and clears them.
__device__ __forceinline__ void flush_diff_slot(const DiffSlot &d, float *macc, AlbedoCache &ca, EmissionCache &ce) {
    ca.flush(d.g.albedo);
    ce.flush(d.g.emission);
    for (int k = 0; k < 6 * kMediaAcc; ++k) {
        if (k / 6 >= (int)d.num_media) break;
        if (macc[k] != 0.0f) {
            int mi = k / 6, c = k % 6;
            atomicAdd(c < 3 ? d.g.sigma_a + 3 * mi + c : d.g.sigma_s + 3 * mi + (c - 3), macc[k]);
        }
        macc[k] = 0.0f;
    }
}

// Register budget: six 128-thread blocks per SM (80 registers, some spilled),
// as the single-scene adjoint runs: measured 5% faster than the compiler's
// 96 registers (five blocks) on the batched adjoints of the 64-scene workload.
__global__ void __launch_bounds__(128, 6) k_diff_adjoint_batch(SceneTable *t) {
    float macc[6 * kMediaAcc];
    for (int k = 0; k < 6 * kMediaAcc; ++k) macc[k] = 0.0f;
    AlbedoCache ca;
    EmissionCache ce;
    ca.init();
    ce.init();
    uint32_t held = 0xFFFFFFFFu;  // slot whose gradients the caches hold
    const unsigned long long total = t->total_items;
    for (;;) {
        const unsigned long long base = fetch_chunk(&t->fetch);
        if (base >= total) break;
        const unsigned long long gi = base + (threadIdx.x & 31u);
        if (gi < total) {
            // the slot of sample chunk gi: the last i with ibegin[i] <= gi
            uint32_t lo = 0, hi = t->count;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (t->ibegin[mid] <= gi) lo = mid;
                else hi = mid;
            }
            const uint32_t sid = lo;
            if (sid != held) {
                if (held != 0xFFFFFFFFu) flush_diff_slot(t->diff[held], macc, ca, ce);
                held = sid;
            }
            const SceneSlot &sl = t->slots[sid];
            const DiffSlot &d = t->diff[sid];
            const uint32_t npix = sl.a.width * sl.a.height;
            const uint32_t spp = (uint32_t)(sl.a.total / npix);
            const uint32_t chunks = (spp + kAdjointChunk - 1) / kAdjointChunk;
            const unsigned long long local = gi - t->ibegin[sid];
            const uint32_t pixel = (uint32_t)(local / chunks), c = (uint32_t)(local - (unsigned long long)pixel * chunks);
            const uint32_t s0 = c * kAdjointChunk, s1 = s0 + kAdjointChunk < spp ? s0 + kAdjointChunk : spp;
            diff_adjoint_samples(sl.s, d.p, sl.a, d.g, pixel, s0, s1, macc, ca, ce);
        }
    }
    if (held != 0xFFFFFFFFu) flush_diff_slot(t->diff[held], macc, ca, ce);
}

}  // namespace

// Rays of an iteration up to which k_trace_tail traces it on `blocks` blocks.
static uint32_t coop_limit(int blocks) { return (uint32_t)blocks * kCoopWarps * kCoopRaysPerWarp; }

template <class F>
static int blocks_for(F kernel, int threads, int sms, size_t smem = 0) {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem);
    return sms * (b > 0 ? b : 1);
}

// dynamic shared memory of a traversal kernel with `threads` threads per block
template <class B>
static size_t trav_smem(int threads) {
    return (size_t)B::kSharedBytesPerThread * (size_t)threads;
}

void query_launch_shape(int device, bool batch, LaunchShape *out) {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    const int sms = prop.multiProcessorCount;
    out->sms = sms;
    const bool w8 = out->bvh_width == 8, w4 = out->bvh_width == 4;
    const int tt = out->trace_threads;
    if (batch) {
        out->trace_blocks = w8   ? blocks_for(k_trace<ManyScenes, Bvh8>, tt, sms, trav_smem<Bvh8>(tt))
                            : w4 ? blocks_for(k_trace<ManyScenes, Bvh4>, tt, sms, trav_smem<Bvh4>(tt))
                                 : blocks_for(k_trace<ManyScenes, Bvh2>, tt, sms, trav_smem<Bvh2>(tt));
        out->shade_blocks = blocks_for(k_shade<ManyScenes>, out->shade_threads, sms);
    } else {
        out->trace_blocks = w8   ? blocks_for(k_trace<OneScene, Bvh8>, tt, sms, trav_smem<Bvh8>(tt))
                            : w4 ? blocks_for(k_trace<OneScene, Bvh4>, tt, sms, trav_smem<Bvh4>(tt))
                                 : blocks_for(k_trace<OneScene, Bvh2>, tt, sms, trav_smem<Bvh2>(tt));
        out->shade_blocks = blocks_for(k_shade<OneScene>, out->shade_threads, sms);
    }
    out->tail_blocks = batch ? blocks_for(k_trace_tail<ManyScenes>, kCoopWarps * 32, sms)
                             : blocks_for(k_trace_tail<OneScene>, kCoopWarps * 32, sms);
    out->coop_limit = out->bvh_width == 2 ? coop_limit(out->tail_blocks) : 0u;
    out->dtail_blocks = blocks_for(k_trace_tail<DiffOne>, kCoopWarps * 32, sms);
    out->dtail_batch_blocks = blocks_for(k_trace_tail<DiffMany>, kCoopWarps * 32, sms);
    out->atail_blocks = blocks_for(k_trace_tail<AdjOne>, kCoopWarps * 32, sms);
    out->atail_batch_blocks = blocks_for(k_trace_tail<AdjMany>, kCoopWarps * 32, sms);
    out->isect_blocks = w8   ? blocks_for(k_intersect<Bvh8>, 128, sms, trav_smem<Bvh8>(128))
                        : w4 ? blocks_for(k_intersect<Bvh4>, 128, sms, trav_smem<Bvh4>(128))
                             : blocks_for(k_intersect<Bvh2>, 128, sms, trav_smem<Bvh2>(128));
    out->diff_blocks = blocks_for(k_diff_adjoint, 128, sms);
    out->dtrace_blocks = blocks_for(k_trace<DiffOne, Bvh2>, 256, sms, trav_smem<Bvh2>(256));
    out->dshade_blocks = blocks_for(k_dshade<DiffOne>, 256, sms);
    out->dtrace_batch_blocks = blocks_for(k_trace<DiffMany, Bvh2>, 256, sms, trav_smem<Bvh2>(256));
    out->dshade_batch_blocks = blocks_for(k_dshade<DiffMany>, 256, sms);
    out->diff_adj_batch_blocks = blocks_for(k_diff_adjoint_batch, 128, sms);
    out->atrace_blocks = blocks_for(k_trace<AdjOne, Bvh2>, 256, sms, trav_smem<Bvh2>(256));
    out->ashade_blocks = blocks_for(k_dshade<AdjOne>, 256, sms);
    out->atrace_batch_blocks = blocks_for(k_trace<AdjMany, Bvh2>, 256, sms, trav_smem<Bvh2>(256));
    out->ashade_batch_blocks = blocks_for(k_dshade<AdjMany>, 256, sms);
}

cudaError_t preload_wave_kernels() {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k_raygen<OneScene>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_trace<OneScene, Bvh2>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_trace<OneScene, Bvh4>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_trace<OneScene, Bvh8>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_shade<OneScene>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_trace_tail<OneScene>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_add_counts);
    return e;
}

cudaError_t launch_dwave_init(const DevScene &s, const DiffParams &p, const DiffWave &d, const Wavefront &w,
                              const RenderArgs &a, const FilmPtrs &f, const LaunchShape &ls, cudaStream_t st) {
    k_raygen<DiffOne><<<ls.dshade_blocks, 256, 0, st>>>(DiffOne{s, a, f, p, d}, w);
    return cudaGetLastError();
}

cudaError_t launch_dwave_stage(int stage, const DevScene &s, const DiffParams &p, const DiffWave &d,
                               const Wavefront &w, const RenderArgs &a, const FilmPtrs &f, int cur,
                               const LaunchShape &ls, cudaStream_t st) {
    const DiffOne src{s, a, f, p, d};
    if (stage == kStageTrace) {
        const uint32_t coop = coop_limit(ls.dtail_blocks);
        k_trace<DiffOne, Bvh2><<<ls.dtrace_blocks, 256, trav_smem<Bvh2>(256), st>>>(src, w, cur, coop);
        k_trace_tail<DiffOne><<<ls.dtail_blocks, kCoopWarps * 32, 0, st>>>(src, w, cur, coop);
    } else {
        k_dshade<DiffOne><<<ls.dshade_blocks, 256, 0, st>>>(src, w, cur);
    }
    return cudaGetLastError();
}

cudaError_t launch_dwave_batch_init(const SceneTable *t, const DiffWave &d, const Wavefront &w, const LaunchShape &ls,
                                    cudaStream_t st) {
    k_raygen<DiffMany><<<ls.dshade_batch_blocks, 256, 0, st>>>(DiffMany{t, d}, w);
    return cudaGetLastError();
}

cudaError_t launch_dwave_batch_stage(int stage, const SceneTable *t, const DiffWave &d, const Wavefront &w, int cur,
                                     const LaunchShape &ls, cudaStream_t st) {
    const DiffMany src{t, d};
    if (stage == kStageTrace) {
        const uint32_t coop = coop_limit(ls.dtail_batch_blocks);
        k_trace<DiffMany, Bvh2><<<ls.dtrace_batch_blocks, 256, trav_smem<Bvh2>(256), st>>>(src, w, cur, coop);
        k_trace_tail<DiffMany><<<ls.dtail_batch_blocks, kCoopWarps * 32, 0, st>>>(src, w, cur, coop);
    } else {
        k_dshade<DiffMany><<<ls.dshade_batch_blocks, 256, 0, st>>>(src, w, cur);
    }
    return cudaGetLastError();
}

cudaError_t launch_awave_init(const DevScene &s, const DiffParams &p, const DiffWave &d, const DiffGrads &g,
                              const Wavefront &w, const RenderArgs &a, const LaunchShape &ls, cudaStream_t st) {
    k_raygen<AdjOne><<<ls.ashade_blocks, 256, 0, st>>>(AdjOne{s, a, p, d, g}, w);
    return cudaGetLastError();
}

cudaError_t launch_awave_stage(int stage, const DevScene &s, const DiffParams &p, const DiffWave &d,
                               const DiffGrads &g, const Wavefront &w, const RenderArgs &a, int cur,
                               const LaunchShape &ls, cudaStream_t st) {
    const AdjOne src{s, a, p, d, g};
    if (stage == kStageTrace) {
        const uint32_t coop = coop_limit(ls.atail_blocks);
        k_trace<AdjOne, Bvh2><<<ls.atrace_blocks, 256, trav_smem<Bvh2>(256), st>>>(src, w, cur, coop);
        k_trace_tail<AdjOne><<<ls.atail_blocks, kCoopWarps * 32, 0, st>>>(src, w, cur, coop);
    } else {
        k_dshade<AdjOne><<<ls.ashade_blocks, 256, 0, st>>>(src, w, cur);
    }
    return cudaGetLastError();
}

cudaError_t launch_awave_batch_init(const SceneTable *t, const DiffWave &d, const Wavefront &w, const LaunchShape &ls,
                                    cudaStream_t st) {
    k_raygen<AdjMany><<<ls.ashade_batch_blocks, 256, 0, st>>>(AdjMany{t, d}, w);
    return cudaGetLastError();
}

cudaError_t launch_awave_batch_stage(int stage, const SceneTable *t, const DiffWave &d, const Wavefront &w, int cur,
                                     const LaunchShape &ls, cudaStream_t st) {
    const AdjMany src{t, d};
    if (stage == kStageTrace) {
        const uint32_t coop = coop_limit(ls.atail_batch_blocks);
        k_trace<AdjMany, Bvh2><<<ls.atrace_batch_blocks, 256, trav_smem<Bvh2>(256), st>>>(src, w, cur, coop);
        k_trace_tail<AdjMany><<<ls.atail_batch_blocks, kCoopWarps * 32, 0, st>>>(src, w, cur, coop);
    } else {
        k_dshade<AdjMany><<<ls.ashade_batch_blocks, 256, 0, st>>>(src, w, cur);
    }
    return cudaGetLastError();
}

cudaError_t launch_diff_film_batch(const SceneTable *t, unsigned long long total_pixels, int sms, cudaStream_t st) {
    if (total_pixels == 0) return cudaSuccess;
    k_diff_film_batch<<<sms * 8, 256, 0, st>>>(t, total_pixels);
    return cudaGetLastError();
}

cudaError_t launch_diff_film(const float *sample_I, const RenderArgs &a, const FilmPtrs &f, cudaStream_t st) {
    const uint32_t npix = a.width * a.height;
    if (npix == 0 || a.total == 0) return cudaSuccess;
    const uint32_t blocks = (npix + 255) / 256 < 65535 ? (npix + 255) / 256 : 65535;
    k_diff_film<<<blocks, 256, 0, st>>>(sample_I, a, f);
    return cudaGetLastError();
}

cudaError_t launch_diff_adjoint(const DevScene &s, const DiffParams &p, const RenderArgs &a, const DiffGrads &g,
                                uint32_t num_media, unsigned long long *fetch, const LaunchShape &ls,
                                cudaStream_t st) {
    if (a.total == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k_diff_adjoint<<<ls.diff_blocks, 128, 0, st>>>(s, p, a, g, num_media, fetch);
    return cudaGetLastError();
}

cudaError_t launch_diff_adjoint_batch(SceneTable *t, const LaunchShape &ls, cudaStream_t st) {
    k_diff_adjoint_batch<<<ls.diff_adj_batch_blocks, 128, 0, st>>>(t);
    return cudaGetLastError();
}

cudaError_t launch_intersect(const DevScene &s, const float4 *rays, float4 *hits, unsigned long long n,
                             uint32_t *fetch, const LaunchShape &ls, cudaStream_t st) {
    const unsigned long long kChunk = 1ull << 30;
    for (unsigned long long off = 0; off < n; off += kChunk) {
        uint32_t m = (uint32_t)(n - off < kChunk ? n - off : kChunk);
        cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
        unsigned long long need = (m + 127) / 128;
        int blocks = (int)(need < (unsigned long long)ls.isect_blocks ? need : ls.isect_blocks);
        if (ls.bvh_width == 8)
            k_intersect<Bvh8><<<blocks, 128, trav_smem<Bvh8>(128), st>>>(s, rays + 2 * off, hits + off, m, fetch);
        else if (ls.bvh_width == 4)
            k_intersect<Bvh4><<<blocks, 128, trav_smem<Bvh4>(128), st>>>(s, rays + 2 * off, hits + off, m, fetch);
        else
            k_intersect<Bvh2><<<blocks, 128, trav_smem<Bvh2>(128), st>>>(s, rays + 2 * off, hits + off, m, fetch);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_add_counts(const FilmPtrs &f, uint32_t npix, uint32_t spp, cudaStream_t st) {
    k_add_counts<<<(npix + 255) / 256, 256, 0, st>>>(f, npix, spp);
    return cudaGetLastError();
}

template <class Src>
static cudaError_t stage(int stage, const Src &src, const Wavefront &w, int cur, const LaunchShape &ls,
                         cudaStream_t st) {
    const bool w8 = ls.bvh_width == 8;
    if (stage == kStageTrace) {
        const int tt = ls.trace_threads;
        if (w8) k_trace<Src, Bvh8><<<ls.trace_blocks, tt, trav_smem<Bvh8>(tt), st>>>(src, w, cur);
        else if (ls.bvh_width == 4) k_trace<Src, Bvh4><<<ls.trace_blocks, tt, trav_smem<Bvh4>(tt), st>>>(src, w, cur);
        else {  // BVH2: the iterations of at most coop_limit rays go to k_trace_tail
            k_trace<Src, Bvh2><<<ls.trace_blocks, tt, trav_smem<Bvh2>(tt), st>>>(src, w, cur, ls.coop_limit);
            if (ls.coop_limit) k_trace_tail<Src><<<ls.tail_blocks, kCoopWarps * 32, 0, st>>>(src, w, cur, ls.coop_limit);
        }
    } else {
        k_shade<Src><<<ls.shade_blocks, ls.shade_threads, 0, st>>>(src, w, cur);
    }
    return cudaGetLastError();
}

cudaError_t launch_wave_init(const DevScene &s, const Wavefront &w, const RenderArgs &a, const FilmPtrs &f,
                             const LaunchShape &ls, cudaStream_t st) {
    k_raygen<OneScene><<<ls.sms * 8, 256, 0, st>>>(OneScene{s, a, f}, w);
    return cudaGetLastError();
}

cudaError_t launch_wave_stage(int st_, const DevScene &s, const Wavefront &w, const RenderArgs &a,
                              const FilmPtrs &f, int cur, const LaunchShape &ls, cudaStream_t st) {
    return stage(st_, OneScene{s, a, f}, w, cur, ls, st);
}

cudaError_t launch_batch_init(const SceneTable *t, const Wavefront &w, const LaunchShape &ls, cudaStream_t st) {
    k_raygen<ManyScenes><<<ls.sms * 8, 256, 0, st>>>(ManyScenes{t}, w);
    return cudaGetLastError();
}

cudaError_t launch_batch_stage(int st_, const SceneTable *t, const Wavefront &w, int cur, const LaunchShape &ls,
                               cudaStream_t st) {
    return stage(st_, ManyScenes{t}, w, cur, ls, st);
}

cudaError_t launch_loop_condition(const Wavefront &w, const SceneTable *t, cudaGraphConditionalHandle h, int cur,
                                  uint32_t iters, cudaStream_t st) {
    k_loop_condition<<<1, 1, 0, st>>>(w.counters, t, h, cur, iters);
    return cudaGetLastError();
}

}  // namespace lt
