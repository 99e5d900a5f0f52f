// bvh8_check.cpp -- host check of the compressed 8-wide BVH (lt_bvh8.cpp).
//
// Builds the BVH2 of a scene on the host, collapses it, and checks
//  * structure: every index a traversal can form is in range, every slot
//    holds at most 3 triangles, each triangle appears exactly once;
//  * conservativeness: each child's dequantised box (p + q * cell in float,
//    the traversal's expression) encloses the BVH2 box it came from;
//  * traversal: a step-by-step host emulation of the device traversal
//    (node groups, octant-ordered hit bits, triangle groups, stack) gives the
//    closest hit that brute force gives, on seeded random rays.
// Prints "ok <nodes> <depth>" and exits 0, or prints the first failure and exits 1.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <random>
#include <string>
#include <vector>

#include "lt_scene.h"

using namespace lt;

static float bits_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

struct Hit { float t, u, v; uint32_t prim; };

// the device's triangle test (Embree's Moeller-Trumbore rule), on the host
static void tri_test(const float *tri, const float O[3], const float D[3], float tnear, Hit &h) {
    float v0[3] = {tri[0], tri[1], tri[2]}, e1[3] = {tri[4], tri[5], tri[6]}, e2[3] = {tri[8], tri[9], tri[10]};
    auto cross = [](const float a[3], const float b[3], float o[3]) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto edot = [](const float a[3], const float b[3]) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); };
    float Ng[3], C[3] = {v0[0] - O[0], v0[1] - O[1], v0[2] - O[2]}, R[3];
    cross(e2, e1, Ng);
    cross(C, D, R);
    float den = edot(Ng, D), absden = fabsf(den);
    uint32_t sgn = f_bits(den) & 0x80000000u;
    float U = bits_f(f_bits(edot(R, e2)) ^ sgn), V = bits_f(f_bits(edot(R, e1)) ^ sgn);
    if (den != 0.0f && U >= 0.0f && V >= 0.0f && U + V <= absden) {
        float T = bits_f(f_bits(edot(Ng, C)) ^ sgn);
        if (absden * tnear < T && T <= absden * h.t) {
            h.t = T / absden;
            h.u = U / absden;
            h.v = V / absden;
            h.prim = f_bits(tri[3]);
        }
    }
}

static int fails = 0;
#define CHECK(cond, ...)                      \
    do {                                      \
        if (!(cond)) {                        \
            if (fails++ < 5) {                \
                printf("FAIL %s: ", #cond);   \
                printf(__VA_ARGS__);          \
                printf("\n");                 \
            }                                 \
        }                                     \
    } while (0)

static float cell_of(uint8_t e) { return bits_f((uint32_t)e << 23); }

// Host emulation of traverse8 (lt_kernels.cu), one ray, no warp postponing.
static Hit traverse8(const std::vector<Bvh8Node> &N, const std::vector<float> &T, const float O[3], const float D[3],
                     float tnear, uint32_t *visits) {
    Hit h{INFINITY, 0, 0, 0xFFFFFFFFu};
    float inv[3];
    for (int c = 0; c < 3; ++c) inv[c] = 1.0f / (fabsf(D[c]) > 1e-30f ? D[c] : copysignf(1e-30f, D[c]));
    uint32_t oct = (D[0] < 0 ? 1u : 0u) | (D[1] < 0 ? 2u : 0u) | (D[2] < 0 ? 4u : 0u);
    uint32_t ng[2] = {0u, (1u << (24u + oct)) | 1u}, tg[2] = {0u, 0u};
    std::vector<std::pair<uint32_t, uint32_t>> st;
    for (int guard = 0; guard < 1 << 22; ++guard) {
        if (ng[1] > 0x00FFFFFFu) {
            uint32_t b = 31u - (uint32_t)__builtin_clz(ng[1]);
            uint32_t slot = (b - 24u) ^ oct;
            uint32_t imask = ng[1] & 0xFFu;
            uint32_t idx = ng[0] + (uint32_t)__builtin_popcount(imask & ((1u << slot) - 1u));
            ng[1] &= ~(1u << b);
            if (ng[1] > 0x00FFFFFFu) st.push_back({ng[0], ng[1]});
            CHECK(idx < N.size(), "node index %u of %zu", idx, N.size());
            if (idx >= N.size()) return h;
            ++*visits;
            const Bvh8Node &n = N[idx];
            uint32_t hits = 0;
            for (uint32_t s = 0; s < 8; ++s) {
                if (n.meta[s] == 0) continue;
                float t0 = tnear, t1 = h.t;
                for (int c = 0; c < 3; ++c) {
                    float lo = fmaf((float)n.qlo[c][s], cell_of(n.e[c]) * inv[c], (n.p[c] - O[c]) * inv[c]);
                    float hi = fmaf((float)n.qhi[c][s], cell_of(n.e[c]) * inv[c], (n.p[c] - O[c]) * inv[c]);
                    t0 = fmaxf(t0, fminf(lo, hi));
                    t1 = fminf(t1, fmaxf(lo, hi));
                }
                if (t0 <= t1 * 1.0000004f) {
                    if (n.imask & (1u << s)) hits |= 1u << (24u + (s ^ oct));
                    else hits |= (uint32_t)(n.meta[s] >> 5) << (n.meta[s] & 31u);
                }
            }
            ng[0] = n.base_child;
            ng[1] = (hits & 0xFF000000u) | n.imask;
            tg[0] = n.base_tri;
            tg[1] = hits & 0x00FFFFFFu;
        } else {
            tg[0] = ng[0];
            tg[1] = ng[1];
            ng[0] = ng[1] = 0u;
        }
        while (tg[1]) {
            uint32_t t = (uint32_t)__builtin_ctz(tg[1]);
            tg[1] &= tg[1] - 1u;
            CHECK(12 * (size_t)(tg[0] + t) < T.size(), "triangle index %u", tg[0] + t);
            if (12 * (size_t)(tg[0] + t) >= T.size()) return h;
            tri_test(&T[12 * (size_t)(tg[0] + t)], O, D, tnear, h);
        }
        if (ng[1] <= 0x00FFFFFFu) {
            if (st.empty()) return h;
            ng[0] = st.back().first;
            ng[1] = st.back().second;
            st.pop_back();
        }
    }
    CHECK(false, "traversal did not end");
    return h;
}

// Host emulation of the device's 4-wide traversal (traverse4): slab tests of
// the node's child slots, hit children taken nearest first (the rest stacked),
// leaf references into the BVH2's leaf-ordered triangles.
static Hit traverse4(const std::vector<Bvh4Node> &N, const std::vector<float> &T, const float O[3], const float D[3],
                     float tnear, uint32_t *visits) {
    Hit h{INFINITY, 0, 0, 0xFFFFFFFFu};
    float inv[3];
    for (int c = 0; c < 3; ++c) inv[c] = 1.0f / (fabsf(D[c]) > 1e-30f ? D[c] : copysignf(1e-30f, D[c]));
    std::vector<int32_t> st;
    st.push_back(0);
    int guard = 0;
    while (!st.empty() && ++guard < 10000000) {
        const int32_t ref = st.back();
        st.pop_back();
        if (ref < 0) {
            const uint32_t code = ~(uint32_t)ref, first = code >> kLeafBits, cnt = code & ((1u << kLeafBits) - 1u);
            for (uint32_t k = 0; k < cnt; ++k) {
                CHECK(12 * (size_t)(first + k) < T.size(), "4-wide leaf triangle %u", first + k);
                if (12 * (size_t)(first + k) >= T.size()) return h;
                tri_test(&T[12 * (size_t)(first + k)], O, D, tnear, h);
            }
            continue;
        }
        CHECK((size_t)ref < N.size(), "4-wide node %d", ref);
        if ((size_t)ref >= N.size()) return h;
        const Bvh4Node &n = N[(size_t)ref];
        ++*visits;
        float tk[4];
        int32_t ck[4];
        int nh = 0;
        for (int s = 0; s < 4; ++s) {
            if (n.ref[s] == kEmptyRef4) continue;
            CHECK((uint32_t)s < n.count, "4-wide node %d slot %d beyond its count", ref, s);
            const float lo[3] = {n.lo_x[s], n.lo_y[s], n.lo_z[s]}, hi[3] = {n.hi_x[s], n.hi_y[s], n.hi_z[s]};
            float tmin = tnear, tmax = h.t;
            for (int c = 0; c < 3; ++c) {
                const float a = (lo[c] - O[c]) * inv[c], b = (hi[c] - O[c]) * inv[c];
                tmin = fmaxf(tmin, fminf(a, b));
                tmax = fminf(tmax, fmaxf(a, b));
            }
            if (tmin <= tmax * 1.0000004f) {
                tk[nh] = tmin;
                ck[nh] = n.ref[s];
                ++nh;
            }
        }
        for (int i = 1; i < nh; ++i)  // nearest first
            for (int j = i; j > 0 && tk[j] < tk[j - 1]; --j) {
                std::swap(tk[j], tk[j - 1]);
                std::swap(ck[j], ck[j - 1]);
            }
        for (int i = nh - 1; i >= 0; --i) st.push_back(ck[i]);
        CHECK(st.size() <= 64, "4-wide stack depth %zu", st.size());
    }
    return h;
}

static void add_sphere(std::vector<float> &P, std::vector<uint32_t> &I, float cx, float cy, float cz, float r,
                       int sl, int stc) {
    uint32_t base = (uint32_t)(P.size() / 3);
    for (int i = 0; i <= stc; ++i)
        for (int j = 0; j <= sl; ++j) {
            float ph = (float)M_PI * i / stc, th = 2.0f * (float)M_PI * j / sl;
            P.push_back(cx + r * sinf(ph) * cosf(th));
            P.push_back(cy + r * cosf(ph));
            P.push_back(cz + r * sinf(ph) * sinf(th));
        }
    for (int i = 0; i < stc; ++i)
        for (int j = 0; j < sl; ++j) {
            uint32_t a = base + i * (sl + 1) + j, b = a + sl + 1;
            I.insert(I.end(), {a, b, a + 1, a + 1, b, b + 1});
        }
}

static int run_case(const char *name, std::vector<float> P, std::vector<uint32_t> I, int nrays) {
    lt_material_desc mat{LT_BSDF_LAMBERT, {0.5f, 0.5f, 0.5f}, 1.5f, -1};
    lt_mesh_desc mesh{P.data(), nullptr, I.data(), (uint32_t)(P.size() / 3), (uint32_t)(I.size() / 3), 0, 0,
                      {0, 0, 0}, 0.0f};
    lt_scene_desc desc;
    memset(&desc, 0, sizeof desc);
    desc.camera = lt_camera_desc{1.0f, 0.0f, 5.0f, 0.8f, {0, 0, 0}, 8, 8};
    desc.materials = &mat;
    desc.num_materials = 1;
    desc.meshes = &mesh;
    desc.num_meshes = 1;
    HostScene hs;
    std::string err;
    if (build_host_scene(&desc, &hs, &err) != LT_OK) {
        printf("FAIL %s: %s\n", name, err.c_str());
        return 1;
    }
    build_bvh(&hs);
    std::vector<Bvh8Node> N;
    std::vector<float> T;
    uint32_t depth = build_bvh8(hs.nodes, hs.leaf_tris, &N, &T);
    const size_t ntri = hs.tri_geom.size();
    // structure
    CHECK(T.size() == 12 * ntri, "%s: %zu triangle floats for %zu triangles", name, T.size(), ntri);
    CHECK(2 * depth + 2 <= 64, "%s: depth %u", name, depth);
    std::vector<int> seen(ntri, 0);
    for (size_t k = 0; k < T.size() / 12; ++k) {
        uint32_t prim = f_bits(T[12 * k + 3]);
        CHECK(prim < ntri, "%s: prim %u", name, prim);
        if (prim < ntri) seen[prim]++;
    }
    for (size_t t = 0; t < ntri; ++t) CHECK(seen[t] == 1, "%s: triangle %zu appears %d times", name, t, seen[t]);
    for (size_t i = 0; i < N.size(); ++i) {
        const Bvh8Node &n = N[i];
        uint32_t inner = (uint32_t)__builtin_popcount(n.imask);
        CHECK(inner == 0 || n.base_child + inner <= N.size(), "%s: node %zu children", name, i);
        for (int s = 0; s < 8; ++s) {
            if (n.meta[s] == 0) continue;
            if (n.imask & (1u << s)) {
                CHECK((n.meta[s] & 31u) == 24u + (uint32_t)s, "%s: node %zu slot %d meta", name, i, s);
            } else {
                uint32_t cnt = (uint32_t)__builtin_popcount(n.meta[s] >> 5), off = n.meta[s] & 31u;
                CHECK(cnt >= 1 && cnt <= 3 && off + cnt <= 24, "%s: node %zu slot %d leaf", name, i, s);
                CHECK(12 * (size_t)(n.base_tri + off + cnt) <= T.size(), "%s: node %zu slot %d tris", name, i, s);
                // dequantised box encloses its triangles (which lie in the BVH2 leaf box)
                for (uint32_t k = 0; k < cnt; ++k) {
                    const float *tr = &T[12 * (size_t)(n.base_tri + off + k)];
                    for (int c = 0; c < 3; ++c) {
                        float lo = fmaf((float)n.qlo[c][s], cell_of(n.e[c]), n.p[c]);
                        float hi = fmaf((float)n.qhi[c][s], cell_of(n.e[c]), n.p[c]);
                        float v0 = tr[c], v1 = tr[c] - tr[4 + c], v2 = tr[c] + tr[8 + c];
                        float mn = fminf(v0, fminf(v1, v2)), mx = fmaxf(v0, fmaxf(v1, v2));
                        CHECK(lo <= mn && hi >= mx, "%s: node %zu slot %d axis %d [%g %g] vs [%g %g]", name, i, s, c,
                              lo, hi, mn, mx);
                    }
                }
            }
        }
    }
    // traversal vs brute force
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t k = 0; k < P.size(); ++k) {
        lo[k % 3] = fminf(lo[k % 3], P[k]);
        hi[k % 3] = fmaxf(hi[k % 3], P[k]);
    }
    if (P.empty())  // rays through the unit box around the origin
        for (int c = 0; c < 3; ++c) { lo[c] = -1.0f; hi[c] = 1.0f; }
    std::mt19937 rng(2);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    std::normal_distribution<float> nd(0.0f, 1.0f);
    uint64_t visits = 0;
    int mism = 0;
    for (int r = 0; r < nrays; ++r) {
        float O[3], D[3];
        for (int c = 0; c < 3; ++c) O[c] = lo[c] - 0.2f * (hi[c] - lo[c]) + 1.4f * (hi[c] - lo[c]) * u01(rng);
        float l = 0.0f;
        for (int c = 0; c < 3; ++c) { D[c] = nd(rng); l += D[c] * D[c]; }
        for (int c = 0; c < 3; ++c) D[c] /= sqrtf(l);
        uint32_t v = 0;
        Hit a = traverse8(N, T, O, D, 0.0f, &v);
        visits += v;
        Hit b{INFINITY, 0, 0, 0xFFFFFFFFu};
        for (size_t k = 0; k < ntri; ++k) tri_test(&hs.leaf_tris[12 * k], O, D, 0.0f, b);
        bool same = (a.prim == 0xFFFFFFFFu) == (b.prim == 0xFFFFFFFFu) && (a.prim == 0xFFFFFFFFu || a.t == b.t);
        if (!same) ++mism;
    }
    CHECK(mism == 0, "%s: %d of %d rays differ from brute force", name, mism, nrays);
    printf("%s: %zu wide nodes, depth %u, %.2f node visits per ray\n", name, N.size(), depth,
           (double)visits / nrays);
    // 4-wide tree: every BVH2 node's children, inner ones opened; BVH2 leaves
    std::vector<Bvh4Node> N4;
    const uint32_t depth4 = build_bvh4(hs.nodes, &N4);
    CHECK(3 * depth4 + 1 <= 64, "%s: 4-wide depth %u", name, depth4);
    std::vector<int> seen4(ntri, 0);
    for (size_t i = 0; i < N4.size(); ++i) {
        const Bvh4Node &n = N4[i];
        CHECK(n.count >= 2 && n.count <= 4, "%s: 4-wide node %zu has %u children", name, i, n.count);
        for (uint32_t s = 0; s < 4; ++s) {
            if (s >= n.count) {
                CHECK(n.ref[s] == kEmptyRef4, "%s: 4-wide node %zu slot %u not empty", name, i, s);
                continue;
            }
            if (n.ref[s] >= 0) {
                CHECK((size_t)n.ref[s] < N4.size() && (size_t)n.ref[s] > i, "%s: 4-wide node %zu child %d", name, i,
                      n.ref[s]);
            } else {
                const uint32_t code = ~(uint32_t)n.ref[s], first = code >> kLeafBits,
                               cnt = code & ((1u << kLeafBits) - 1u);
                for (uint32_t k = 0; k < cnt; ++k) {
                    CHECK(12 * (size_t)(first + k) < hs.leaf_tris.size(), "%s: 4-wide leaf range", name);
                    const uint32_t prim = f_bits(hs.leaf_tris[12 * (size_t)(first + k) + 3]);
                    if (prim < ntri) seen4[prim]++;
                }
            }
        }
    }
    for (size_t t = 0; t < ntri; ++t) CHECK(seen4[t] == 1, "%s: triangle %zu in %d 4-wide leaves", name, t, seen4[t]);
    std::mt19937 rng4(3);
    uint64_t visits4 = 0;
    int mism4 = 0;
    for (int r = 0; r < nrays; ++r) {
        float O[3], D[3];
        for (int c = 0; c < 3; ++c) O[c] = lo[c] - 0.2f * (hi[c] - lo[c]) + 1.4f * (hi[c] - lo[c]) * u01(rng4);
        float l = 0.0f;
        for (int c = 0; c < 3; ++c) { D[c] = nd(rng4); l += D[c] * D[c]; }
        for (int c = 0; c < 3; ++c) D[c] /= sqrtf(l);
        uint32_t v = 0;
        Hit a = traverse4(N4, hs.leaf_tris, O, D, 0.0f, &v);
        visits4 += v;
        Hit b{INFINITY, 0, 0, 0xFFFFFFFFu};
        for (size_t k = 0; k < ntri; ++k) tri_test(&hs.leaf_tris[12 * k], O, D, 0.0f, b);
        bool same = (a.prim == 0xFFFFFFFFu) == (b.prim == 0xFFFFFFFFu) && (a.prim == 0xFFFFFFFFu || a.t == b.t);
        if (!same) ++mism4;
    }
    CHECK(mism4 == 0, "%s: %d of %d rays differ from brute force (4-wide)", name, mism4, nrays);
    printf("%s: %zu 4-wide nodes, depth %u, %.2f node visits per ray\n", name, N4.size(), depth4,
           (double)visits4 / nrays);
    return 0;
}

int main() {
    {  // one sphere
        std::vector<float> P;
        std::vector<uint32_t> I;
        add_sphere(P, I, 0, 0, 0, 1, 48, 24);
        run_case("sphere", P, I, 4000);
    }
    {  // spheres of different sizes plus a triangle soup
        std::vector<float> P;
        std::vector<uint32_t> I;
        add_sphere(P, I, -2, 0, 0, 0.5f, 16, 8);
        add_sphere(P, I, 1, 1, 0, 1.2f, 64, 32);
        add_sphere(P, I, 0, -1, 2, 0.05f, 8, 4);
        std::mt19937 rng(5);
        std::uniform_real_distribution<float> u(-3.0f, 3.0f);
        for (int k = 0; k < 3000; ++k) {
            uint32_t b = (uint32_t)(P.size() / 3);
            float c[3] = {u(rng), u(rng), u(rng)};
            for (int v = 0; v < 3; ++v)
                for (int a = 0; a < 3; ++a) P.push_back(c[a] + 0.1f * u(rng));
            I.insert(I.end(), {b, b + 1, b + 2});
        }
        run_case("mixed", P, I, 3000);
    }
    {  // tiny: fewer triangles than one leaf, and exactly five
        std::vector<float> P = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 1, 1, 2, 0, 1};
        std::vector<uint32_t> I = {0, 1, 2};
        run_case("one", P, I, 500);
        I = {0, 1, 2, 1, 2, 3, 2, 3, 4, 3, 4, 5, 0, 4, 5};
        run_case("five", P, I, 500);
    }
    {  // empty: no triangles at all (every ray misses)
        run_case("empty", {}, {}, 200);
    }
    {  // flat: all triangles in one plane (zero extent on an axis)
        std::vector<float> P;
        std::vector<uint32_t> I;
        for (int i = 0; i <= 40; ++i)
            for (int j = 0; j <= 40; ++j) P.insert(P.end(), {(float)i, 0.0f, (float)j});
        for (int i = 0; i < 40; ++i)
            for (int j = 0; j < 40; ++j) {
                uint32_t a = (uint32_t)(i * 41 + j);
                I.insert(I.end(), {a, a + 41, a + 1, a + 1, a + 41, a + 42});
            }
        run_case("plane", P, I, 3000);
    }
    if (fails) {
        printf("%d failures\n", fails);
        return 1;
    }
    printf("ok\n");
    return 0;
}
