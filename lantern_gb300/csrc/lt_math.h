// lt_math.h -- vector math, sampler and sampling routines shared by the host
// (scene setup) and the device (kernels).
//
// Every operation is the single-rounded IEEE float operation, in the order the
// reference source spells it out; no fused multiply-add (device code is built
// with -fmad=false, host code with -ffp-contract=off). Vector dot products are
// (x*x + y*y) + z*z and normalize(a) = a * (1 / sqrt(dot(a, a))), except in the
// triangle test, which keeps Embree's x*x + (y*y + z*z).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define LT_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define LT_HD inline
#endif

namespace lt {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;  // (float)M_1_PI
constexpr uint32_t kMiss = 0xFFFFFFFFu;

struct v3 { float x, y, z; };

LT_HD v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
LT_HD v3 operator+(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
LT_HD v3 operator-(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
LT_HD v3 operator*(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
LT_HD v3 operator*(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
LT_HD v3 operator/(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
LT_HD v3 operator-(v3 a) { return mk(-a.x, -a.y, -a.z); }
LT_HD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
LT_HD v3 cross(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
LT_HD float length(v3 a) { return sqrtf(dot(a, a)); }
LT_HD v3 normalize(v3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
// vector_math.h:17-22: "all" means every component is zero
LT_HD bool is_black(v3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
LT_HD v3 ld3(const float *p) { return mk(p[0], p[1], p[2]); }

LT_HD float bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
LT_HD uint32_t float_to_bits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

// ------------------------------------------------------------------ sampler
// PCG32 XSH-RR as UniformSampler (math/uniform_sampler.h:17-57). The
// increment is (sequence | 1); the constructor advances once.
struct Pcg {
    uint64_t state, inc;
    LT_HD uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    }
    // NextFloat: 23 random mantissa bits in [1, 2), minus 1
    LT_HD float next_float() { return bits_to_float((next() >> 9u) | 0x3F800000u) - 1.0f; }
    LT_HD uint32_t next_discrete(uint32_t range) { return (uint32_t)((float)range * next_float()); }
};

LT_HD Pcg pcg_make(uint64_t seed, uint64_t seq) {
    Pcg g;
    g.state = seed;
    g.inc = seq | 1u;
    (void)g.next();
    return g;
}

// MurmurHash3 mix + finalize (integrator.cpp:46-72)
LT_HD uint32_t hash_mix(uint32_t h, uint32_t k) {
    k *= 0xcc9e2d51u;
    k = (k << 15) | (k >> 17);
    k *= 0x1b873593u;
    h ^= k;
    h = ((h << 13) | (h >> 19)) * 5u + 0xe6546b64u;
    return h;
}
LT_HD uint32_t hash_fin(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
// Sampler of sample (key, frame): the reference seeds with (tile, frame)
// (integrator.cpp:84-89); this library keys by pixel.
LT_HD Pcg sampler_for(uint32_t key, uint32_t frame) {
    return pcg_make(hash_fin(hash_mix(hash_mix(0u, key), frame)), frame);
}

// ------------------------------------------------------------------ sampling
// RotateToWorld (math/vector_math.cpp:12-33)
LT_HD v3 rotate_to_world(float x, float y, float z, v3 n) {
    v3 major;
    if (fabsf(n.x) < 0.57735026919f) major = mk(1, 0, 0);
    else if (fabsf(n.y) < 0.57735026919f) major = mk(0, 1, 0);
    else major = mk(0, 0, 1);
    v3 u = normalize(cross(n, major));
    v3 v = cross(n, u);
    return (u * x + v * y) + n * z;
}

// UniformSampleDisc (math/sampling.h:29-36): 2 draws
LT_HD void sample_disc(Pcg &g, float radius, float &x, float &y) {
    float rnd = g.next_float();
    float r = sqrtf(rnd) * radius;
    float theta = g.next_float() * 2.0f * kPi;
    x = r * cosf(theta);
    y = r * sinf(theta);
}

// CosineSampleHemisphere (math/sampling.h:48-58): 2 draws
LT_HD v3 cosine_hemisphere(v3 n, Pcg &g) {
    float x, y;
    sample_disc(g, 1.0f, x, y);
    float z = sqrtf(1.0f - x * x - y * y);
    return normalize(rotate_to_world(x, y, z, n));
}

// UniformSampleSphere (math/sampling.h:72-84): 2 draws
LT_HD v3 uniform_sphere(Pcg &g) {
    float cphi = 2.0f * g.next_float() - 1.0f;
    float sphi = sqrtf(1.0f - cphi * cphi);
    float theta = 2.0f * kPi * g.next_float();
    return mk(sphi * sinf(theta), cphi, sphi * cosf(theta));
}

// Henyey-Greenstein direction about `dir` (extension; g == 0 is the
// reference's uniform sphere): 2 draws
LT_HD v3 hg_sample(Pcg &g, v3 dir, float gg) {
    if (gg == 0.0f) return uniform_sphere(g);
    float u1 = g.next_float(), u2 = g.next_float();
    float sq = (1.0f - gg * gg) / (1.0f - gg + 2.0f * gg * u1);
    float cost = (1.0f + gg * gg - sq * sq) / (2.0f * gg);
    if (cost < -1.0f) cost = -1.0f;
    if (cost > 1.0f) cost = 1.0f;
    float sint = sqrtf(fmaxf(0.0f, 1.0f - cost * cost));
    float phi = 2.0f * kPi * u2;
    return normalize(rotate_to_world(sint * cosf(phi), sint * sinf(phi), cost, dir));
}

// PowerHeuristic with one sample each (math/sampling.h:16-21)
LT_HD float power_heuristic(float f, float g) {
    float a = 1.0f * f, b = 1.0f * g;
    return (a * a) / (a * a + b * b);
}

// ------------------------------------------------------------------ camera
// PinholeCamera (pinhole_camera.cpp:27-40, pinhole_camera.h:216-236) reduced to
// what ray generation needs.
struct Camera {
    v3 origin, mx, my, mz;
    float tanx, tany;
    uint32_t width, height;
};

inline Camera make_camera(float phi, float theta, float radius, uint32_t w, uint32_t h, v3 target, float fov) {
    Camera c;
    c.width = w;
    c.height = h;
    c.tanx = tanf(fov * 0.5f);
    c.tany = tanf(fov * 0.5f * (float)h / (float)w);
    float x = radius * sinf(phi) * sinf(theta);
    float y = radius * cosf(phi);
    float z = radius * sinf(phi) * cosf(theta);
    c.origin = target + mk(x, y, z);
    const float up = 1.0f;
    v3 za = normalize(c.origin - target);
    v3 xa;
    if (za.x == 0.0f && (za.y == 1.0f || za.y == -1.0f) && za.z == 0.0f) xa = normalize(cross(mk(0, 0, up), za));
    else xa = normalize(cross(mk(0, up, 0), za));
    v3 ya = cross(za, xa);
    c.mx = mk(xa.x, ya.x, za.x);
    c.my = mk(xa.y, ya.y, za.y);
    c.mz = mk(xa.z, ya.z, za.z);
    return c;
}

// Tent reconstruction filter, 32-bin inverse CDF
// (reconstruction_filter.cpp:34-87,106-142). cdf has 33 entries.
struct TentFilter {
    float cdf[33];
    float bin_size;
};

inline TentFilter make_tent_filter() {
    TentFilter f;
    const float width = 1.0f;
    f.bin_size = width / 31;
    float norm = 0.0f, pdf[32];
    for (uint32_t i = 0; i < 31; ++i) {
        float t = width - fabsf((float)i * f.bin_size);
        pdf[i] = t;
        norm += t;
    }
    pdf[31] = 0.0f;
    for (uint32_t i = 0; i < 31; ++i) pdf[i] /= norm;
    f.cdf[0] = 0.0f;
    for (uint32_t i = 1; i < 32; ++i) f.cdf[i] = f.cdf[i - 1] + pdf[i - 1];
    f.cdf[32] = 1.0f;
    return f;
}

LT_HD float tent_sample(const TentFilter &f, float x) {
    bool negative = x < 0.5f;
    x = negative ? x * 2.0f : (x - 0.5f) * 2.0f;
    uint32_t index = 32;
    for (uint32_t i = 1; i < 33; ++i) {
        if (x < f.cdf[i]) { index = i - 1; break; }
    }
    float pdf = f.cdf[index + 1] - f.cdf[index];
    float u = f.bin_size * ((float)index + ((x - f.cdf[index]) / pdf));
    return negative ? -u : u;
}

// CalculateRayFromPixel direction (pinhole_camera.cpp:100-110), not normalised
LT_HD v3 camera_dir(const Camera &c, uint32_t x, uint32_t y, float u, float v) {
    v3 view = mk((((float)x + 0.5f + u) / (float)c.width * 2.0f - 1.0f) * c.tanx,
                 -(((float)y + 0.5f + v) / (float)c.height * 2.0f - 1.0f) * c.tany, -1.0f);
    return mk(dot(view, c.mx), dot(view, c.my), dot(view, c.mz));
}

}  // namespace lt
