// ref_driver.cpp -- headless driver around the reference integrator.
//
// TEST INFRASTRUCTURE ONLY: exposes Lantern's own Scene::LoadSceneFromJSON and
// Integrator::RenderFrame (integrator.cpp:28-43) through a C ABI so that tests
// and bench.py's reference arm can call the reference CPU path unmodified.
// The reference renders one sample per pixel per RenderFrame call into the
// film it swaps in at the start of the call (integrator.cpp:35); here the two
// films of that swap are kept and returned separately (film A is the one the
// integrator is constructed with, so frame 0 lands in B).
//
// The integrator's frame counter is private and starts at 0; a caller that
// wants an independent second render starts it elsewhere, which is why the
// class's private section is opened below. Nothing else is changed. Every
// standard and shim header is included first so that only the two reference
// class definitions see the redefinition.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <experimental/filesystem>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>
#include "embree3/rtcore.h"
#include "math/vector_types.h"
#include "math/uniform_sampler.h"
#include "camera/frame_buffer.h"
#include "camera/reconstruction_filter.h"
#include "camera/pinhole_camera.h"
#include "scene/light.h"
#include "scene/image_cache.h"
#include "stb_image.h"
#define private public
#include "integrator/integrator.h"
#include "scene/scene.h"
#undef private
#include "camera/frame_buffer.h"
#include "camera/pinhole_camera.h"

#include <atomic>
#include <chrono>
#include <cstring>

extern "C" std::atomic<unsigned long long> lt_ref_ray_count;

// The two loop constants of RenderPixel (integrator.cpp:114 maxBounces and the
// Russian-roulette threshold at :235) become these variables in the staged copy.
extern "C" {
unsigned lt_ref_max_bounces = 1500;
unsigned lt_ref_rr_depth = 3;
}

extern "C" {

void *lref_scene_load(const char *json_path) {
    auto *s = new Lantern::Scene();
    if (!s->LoadSceneFromJSON(json_path)) {
        delete s;
        return nullptr;
    }
    return s;
}

void lref_scene_free(void *s) { delete (Lantern::Scene *)s; }

void lref_scene_size(void *s, unsigned *w, unsigned *h) {
    auto *sc = (Lantern::Scene *)s;
    *w = sc->Camera->FrameBufferWidth;
    *h = sc->Camera->FrameBufferHeight;
}

// Render `frames` RenderFrame calls starting at frame `first_frame`.
// Outputs films A and B (rgb W*H*3, bounces, counts); returns wall seconds of
// the RenderFrame loop and the number of closest-hit queries made.
double lref_render(void *s, unsigned first_frame, unsigned frames, unsigned max_bounces, unsigned rr_depth,
                   float *rgb_a, unsigned *b_a, unsigned *c_a, float *rgb_b, unsigned *b_b, unsigned *c_b,
                   unsigned long long *rays) {
    auto *sc = (Lantern::Scene *)s;
    unsigned w = sc->Camera->FrameBufferWidth, h = sc->Camera->FrameBufferHeight;
    lt_ref_max_bounces = max_bounces;
    lt_ref_rr_depth = rr_depth;
    Lantern::FrameBuffer fa(w, h), fb(w, h);
    std::atomic<Lantern::FrameBuffer *> swap(&fb);
    Lantern::Integrator integ(sc, &fa, &swap);
    integ.m_frameNumber = first_frame;
    unsigned long long r0 = lt_ref_ray_count.load();
    auto t0 = std::chrono::steady_clock::now();
    for (unsigned f = 0; f < frames; ++f) integ.RenderFrame();
    auto t1 = std::chrono::steady_clock::now();
    if (rays) *rays = lt_ref_ray_count.load() - r0;
    size_t n = (size_t)w * h;
    if (rgb_a) std::memcpy(rgb_a, fa.ColorData, n * 3 * sizeof(float));
    if (b_a) std::memcpy(b_a, fa.Bounces, n * sizeof(unsigned));
    if (c_a) std::memcpy(c_a, fa.ColorSampleCount, n * sizeof(unsigned));
    if (rgb_b) std::memcpy(rgb_b, fb.ColorData, n * 3 * sizeof(float));
    if (b_b) std::memcpy(b_b, fb.Bounces, n * sizeof(unsigned));
    if (c_b) std::memcpy(c_b, fb.ColorSampleCount, n * sizeof(unsigned));
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"

// Building blocks of the reference, for golden vectors.
#include "camera/reconstruction_filter.h"
#include "math/uniform_sampler.h"

extern "C" {

// UniformSampler(seed, sequence) stream (math/uniform_sampler.h:17-57)
void lref_pcg_stream(unsigned long long seed, unsigned long long seq, unsigned n, unsigned *out_uint,
                     float *out_float) {
    Lantern::UniformSampler s(seed, seq);
    for (unsigned i = 0; i < n; ++i) {
        if (out_uint) out_uint[i] = s.NextUInt();
        else out_float[i] = s.NextFloat();
    }
}

// Tent ReconstructionFilter::Sample (camera/reconstruction_filter.cpp:34-87)
void lref_filter_sample(const float *x, unsigned n, float *out) {
    Lantern::ReconstructionFilter f(Lantern::ReconstructionFilter::Type::Tent);
    for (unsigned i = 0; i < n; ++i) out[i] = f.Sample(x[i]);
}

// PinholeCamera::CalculateRayFromPixel with a sampler(seed, seq)
// (camera/pinhole_camera.cpp:88-113); out = org.xyz, dir.xyz
void lref_camera_ray(void *s, unsigned x, unsigned y, unsigned long long seed, unsigned long long seq,
                     float *out) {
    auto *sc = (Lantern::Scene *)s;
    Lantern::UniformSampler smp(seed, seq);
    RTCRay r = sc->Camera->CalculateRayFromPixel(x, y, &smp);
    out[0] = r.org_x; out[1] = r.org_y; out[2] = r.org_z;
    out[3] = r.dir_x; out[4] = r.dir_y; out[5] = r.dir_z;
}

// stbi_load(path, &w, &h, &n, 0) of the reference's vendored stb_image (its
// image cache, image_cache.cpp:23-31): the texels are copied into `out` when it
// holds w*h*n bytes. Returns 0, or -1 when stb_image fails.
int lref_image_load(const char *path, unsigned char *out, size_t cap, int *w, int *h, int *n) {
    unsigned char *d = stbi_load(path, w, h, n, 0);
    if (!d) return -1;
    const size_t size = (size_t)*w * (size_t)*h * (size_t)*n;
    if (out && cap >= size) memcpy(out, d, size);
    stbi_image_free(d);
    return 0;
}

}  // extern "C"
