// cpp_adapter.cpp -- the C++ drop-in for the reference's Integrator, as a host
// application would write it against include/lantern_gpu.h.
//
// The reference renders with `Integrator(Scene*, FrameBuffer* current,
// std::atomic<FrameBuffer*>* swap)` and one `RenderFrame()` per sample
// (integrator.h:24-51, integrator.cpp:28-43): the film pointer is exchanged at
// the start of each call, one sample per pixel is added to the current film,
// and the frame number advances. GpuIntegrator keeps that shape on top of
// lt_render with the film in host memory (FrameBuffer's own layout: packed
// float3 colour sums, uint bounces, uint sample counts).
//
// Usage: cpp_adapter <scene.json> <frames> <out.bin>
// Renders <frames> RenderFrame() calls alternating between two films (as the
// reference's render loop does) and writes both films' sums, bounces and
// counts added together: width, height (uint32), then rgb (float32 x 3 per
// pixel), bounces, counts (uint32 per pixel). Exit status 0 on success.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>
#include <stdexcept>
#include <vector>

#include "lantern_gpu.h"

#ifdef LT_REFERENCE_FRAME_BUFFER
// The reference's own FrameBuffer (camera/frame_buffer.{h,cpp}): raw arrays of
// float3 colour sums, uint bounces and uint sample counts.
#include "camera/frame_buffer.h"
static_assert(sizeof(float3) == 12, "FrameBuffer::ColorData must be packed float3 for lt_film");
static float *color_of(Lantern::FrameBuffer *f) { return &f->ColorData[0].x; }
static uint32_t *bounces_of(Lantern::FrameBuffer *f) { return f->Bounces; }
static uint32_t *counts_of(Lantern::FrameBuffer *f) { return f->ColorSampleCount; }
#else
// Without the reference tree: a stand-in with the film fields RenderFrame
// touches, in the reference's layout (camera/frame_buffer.h:17-34).
namespace Lantern {
struct float3 {
    float x, y, z;
};
struct FrameBuffer {
    FrameBuffer(uint32_t w, uint32_t h) : Width(w), Height(h), ColorData(w * h), Bounces(w * h), ColorSampleCount(w * h) {}
    uint32_t Width, Height;
    std::vector<float3> ColorData;
    std::vector<uint32_t> Bounces;
    std::vector<uint32_t> ColorSampleCount;
    bool Empty = true;
};
}  // namespace Lantern
static float *color_of(Lantern::FrameBuffer *f) { return &f->ColorData[0].x; }
static uint32_t *bounces_of(Lantern::FrameBuffer *f) { return f->Bounces.data(); }
static uint32_t *counts_of(Lantern::FrameBuffer *f) { return f->ColorSampleCount.data(); }
#endif

class GpuIntegrator {
public:
    GpuIntegrator(const char *sceneJson, Lantern::FrameBuffer *current, std::atomic<Lantern::FrameBuffer *> *swap,
                  uint32_t maxDepth, uint32_t rrDepth)
        : m_current(current), m_swap(swap), m_maxDepth(maxDepth), m_rrDepth(rrDepth) {
        if (lt_ctx_create(0, &m_ctx) != LT_OK) throw std::runtime_error(lt_last_error(nullptr));
        if (lt_scene_load_json(m_ctx, sceneJson) != LT_OK) throw std::runtime_error(lt_last_error(m_ctx));
    }
    ~GpuIntegrator() { lt_ctx_destroy(m_ctx); }

    void RenderFrame() {
        m_current = std::atomic_exchange(m_swap, m_current);
        m_current->Empty = false;
        lt_film film = {color_of(m_current), bounces_of(m_current), counts_of(m_current), m_current->Width,
                        m_current->Height, /*on_device=*/0};
        lt_render_params p = {/*spp=*/1, m_frame, m_maxDepth, m_rrDepth};
        if (lt_render(m_ctx, &p, &film) != LT_OK) throw std::runtime_error(lt_last_error(m_ctx));
        ++m_frame;
    }

private:
    lt_ctx *m_ctx = nullptr;
    Lantern::FrameBuffer *m_current;
    std::atomic<Lantern::FrameBuffer *> *m_swap;
    uint32_t m_maxDepth, m_rrDepth;
    uint32_t m_frame = 0;
};

int main(int argc, char **argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: %s scene.json frames out.bin\n", argv[0]);
        return 2;
    }
    try {
        // the film size comes from the scene: a throwaway context reads it
        lt_ctx *probe = nullptr;
        if (lt_ctx_create(0, &probe) != LT_OK || lt_scene_load_json(probe, argv[1]) != LT_OK) {
            fprintf(stderr, "scene: %s\n", lt_last_error(probe));
            return 1;
        }
        lt_scene_info info;
        lt_scene_info_get(probe, &info);
        lt_ctx_destroy(probe);
        Lantern::FrameBuffer a(info.width, info.height), b(info.width, info.height);
        std::atomic<Lantern::FrameBuffer *> swap(&b);
        GpuIntegrator integrator(argv[1], &a, &swap, 8, 3);
        const int frames = atoi(argv[2]);
        for (int k = 0; k < frames; ++k) integrator.RenderFrame();
        const size_t n = (size_t)info.width * info.height;
        FILE *f = fopen(argv[3], "wb");
        if (!f) return 1;
        fwrite(&info.width, 4, 1, f);
        fwrite(&info.height, 4, 1, f);
        for (size_t i = 0; i < n; ++i) {
            const float c[3] = {a.ColorData[i].x + b.ColorData[i].x, a.ColorData[i].y + b.ColorData[i].y,
                                a.ColorData[i].z + b.ColorData[i].z};
            fwrite(c, 4, 3, f);
        }
        for (size_t i = 0; i < n; ++i) {
            const uint32_t v = a.Bounces[i] + b.Bounces[i];
            fwrite(&v, 4, 1, f);
        }
        for (size_t i = 0; i < n; ++i) {
            const uint32_t v = a.ColorSampleCount[i] + b.ColorSampleCount[i];
            fwrite(&v, 4, 1, f);
        }
        fclose(f);
    } catch (const std::exception &e) {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
