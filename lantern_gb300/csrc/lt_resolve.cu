// lt_resolve.cu -- the visualizer's final pass without a window: film sums to
// a displayable image in device memory.
//
// Per pixel (visualizer.cpp:352-364, then final_resolve_ps.glsl:24-43):
//   c = exposure * (ColorData / ColorSampleCount, 1)
//   clamp:  c = clamp(c, 0, 1)
//   filmic: x = max(0, c - 0.004); c = x (6.2 x + 0.5) / (x (6.2 x + 1.7) + 0.06); alpha 1; clamp
// and the 8-bit image is the UNORM conversion round(c * 255) of the swapchain's
// B8G8R8A8 / R8G8B8A8 UNORM format (stored here as RGBA). The min / max / sum of
// the sample counts (the visualizer's SPP readout) are reduced on the way.
// One thread per pixel; HBM-bound: 16 B read, 16 + 4 B written per pixel.
#include <cuda_runtime.h>

#include "lt_device.h"

namespace lt {

namespace {

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

__device__ __forceinline__ float filmic(float c) {
    float x = fmaxf(0.0f, c - 0.004f);
    return clamp01((x * (6.2f * x + 0.5f)) / (x * (6.2f * x + 1.7f) + 0.06f));
}

__device__ __forceinline__ unsigned char unorm8(float c) { return (unsigned char)__float2int_rn(c * 255.0f); }

__global__ void __launch_bounds__(256) k_resolve(const float *__restrict__ rgb, const uint32_t *__restrict__ counts,
                                                 uint32_t npix, int tonemap, float exposure, float4 *out,
                                                 uchar4 *out8, SppStats *stats) {
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    unsigned long long sum = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
        const uint32_t n = counts[i];
        const float fn = (float)n;
        float4 c = make_float4(exposure * (rgb[3 * (size_t)i] / fn), exposure * (rgb[3 * (size_t)i + 1] / fn),
                               exposure * (rgb[3 * (size_t)i + 2] / fn), exposure * 1.0f);
        if (tonemap == 1) c = make_float4(filmic(c.x), filmic(c.y), filmic(c.z), 1.0f);
        else c = make_float4(clamp01(c.x), clamp01(c.y), clamp01(c.z), clamp01(c.w));
        if (out) out[i] = c;
        if (out8) out8[i] = make_uchar4(unorm8(c.x), unorm8(c.y), unorm8(c.z), unorm8(c.w));
        lo = min(lo, n);
        hi = max(hi, n);
        sum += n;
    }
    if (!stats) return;
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
        sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
    }
    if ((threadIdx.x & 31u) == 0) {
        atomicMin(&stats->min_spp, lo);
        atomicMax(&stats->max_spp, hi);
        atomicAdd(&stats->sum_spp, sum);
    }
}

}  // namespace

cudaError_t launch_resolve(const float *rgb, const uint32_t *counts, uint32_t npix, int tonemap, float exposure,
                           float4 *out, uchar4 *out8, SppStats *stats, int sms, cudaStream_t st) {
    if (stats) {
        const SppStats init{0xFFFFFFFFu, 0u, 0ull};
        cudaError_t e = cudaMemcpyAsync(stats, &init, sizeof init, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return e;
    }
    if (npix == 0) return cudaSuccess;
    uint32_t blocks = (npix + 255) / 256;
    const uint32_t cap = (uint32_t)sms * 8u;  // 8 blocks of 256 threads per SM
    if (blocks > cap) blocks = cap;
    k_resolve<<<blocks, 256, 0, st>>>(rgb, counts, npix, tonemap, exposure, out, out8, stats);
    return cudaGetLastError();
}

}  // namespace lt
