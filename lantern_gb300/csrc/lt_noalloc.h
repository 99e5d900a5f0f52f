// lt_noalloc.h -- sizes of the fixed device scratch behind lt_render_noalloc.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "lantern_gpu.h"

namespace lt {

// Per path: two copies (ping-pong) of PCG state 8, pixel 4, frame 4,
// throughput 12, bounces 4, flags 4, IOR 4 (2 x 40); two ray buffers 2 x 32;
// hit 16; two connection rays 2 x 32; two connection records 2 x 32 = 288 B.
constexpr size_t kNoAllocBytesPerPath = 288;
// Each of the 19 arrays carved from the scratch is rounded up to 256 bytes,
// plus the counters block.
constexpr size_t kNoAllocScratchBytes =
    (size_t)LT_NOALLOC_MAX_PATHS * kNoAllocBytesPerPath + 20 * 256;

// Device address of the scratch on `device` (which must be current); looked up
// with cudaGetSymbolAddress on the first call per device and cached.
cudaError_t noalloc_scratch(int device, void **ptr);

}  // namespace lt
