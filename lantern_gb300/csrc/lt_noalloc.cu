// lt_noalloc.cu -- fixed device scratch for lt_render_noalloc.
//
// Some callers cannot let this library call cudaMalloc during a render: a host
// application that hands the library a fixed GPU memory budget at start-up and
// forbids later allocations, or a real-time loop where an allocation (which may
// synchronise the whole device) would stall other work. For them the wavefront
// state (path slots, ray queues, connection records, counters) lives in the
// file-scope array below instead of a cudaMalloc'd arena. It is reserved on
// every GPU that loads the library and stays there until the process exits.
//
// Host code must not pass `g_noalloc_scratch` itself to a kernel: in host code
// that name is a host-side stand-in, not the device address. The address is
// fetched once per device with cudaGetSymbolAddress (with that device current)
// and cached here.
#include <cuda_runtime.h>

#include <mutex>

#include "lt_noalloc.h"

namespace lt {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {nullptr};
}  // namespace

cudaError_t noalloc_scratch(int device, void **ptr) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[device]) {
        // the caller has made `device` current
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[device] = p;
    }
    *ptr = g_addr[device];
    return cudaSuccess;
}

}  // namespace lt
