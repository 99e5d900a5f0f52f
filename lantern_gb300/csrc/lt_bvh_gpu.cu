// lt_bvh_gpu.cu -- binned-SAH BVH2 build on the GPU (replaces rtcCommitScene,
// scene.cpp:86, for this library's traversal layout).
//
// Level-synchronous, top-down: every node still to be split is one task, and
// one block of kBlock threads handles one task per launch (one launch per
// tree level; no block ever waits on another). A task
//   1. reduces the centroid bounds of its triangle range,
//   2. bins the centroids into 32 bins per axis in shared memory (counts and
//      bin boxes),
//   3. sweeps the bins for the least SAH cost (area x count on both sides) --
//      the same bins, float operations and tie order as the host builder in
//      lt_scene.cpp, so both pick the same split,
//   4. partitions its range stably into the other index buffer (midpoint of
//      the range when no bin split separates the triangles),
//   5. reduces the two children's boxes and writes its 64-byte node with
//      both child boxes; a child of at most kLeafMax triangles becomes a leaf
//      (its triangles are written to the leaf-ordered triangle array), a larger
//      one gets a node index and becomes a task of the next level.
// Triangle ranges never move once assigned, so leaves can be written as soon
// as they are made.
#include <cuda_runtime.h>

#include <vector>

#include "lt_bvh_gpu.h"

namespace lt {

namespace {

constexpr int kBlock = 256;
constexpr int kBinsG = 32;
constexpr uint32_t kLeafMaxG = 4;

struct Task {
    uint32_t node, begin, end, depth;
};

// order-preserving map of floats to ints for atomicMin / atomicMax
__device__ __forceinline__ int f2o(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

__device__ __forceinline__ float box_area(const float lo[3], const float hi[3]) {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (!(dx >= 0.0f)) return 0.0f;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

// per-triangle box and centroid from (v0, e1 = v0 - v1, e2 = v2 - v0)
__global__ void k_prim_bounds(const float *__restrict__ tri, uint32_t n, float *__restrict__ box,
                              float *__restrict__ cen, uint32_t *__restrict__ idx) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const float *d = tri + 9 * (size_t)t;
        float lo[3], hi[3];
        for (int c = 0; c < 3; ++c) {
            float a = d[c], b = d[c] - d[3 + c], e = d[c] + d[6 + c];
            lo[c] = fminf(fminf(a, b), e);
            hi[c] = fmaxf(fmaxf(a, b), e);
            box[6 * (size_t)t + c] = lo[c];
            box[6 * (size_t)t + 3 + c] = hi[c];
            cen[3 * (size_t)t + c] = 0.5f * (lo[c] + hi[c]);
        }
        idx[t] = t;
    }
}

template <typename T>
__device__ __forceinline__ T block_reduce_min_max(T v, bool is_max, T *sh) {
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = is_max ? (w > v ? w : v) : (w < v ? w : v);
    }
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < (kBlock >> 5) ? sh[lane] : sh[0];
        for (int o = 16; o > 0; o >>= 1) {
            T w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
            v = is_max ? (w > v ? w : v) : (w < v ? w : v);
        }
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    T r = sh[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
    int b = (int)((c - lo) * scale);
    return b < 0 ? 0 : (b >= kBinsG ? kBinsG - 1 : b);
}

// Box of the triangles idx[b, e): block reduction. Returns lo/hi in all threads.
__device__ void range_box(const float *__restrict__ box, const uint32_t *__restrict__ idx, uint32_t b, uint32_t e,
                          float lo[3], float hi[3], float *sh) {
    float l[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
    float h[3] = {-l[0], -l[0], -l[0]};
    for (uint32_t i = b + threadIdx.x; i < e; i += kBlock) {
        const float *p = box + 6 * (size_t)idx[i];
        for (int c = 0; c < 3; ++c) {
            l[c] = fminf(l[c], p[c]);
            h[c] = fmaxf(h[c], p[3 + c]);
        }
    }
    for (int c = 0; c < 3; ++c) {
        lo[c] = block_reduce_min_max(l[c], false, sh);
        hi[c] = block_reduce_min_max(h[c], true, sh);
    }
}

__device__ void write_leaf(const float *__restrict__ tri, const uint32_t *__restrict__ idx, uint32_t b, uint32_t e,
                           float4 *__restrict__ leaf_tris) {
    for (uint32_t i = b + threadIdx.x; i < e; i += kBlock) {
        uint32_t t = idx[i];
        const float *d = tri + 9 * (size_t)t;
        leaf_tris[3 * (size_t)i] = make_float4(d[0], d[1], d[2], __uint_as_float(t));
        leaf_tris[3 * (size_t)i + 1] = make_float4(d[3], d[4], d[5], 0.0f);
        leaf_tris[3 * (size_t)i + 2] = make_float4(d[6], d[7], d[8], 0.0f);
    }
}

struct BuildArgs {
    const float *tri;
    const float *box;
    const float *cen;
    const uint32_t *idx_in;
    uint32_t *idx_out;
    const Task *tasks;
    Task *next_tasks;
    uint32_t *counters;   // [0] next task count, [1] node count, [2] max depth, [3] leaf triangles
    float4 *nodes;        // BvhNode, 4 float4 each
    float4 *leaf_tris;
};

__global__ void __launch_bounds__(kBlock) k_build_level(BuildArgs A) {
    __shared__ float shf[32];
    __shared__ int bin_lo[3][kBinsG][3], bin_hi[3][kBinsG][3];
    __shared__ uint32_t bin_cnt[3][kBinsG];
    __shared__ int best_axis_s, best_bin_s;
    __shared__ uint32_t scan_s[kBlock / 32 + 1];
    __shared__ uint32_t child_node_s[2];

    const Task T = A.tasks[blockIdx.x];
    const uint32_t b = T.begin, e = T.end, count = e - b;

    // 1. centroid bounds
    float cl[3], ch[3];
    {
        float l[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
        float h[3] = {-l[0], -l[0], -l[0]};
        for (uint32_t i = b + threadIdx.x; i < e; i += kBlock) {
            const float *p = A.cen + 3 * (size_t)A.idx_in[i];
            for (int c = 0; c < 3; ++c) {
                l[c] = fminf(l[c], p[c]);
                h[c] = fmaxf(h[c], p[c]);
            }
        }
        for (int c = 0; c < 3; ++c) {
            cl[c] = block_reduce_min_max(l[c], false, shf);
            ch[c] = block_reduce_min_max(h[c], true, shf);
        }
    }
    float scale[3];
    for (int ax = 0; ax < 3; ++ax) {
        float ext = ch[ax] - cl[ax];
        scale[ax] = ext > 0.0f ? (float)kBinsG / ext : 0.0f;
    }
    // 2. bins
    for (int k = threadIdx.x; k < 3 * kBinsG; k += kBlock) {
        int ax = k / kBinsG, bb = k % kBinsG;
        bin_cnt[ax][bb] = 0;
        for (int c = 0; c < 3; ++c) {
            bin_lo[ax][bb][c] = f2o(__int_as_float(0x7f800000));
            bin_hi[ax][bb][c] = f2o(-__int_as_float(0x7f800000));
        }
    }
    __syncthreads();
    for (uint32_t i = b + threadIdx.x; i < e; i += kBlock) {
        uint32_t t = A.idx_in[i];
        const float *p = A.cen + 3 * (size_t)t;
        const float *bx = A.box + 6 * (size_t)t;
        for (int ax = 0; ax < 3; ++ax) {
            if (scale[ax] == 0.0f) continue;
            int bb = bin_of(p[ax], cl[ax], scale[ax]);
            atomicAdd(&bin_cnt[ax][bb], 1u);
            for (int c = 0; c < 3; ++c) {
                atomicMin(&bin_lo[ax][bb][c], f2o(bx[c]));
                atomicMax(&bin_hi[ax][bb][c], f2o(bx[3 + c]));
            }
        }
    }
    __syncthreads();
    // 3. SAH sweep (thread 0, axes in order, first minimum wins)
    if (threadIdx.x == 0) {
        int best_axis = -1, best_bin = -1;
        float best_cost = __int_as_float(0x7f800000);
        for (int ax = 0; ax < 3; ++ax) {
            if (scale[ax] == 0.0f) continue;
            float rarea[kBinsG];
            uint32_t rc[kBinsG];
            float alo[3], ahi[3];
            for (int c = 0; c < 3; ++c) { alo[c] = __int_as_float(0x7f800000); ahi[c] = -alo[c]; }
            uint32_t cc = 0;
            for (int bb = kBinsG - 1; bb > 0; --bb) {
                for (int c = 0; c < 3; ++c) {
                    alo[c] = fminf(alo[c], o2f(bin_lo[ax][bb][c]));
                    ahi[c] = fmaxf(ahi[c], o2f(bin_hi[ax][bb][c]));
                }
                cc += bin_cnt[ax][bb];
                rarea[bb] = box_area(alo, ahi);
                rc[bb] = cc;
            }
            for (int c = 0; c < 3; ++c) { alo[c] = __int_as_float(0x7f800000); ahi[c] = -alo[c]; }
            cc = 0;
            for (int bb = 0; bb < kBinsG - 1; ++bb) {
                for (int c = 0; c < 3; ++c) {
                    alo[c] = fminf(alo[c], o2f(bin_lo[ax][bb][c]));
                    ahi[c] = fmaxf(ahi[c], o2f(bin_hi[ax][bb][c]));
                }
                cc += bin_cnt[ax][bb];
                if (cc == 0 || rc[bb + 1] == 0) continue;
                float cost = box_area(alo, ahi) * (float)cc + rarea[bb + 1] * (float)rc[bb + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = bb; }
            }
        }
        best_axis_s = best_axis;
        best_bin_s = best_bin;
    }
    __syncthreads();
    const int best_axis = best_axis_s, best_bin = best_bin_s;
    // 4. stable partition into idx_out
    uint32_t nl = 0;
    if (best_axis >= 0) {
        for (int bb = 0; bb <= best_bin; ++bb) nl += bin_cnt[best_axis][bb];
    }
    if (best_axis < 0 || nl == 0 || nl == count) {
        nl = count / 2;
        for (uint32_t i = b + threadIdx.x; i < e; i += kBlock) A.idx_out[i] = A.idx_in[i];
    } else {
        uint32_t left_base = 0, right_base = 0;
        for (uint32_t c0 = b; c0 < e; c0 += kBlock) {
            uint32_t i = c0 + threadIdx.x;
            bool valid = i < e;
            uint32_t t = valid ? A.idx_in[i] : 0;
            bool left = valid && bin_of(A.cen[3 * (size_t)t + best_axis], cl[best_axis], scale[best_axis]) <= best_bin;
            unsigned m = __ballot_sync(0xFFFFFFFFu, left);
            int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            if (lane == 0) scan_s[warp] = __popc(m);
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t s = 0;
                for (int w = 0; w < kBlock / 32; ++w) { uint32_t v = scan_s[w]; scan_s[w] = s; s += v; }
                scan_s[kBlock / 32] = s;
            }
            __syncthreads();
            uint32_t lrank = scan_s[warp] + __popc(m & ((1u << lane) - 1u));
            uint32_t chunk_left = scan_s[kBlock / 32];
            if (valid) {
                if (left) A.idx_out[b + left_base + lrank] = t;
                else A.idx_out[b + nl + right_base + (threadIdx.x - lrank)] = t;
            }
            uint32_t chunk_valid = (e - c0) < (uint32_t)kBlock ? (e - c0) : (uint32_t)kBlock;
            left_base += chunk_left;
            right_base += chunk_valid - chunk_left;
            __syncthreads();
        }
    }
    __syncthreads();
    // 5. children
    const uint32_t mid = b + nl;
    const uint32_t cb[2] = {b, mid}, ce[2] = {mid, e};
    float lo[2][3], hi[2][3];
    for (int k = 0; k < 2; ++k) range_box(A.box, A.idx_out, cb[k], ce[k], lo[k], hi[k], shf);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 2; ++k) {
            uint32_t cn = ce[k] - cb[k];
            if (cn > kLeafMaxG) {
                child_node_s[k] = atomicAdd(&A.counters[1], 1u);
                uint32_t slot = atomicAdd(&A.counters[0], 1u);
                A.next_tasks[slot] = Task{child_node_s[k], cb[k], ce[k], T.depth + 1};
                atomicMax(&A.counters[2], T.depth + 1);
            } else {
                child_node_s[k] = 0xFFFFFFFFu;
                atomicAdd(&A.counters[3], cn);
            }
        }
        float4 *nd = A.nodes + 4 * (size_t)T.node;
        int r0 = child_node_s[0] != 0xFFFFFFFFu ? (int)child_node_s[0] : leaf_ref(cb[0], ce[0] - cb[0]);
        int r1 = child_node_s[1] != 0xFFFFFFFFu ? (int)child_node_s[1] : leaf_ref(cb[1], ce[1] - cb[1]);
        nd[0] = make_float4(lo[0][0], hi[0][0], lo[0][1], hi[0][1]);
        nd[1] = make_float4(lo[1][0], hi[1][0], lo[1][1], hi[1][1]);
        nd[2] = make_float4(lo[0][2], hi[0][2], lo[1][2], hi[1][2]);
        nd[3] = make_float4(__int_as_float(r0), __int_as_float(r1),
                            __uint_as_float(child_node_s[0] == 0xFFFFFFFFu ? ce[0] - cb[0] : 0u),
                            __uint_as_float(child_node_s[1] == 0xFFFFFFFFu ? ce[1] - cb[1] : 0u));
    }
    __syncthreads();
    for (int k = 0; k < 2; ++k)
        if (child_node_s[k] == 0xFFFFFFFFu) write_leaf(A.tri, A.idx_out, cb[k], ce[k], A.leaf_tris);
}

}  // namespace

cudaError_t build_bvh_gpu(const float *d_tri, uint32_t n, GpuBvh *out, cudaStream_t st) {
    out->nodes = nullptr;
    out->leaf_tris = nullptr;
    out->num_nodes = 0;
    out->max_depth = 0;
    out->build_ms = 0.0f;
    if (n <= kLeafMaxG) return cudaErrorInvalidValue;  // the caller builds tiny scenes on the host
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    size_t max_nodes = (size_t)n;  // inner nodes < n / 2 for leaves of >= 1 triangle
    size_t max_tasks = (size_t)n / 2 + 2;
    char *scratch = nullptr;
    size_t bytes = (size_t)n * (24 + 12 + 4 + 4) + 2 * max_tasks * sizeof(Task) + 64;
    cudaError_t err = cudaMalloc(&scratch, bytes);
    if (err != cudaSuccess) return err;
    float *box = (float *)scratch;
    float *cen = box + 6 * (size_t)n;
    uint32_t *idx0 = (uint32_t *)(cen + 3 * (size_t)n);
    uint32_t *idx1 = idx0 + n;
    Task *tasks0 = (Task *)(idx1 + n);
    Task *tasks1 = tasks0 + max_tasks;
    uint32_t *counters = (uint32_t *)(tasks1 + max_tasks);
    err = cudaMalloc(&out->nodes, max_nodes * 64);
    if (err == cudaSuccess) err = cudaMalloc(&out->leaf_tris, (size_t)n * 48);
    if (err != cudaSuccess) {
        cudaFree(scratch);
        cudaFree(out->nodes);
        out->nodes = nullptr;
        return err;
    }
    k_prim_bounds<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(d_tri, n, box, cen, idx0);
    Task root{0, 0, n, 0};
    uint32_t init[4] = {0, 1, 0, 0};
    cudaMemcpyAsync(tasks0, &root, sizeof root, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(counters, init, sizeof init, cudaMemcpyHostToDevice, st);
    uint32_t ntasks = 1, level = 0;
    uint32_t *idx_in = idx0, *idx_out = idx1;
    Task *tin = tasks0, *tout = tasks1;
    uint32_t host_counters[4];
    while (ntasks > 0 && err == cudaSuccess) {
        BuildArgs a{d_tri, box, cen, idx_in, idx_out, tin, tout, counters, (float4 *)out->nodes,
                    (float4 *)out->leaf_tris};
        k_build_level<<<ntasks, kBlock, 0, st>>>(a);
        err = cudaGetLastError();
        if (err != cudaSuccess) break;
        err = cudaMemcpyAsync(host_counters, counters, sizeof host_counters, cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
        if (err != cudaSuccess) break;
        ntasks = host_counters[0];
        err = cudaMemsetAsync(counters, 0, sizeof(uint32_t), st);
        std::swap(idx_in, idx_out);
        std::swap(tin, tout);
        if (++level > 200) { err = cudaErrorUnknown; break; }  // cannot happen: each level halves a range
    }
    if (err == cudaSuccess && host_counters[3] != n) err = cudaErrorUnknown;  // every triangle in one leaf
    if (err == cudaSuccess) {
        out->num_nodes = host_counters[1];
        out->max_depth = host_counters[2] + 1;
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&out->build_ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(scratch);
    if (err != cudaSuccess) {
        cudaFree(out->nodes);
        cudaFree(out->leaf_tris);
        out->nodes = out->leaf_tris = nullptr;
    }
    return err;
}

}  // namespace lt
