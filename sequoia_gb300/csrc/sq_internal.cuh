// sq_internal.cuh -- host-side internals shared by the C-ABI translation
// units (sq_api.cu, sq_batch.cu): context and BVH objects, the caching device
// allocator, pointer-kind detection and error helpers.
#pragma once

#include "sq_common.cuh"

#include <map>
#include <string>

using sq::Node;

struct sq_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    uint32_t* ctrl = nullptr;  // [0] device error word, [1] work counter, [4..11] trace stats (4 x u64)
    std::multimap<size_t, void*> free_blocks;
    std::map<void*, size_t> live_blocks;
    cudaEvent_t ev[8] = {};
    bool build_timed = false, trace_timed = false;
    uint32_t* host_ctl = nullptr;  // pinned, 64 bytes: per-level task counts of the SAH build
    // fault injection (sq_debug_inject), each armed for one use: 0 = off,
    // else the wait's poll limit + 1; fail_alloc_in: allocations to let
    // through before one fails (-1 = off)
    uint32_t stall_lookback = 0, stall_barrier = 0;
    int64_t fail_alloc_in = -1;
    // banded camera traces into page-locked host memory (created on first
    // use): two streams the bands alternate on, so a band starts while the
    // one before it drains, and a copy stream that moves each finished band
    // to the host while later bands trace
    static constexpr int kMaxBands = 8;
    cudaStream_t band_stream[2] = {}, copy_stream = nullptr;
    cudaEvent_t band_fork = nullptr, band_done[kMaxBands] = {}, band_join[3] = {};
};

struct sq_bvh {
    sq_ctx* ctx = nullptr;
    Node* nodes = nullptr;
    uint32_t cap = 0;
    uint32_t root = 0;
    uint32_t n = 0;
    const float* tris = nullptr;  // device
    float* tris_own = nullptr;
    uint32_t kind = 0;
    float scene[6] = {0, 0, 0, 0, 0, 0};
    uint32_t* codes = nullptr;  // sorted codes (Morton builds)
    uint64_t* codes64 = nullptr;  // sorted 60-bit codes (SQ_BUILD_MORTON64)
    uint32_t* perm = nullptr;   // sorted permutation
    void* nodes8 = nullptr;     // 8-wide quantised nodes (SQ_BUILD_WIDE8)
    void* tris8 = nullptr;      // their 48-byte triangles
    uint32_t n8 = 0;
    uint32_t* meta8 = nullptr;  // device copy of (n8, levels8) not yet read back (cooperative collapse)
    uint32_t levels8 = 0;       // levels of the 8-wide tree
    uint32_t launches8 = 0;     // collapse kernel launches
    uint32_t* ws8 = nullptr;    // collapse queue state (its first word = nodes reserved)
    uint32_t leaf0 = 0;         // first leaf-region slot of the binary tree
};

namespace sqi {

sq_status fail(sq_ctx* c, sq_status st, const char* fmt, ...);
void* dalloc(sq_ctx* c, size_t bytes);
void dfree(sq_ctx* c, void* p);
bool is_device_ptr(const void* p);
sq_status check_device_error(sq_ctx* c, uint32_t* bits_out);
// Camera constants of a camera ray source as the kernels take them: the
// reference camera's origin, or the pinhole's eye, forward / right / up
// basis and image-plane half extents (14 floats).
void camera_params(const sq_ray_source& rs, float* cam);

struct Guard {
    int prev = -1;
    explicit Guard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~Guard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace sqi

#define SQ_CUDA(c, call)                                                                                     \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess)                                                                               \
            return sqi::fail((c), e_ == cudaErrorMemoryAllocation ? SQ_ERR_OOM : SQ_ERR_CUDA, "%s: %s (%s:%d)", \
                             #call, cudaGetErrorString(e_), __FILE__, __LINE__);                             \
    } while (0)
