// sq_common.cuh -- shared device types and helpers of libsequoia_gpu.
//
// Floating point: the library is compiled with -fmad=false, so a*b+c is two
// rounded operations everywhere, and `/`, sqrtf are IEEE round-to-nearest.
// Min/max that must reproduce the reference bit for bit are written as the
// reference's own comparisons (see ref_min / ref_max / simd_max below).
#pragma once

#include <utility>

#include <array>
#include <atomic>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <cuda_runtime.h>

#include "../../include/sequoia_gpu.h"

namespace sq {

constexpr uint32_t kNoHit = 0xFFFFFFFFu;
constexpr uint32_t kLeafFlag = 1u;

// Node record, same bytes as sq_node1 / the reference's Node1.
struct __align__(16) Node {
    float mnx, mny, mnz;
    uint32_t count_flags;  // count in the low 16 bits, flags in the high 16
    float mxx, mxy, mxz;
    uint32_t child;
};
static_assert(sizeof(Node) == 32, "Node must be 32 bytes");

__host__ __device__ inline uint32_t node_count(uint32_t cf) { return cf & 0xFFFFu; }
__host__ __device__ inline bool node_is_leaf(uint32_t cf) { return (cf >> 16) & kLeafFlag; }
__host__ __device__ inline uint32_t pack_cf(uint32_t count, uint32_t flags) { return (count & 0xFFFFu) | (flags << 16); }

// std::min(a, b) == (b < a) ? b : a  (src/vec3.h:179, src/simd_generic.h:164-168)
__device__ __forceinline__ float ref_min(float a, float b) { return (b < a) ? b : a; }
// std::max(a, b) == (a < b) ? b : a  (src/vec3.h:180)
__device__ __forceinline__ float ref_max(float a, float b) { return (a < b) ? b : a; }
// simd max: a > b ? a : b            (src/simd_generic.h:170-174)
__device__ __forceinline__ float simd_max(float a, float b) { return (a > b) ? a : b; }

// Order-preserving map float -> uint32 for atomicMax-based reductions.
__device__ __forceinline__ uint32_t float_to_ordered(float f)
{
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float ordered_to_float(uint32_t u)
{
    uint32_t b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

struct Box {
    float mn[3], mx[3];
};

__device__ __forceinline__ void box_reset(Box& b)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) { b.mn[k] = FLT_MAX; b.mx[k] = -FLT_MAX; }
}

__device__ __forceinline__ void box_grow(Box& b, const Box& o)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) { b.mn[k] = ref_min(b.mn[k], o.mn[k]); b.mx[k] = ref_max(b.mx[k], o.mx[k]); }
}

// Triangle AABB: min(min(v0, v1), v2), max(max(v0, v1), v2)  (src/builder.cpp:130-131)
__device__ __forceinline__ Box tri_box(const float* t)
{
    Box b;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        b.mn[k] = ref_min(ref_min(t[k], t[3 + k]), t[6 + k]);
        b.mx[k] = ref_max(ref_max(t[k], t[3 + k]), t[6 + k]);
    }
    return b;
}

__device__ __forceinline__ void load_tri(const float* __restrict__ tris, uint32_t i, float* t)
{
    const float* p = tris + 9ull * i;
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = __ldg(p + k);
}

__device__ __forceinline__ void store_node(Node* dst, const Box& b, uint32_t child, uint32_t count, uint32_t flags)
{
    float4 a = make_float4(b.mn[0], b.mn[1], b.mn[2], __uint_as_float(pack_cf(count, flags)));
    float4 c = make_float4(b.mx[0], b.mx[1], b.mx[2], __uint_as_float(child));
    reinterpret_cast<float4*>(dst)[0] = a;
    reinterpret_cast<float4*>(dst)[1] = c;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Relaxed (but coherent, untorn) GPU-scope load and store of a word that
// carries all its information itself, e.g. a look-back flag and count packed
// together: nothing else is published with it, so no ordering is needed and
// independent loads may be in flight together.
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// fetch-and-add with acquire-release semantics at GPU scope: the caller's
// earlier writes are visible to whoever later acquires this word, and the
// caller sees the writes released before earlier additions to it.
__device__ __forceinline__ uint32_t atomic_add_acq_rel_u32(uint32_t* p, uint32_t v)
{
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.volatile.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t bit)
{
    if (err) atomicOr(err, bit);
}

// float -> unsigned by truncation toward zero, negative values to 0 (the
// (uint8_t) conversions of src/tracer.cpp:222-225)
__host__ __device__ __forceinline__ uint32_t heat_f2u(float x) { return (x >= 0.0f) ? (uint32_t)x : 0u; }

// One heatmap pixel for a box-test count `tests` (or a packet's tests / k):
//   grey  (uint8)(min(1, tests / 200) * 255) in all three channels
//         (src/tracer.cpp:222-225);
//   ramp  the reference's get_heatmap_colour (src/tracer.cpp:25-45) of
//         tests / 200: black, blue, cyan, green, yellow, red at 0, 0.2, ...,
//         1, linear between neighbours; each channel (uint8)(c * 255).
// The ramp's arithmetic is the reference's, one rounding per operation:
// s = x * 5, i0 = floor(s), i2 = ceil(s), fract = i2 - s,
// c = col[i0] * fract + col[i2] * (1 - fract).
__device__ __forceinline__ void write_heat(uint8_t* hp, float tests, uint32_t ramp)
{
    const float x = tests / 200.0f;
    if (!ramp) {
        const float m = (x < 1.0f) ? x : 1.0f;
        const uint8_t v = (uint8_t)heat_f2u(m * 255.0f);
        hp[0] = v; hp[1] = v; hp[2] = v;
        return;
    }
    // stops: (r, g, b) bits of black, blue, cyan, green, yellow, red
    constexpr uint32_t kR = 0x30u, kG = 0x1Cu, kB = 0x06u;  // bit i: channel of stop i is 1
    float c[3];
    if (!(x > 0.0f)) {
        c[0] = c[1] = c[2] = 0.0f;
    } else if (x >= 1.0f) {
        c[0] = 1.0f; c[1] = 0.0f; c[2] = 0.0f;
    } else {
        const float s = x * 5.0f;
        const int i0 = (int)floorf(s), i2 = (int)ceilf(s);
        const float fract = (float)i2 - s;
        const float rest = 1.0f - fract;
        const uint32_t bits[3] = {kR, kG, kB};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float a = (float)((bits[k] >> i0) & 1u), b = (float)((bits[k] >> i2) & 1u);
            const float pa = a * fract, pb = b * rest;
            c[k] = pa + pb;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) hp[k] = (uint8_t)heat_f2u(c[k] * 255.0f);
}

constexpr int kNumSMs = 152;
constexpr int kMaxDevices = 64;

inline int current_device()
{
    int dev = 0;
    cudaGetDevice(&dev);
    return dev;
}

// A launch setting computed once per device: the first use on each device
// (the current one) computes it under a lock; later uses read it without
// one.  Occupancy, SM counts and function attributes such as the
// shared-memory opt-in belong to one device, so a process that drives
// contexts on several GPUs gets each GPU's own value.  Declare instances as
// function-local statics.
template <class T>
class PerDevice {
public:
    template <class Make>
    T get(Make&& make)
    {
        const int dev = current_device();
        if (dev < 0 || dev >= kMaxDevices) return make();
        if (ready_[dev].load(std::memory_order_acquire)) return value_[dev];
        std::lock_guard<std::mutex> lock(mu_);
        if (!ready_[dev].load(std::memory_order_relaxed)) {
            value_[dev] = make();
            ready_[dev].store(true, std::memory_order_release);
        }
        return value_[dev];
    }

private:
    std::mutex mu_;
    std::atomic<bool> ready_[kMaxDevices] = {};
    T value_[kMaxDevices] = {};
};

// Multiprocessor count of the current device.
inline int sm_count()
{
    static PerDevice<int> cache;
    return cache.get([] {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, current_device());
        return n > 0 ? n : kNumSMs;
    });
}

// Resident blocks per SM of a kernel at a block size on the current device
// (at least 1).
template <class Kernel>
inline int blocks_per_sm(Kernel kernel, int threads)
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0);
    return n > 0 ? n : 1;
}

// Programmatic dependent launch (chains of short kernels on one stream): a
// kernel launched with launch_chained may start while the kernel before it
// on the stream is still running; it calls chain_wait() before its first
// access to anything the earlier kernel writes (the wait returns once that
// kernel has completed and its writes are visible, as at a kernel boundary)
// and chain_release() to let the next kernel start launching.  Without a
// chained launch both are no-ops.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void chain_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
inline cudaError_t launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                  Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Trace statistics of one warp (box tests, triangle tests, requested bytes,
// node visits), summed over the warp's tiles in shared memory by lane 0 and
// added to the four global counters once, when the warp finishes: one atomic
// per counter per warp instead of one per tile, since same-address atomics
// serialise in L2.
struct WarpStats {
    unsigned long long v[4];
    __device__ __forceinline__ void reset(uint32_t lane)
    {
        if (lane == 0) v[0] = v[1] = v[2] = v[3] = 0ull;
    }
    __device__ __forceinline__ void add(uint32_t lane, unsigned long long a, unsigned long long b,
                                        unsigned long long c, unsigned long long d)
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
            b += __shfl_xor_sync(0xFFFFFFFFu, b, o);
            c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
            d += __shfl_xor_sync(0xFFFFFFFFu, d, o);
        }
        if (lane == 0) { v[0] += a; v[1] += b; v[2] += c; v[3] += d; }
    }
    __device__ __forceinline__ void flush(uint32_t lane, unsigned long long* g)
    {
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (v[k]) atomicAdd(g + k, v[k]);
        }
    }
};

}  // namespace sq

// ---------------------------------------------------------------------------
// Host-side launchers implemented in the .cu files, called by sq_api.cu.
namespace sqk {

// LBVH (sq_lbvh.cu)
// err: the context's device error word (SQ_DEVERR_COPY_TIMEOUT)
void scene_bounds(const float* tris, uint32_t n, uint32_t mode, uint32_t* box_ord, uint32_t* err, cudaStream_t s);
void morton_codes(const float* tris, uint32_t n, uint32_t mode, const uint32_t* box_ord, uint32_t* keys, uint32_t* vals,
                  uint32_t* hist, uint32_t digit_bits, uint32_t passes, uint32_t* err, cudaStream_t s);
// flags: n zeroed words; info: 6n float4 (a 48-byte record per boundary side)
// surv: n words of scratch for the nodes left to the global phase;
// surv_count: one zeroed word.
void lbvh_climb(const uint32_t* codes, const uint32_t* perm, const float* tris, uint32_t n, sq::Node* nodes,
                uint32_t* flags, float4* info, uint32_t* surv, uint32_t* surv_count, uint32_t* err, cudaStream_t s);
// The same climb over a batch: mesh m holds sorted positions [off[m],
// off[m + 1]) and gets its own tree, rooted at record root0 + m.
void lbvh_climb_seg(const uint32_t* codes, const uint32_t* perm, const float* tris, uint32_t n, const uint32_t* off,
                    uint32_t M, uint32_t root0, sq::Node* nodes, uint32_t* flags, float4* info, uint32_t* surv,
                    uint32_t* surv_count, uint32_t* err, cudaStream_t s);
// 60-bit codes (build_hierarchy_morton2): codes as low / high words with the
// histograms of 8 digit passes (4 per word); the high words re-ordered by
// the first sort stage; the combined sorted codes and permutation; the
// climb over 64-bit codes
void morton_codes64(const float* tris, uint32_t n, const uint32_t* box_ord, uint32_t* lo, uint32_t* hi,
                    uint32_t* vals, uint32_t* hist, cudaStream_t s);
void gather_high(const uint32_t* hi, const uint32_t* perm1, uint32_t n, uint32_t* hi1, uint32_t* pos, cudaStream_t s);
void combine64(const uint32_t* hi_sorted, const uint32_t* perm2, const uint32_t* lo_sorted, const uint32_t* perm1,
               uint32_t n, uint64_t* codes64, uint32_t* perm, cudaStream_t s);
void lbvh_climb64(const uint64_t* codes, const uint32_t* perm, const float* tris, uint32_t n, sq::Node* nodes,
                  uint32_t* flags, float4* info, uint32_t* surv, uint32_t* surv_count, uint32_t* err,
                  cudaStream_t s);

// onesweep radix sort (sq_sort.cu)
// keys per tile of a pass over n keys (512 per warp of the block: 4096 to 16384)
uint32_t sort_tile_keys(uint32_t n, uint32_t digit_bits);
size_t sort_lookback_words(uint32_t n, uint32_t digit_bits, uint32_t passes);
void sort_histogram(const uint32_t* keys, uint32_t n, uint32_t* hist, uint32_t digit_bits, uint32_t passes,
                    cudaStream_t s);
// Fault injection for the failure-detection tests: the first pass runs
// without its first tile, so the look-back of the tiles after it waits on
// words that nothing publishes and gives up after spin_limit empty polls
// (SQ_DEVERR_LOOKBACK_TIMEOUT).  Only for a one-pass sort whose output
// nothing else reads: every scatter position stays below the true one, so
// all writes stay inside the output.
struct SortStall {
    uint32_t spin_limit;
};
// Runs `passes` onesweep passes; hist/lookback/counters must be zeroed
// before (lookback and counters) and filled (hist).  With iota_values the
// first pass takes each key's index as its value and vals_a is not read.
// Returns which buffer holds the result: 0 = (keys_a, vals_a),
// 1 = (keys_b, vals_b).
int sort_passes(uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b, uint32_t* vals_b, uint32_t n,
                const uint32_t* hist, uint32_t* lookback, uint32_t* counters, uint32_t digit_bits,
                uint32_t passes, uint32_t* err, cudaStream_t s, const SortStall* stall = nullptr,
                bool iota_values = false);

// binned SAH / grid builders (sq_sah.cu)
size_t sah_workspace_bytes(uint32_t n);
size_t sah_batch_workspace_bytes(uint32_t n, uint32_t meshes);
// SAH trees of M meshes in one launch sequence with no host synchronisation
// (graph-capturable): mesh m = triangles [off[m], off[m + 1]) (off on the
// device), root record root0 + m, leaf records at 2n + 2 + position.
int build_sah_batch(const float* tris, uint32_t n, const uint32_t* off, uint32_t M, uint32_t nb, uint32_t leaf_size,
                    uint32_t root0, sq::Node* nodes, void* ws, uint32_t* err, cudaStream_t s);
int build_sah(const float* tris, uint32_t n, uint32_t nb, uint32_t leaf_size, int grid, uint32_t scene_box_cells,
              sq::Node* nodes, float* scene_out, void* ws, uint32_t* sort_keys, uint32_t* sort_vals,
              uint32_t* sort_alt_keys, uint32_t* sort_alt_vals, uint32_t* sort_lookback, uint32_t* sort_counters,
              uint32_t* err, uint32_t* host_ctl, cudaStream_t s);

// traversal (sq_trace.cu)
struct TraceArgs {
    const sq::Node* nodes;
    uint32_t node_count;  // indices are checked against these; a bad index
    uint32_t tri_count;   // ends the ray and raises SQ_DEVERR_TOPOLOGY
    uint32_t root;
    const float* tris;
    uint32_t mode;        // sq_trace_mode
    uint32_t ray_kind;    // sq_ray_kind
    uint32_t width, height;
    float cam[14];        // reference camera: origin in [0..2]; pinhole: basis
    const float* rays;    // explicit rays (8 floats each)
    uint32_t ray_count;
    sq_hit* hits;         // may be null
    uint8_t* heat;        // may be null
    uint32_t* work;       // persistent work counter (zeroed)
    uint32_t* err;
    unsigned long long* stats;  // {box tests, triangle tests, bytes requested, node visits}
    uint32_t refill;      // closest / any-hit: 1 = per-lane ray refill, 0 = 32-ray batches per warp
    uint32_t heat_ramp;   // heatmap pixels: 0 = grey, 1 = the reference's colour ramp (write_heat)
    uint32_t root_group;  // REF mode: start from the node group [root, root + root_group) (1 = the root)
};
void trace(const TraceArgs& a, cudaStream_t s);
// packet / bundle tracers of the reference (sq_coherent.cu): heatmap only
bool coherent_shape_ok(uint32_t bundle, uint32_t k, uint32_t w, uint32_t h);
void trace_coherent(const TraceArgs& a, uint32_t bundle, uint32_t k, cudaStream_t s);

// 8-wide quantised BVH (build: sq_bvh8.cu; traversal: sq_bvh8_trace.cu)
struct Trace8Args {
    const void* nodes;     // 80-byte wide nodes
    const float4* tris8;   // 48-byte triangles in leaf order, id in v0.w
    uint32_t mode, ray_kind, width, height;
    float cam[14];
    const float* rays;
    uint32_t ray_count;
    sq_hit* hits;
    uint8_t* heat;
    uint32_t* work;
    uint32_t* err;
    unsigned long long* stats;
    uint32_t refill;       // 1: per-lane ray refill; 0: whole 32-ray batches per warp
    uint32_t heat_ramp;    // heatmap pixels: 0 = grey, 1 = colour ramp (write_heat)
    // camera rays, tiles schedule: only tiles [tile0, tile_end) of the image
    // (tile_end 0: to the last tile), so an image can be traced in row bands
    uint32_t tile0, tile_end;
};
// Triangles an 8-wide BVH can address: a traversal stack entry holds the
// first triangle of a leaf range in 27 bits (and its count in 4).
constexpr uint32_t kWide8MaxTris = 1u << 27;
uint32_t bvh8_capacity(uint32_t n);
size_t bvh8_node_bytes(uint32_t n);
size_t bvh8_ws_words(uint32_t n);
size_t bvh8_tri_bytes(uint32_t n);
// meta (device, 2 words, may be null): when given and the cooperative
// collapse runs, the node count and level count are copied there on the
// stream instead of being read back (no host synchronisation); host_ctl[4]
// then holds 2 and host_ctl[0] / [3] are not written.  Returns 1 in
// host_ctl[5] when meta was filled that way, else 0.
// Fault injection for the failure-detection tests: the cooperative
// collapse's grid barrier waits for one block more than the grid, so every
// block gives up after spin_limit polls (SQ_DEVERR_SAH_QUEUE) and returns.
struct BarrierStall {
    uint32_t spin_limit;
};
int build_bvh8(const sq::Node* rec, uint32_t root, uint32_t leaf0, const float* tris, uint32_t n, void* nodes8,
               void* tris8, uint32_t* ws, uint32_t* host_ctl, uint32_t* err, cudaStream_t s, uint32_t* meta = nullptr,
               const BarrierStall* stall = nullptr);
void trace8(const Trace8Args& a, cudaStream_t s);

// batched trace over many BVHs and ray tiles (sq_trace.cu, sq_bvh8_trace.cu)
struct BatchJob {
    uint32_t ray_kind;     // sq_ray_kind
    uint32_t width, height;
    uint32_t ray_count;    // rays of this job
    uint32_t ray_offset;   // explicit rays: first ray in the concatenated ray array
    uint32_t out_offset;   // first hit record / heatmap pixel of this job
    uint32_t root;         // binary root record, or 8-wide root node
    uint32_t batch_begin;  // first 32-ray batch of this job
    uint32_t tri_offset;   // subtracted from reported triangle ids
    uint32_t pad;
    const float* rays;     // explicit rays of this job (null: the shared ray array at ray_offset)
    float cam[16];         // reference camera origin, or pinhole basis (14 floats)
};
static_assert(sizeof(BatchJob) == 112, "BatchJob is 112 bytes");

struct BatchTraceArgs {
    const sq::Node* nodes;
    uint32_t node_count, tri_count;
    const void* nodes8;
    const float4* tris8;
    const float* tris;
    const float* rays;
    const BatchJob* jobs;
    uint32_t njobs, total_batches, mode;
    sq_hit* hits;
    uint8_t* heat;
    uint32_t* work;
    uint32_t* err;
    unsigned long long* stats;
    uint32_t refill;       // 8-wide kernel: 1 = per-lane ray refill (see sq_bvh8_trace.cu)
    uint32_t heat_ramp;    // heatmap pixels: 0 = grey, 1 = colour ramp (write_heat)
};
void trace_batch(const BatchTraceArgs& a, int block_threads, cudaStream_t s);
void trace8_batch(const BatchTraceArgs& a, int block_threads, cudaStream_t s);

// 8-wide collapse seeded with several roots, with no host synchronisation
// (a fixed number of level kernels with device-side task counts), so it can
// be captured in a CUDA graph.  ws: bvh8_ws_words(n) + 4 * nroots words.
// Wide node k (k < nroots) is the tree of roots[k].
int build_bvh8_queue(const sq::Node* rec, const uint32_t* roots_dev, uint32_t nroots, uint32_t leaf0, const float* tris,
                     uint32_t n, void* nodes8, void* tris8, uint32_t* ws, uint32_t* err, cudaStream_t s);

}  // namespace sqk

// Shared helpers for locating a 32-ray batch in a job table.
namespace sq {
__device__ __forceinline__ uint32_t find_job(const sqk::BatchJob* __restrict__ jobs, uint32_t njobs, uint32_t b)
{
    uint32_t lo = 0, hi = njobs;  // largest j with jobs[j].batch_begin <= b
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&jobs[mid].batch_begin) <= b) lo = mid; else hi = mid;
    }
    return lo;
}
}  // namespace sq
