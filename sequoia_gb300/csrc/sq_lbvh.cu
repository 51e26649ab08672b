// sq_lbvh.cu -- Morton codes and LBVH emission on the GPU.
//
// Pipeline of a Morton build (Builder::build_hierarchy_morton,
// src/builder.cpp:2474-2508):
//   k_scene_bounds  union of the triangle AABBs (src/builder.cpp:2206-2215)
//   k_morton        30-bit codes (src/builder.cpp:2217-2236) + the digit
//                   histograms of every radix-sort pass, in one read
//   onesweep sort   (sq_sort.cu)
//   k_lbvh_climb    topology, bounds and node records bottom-up: leaf and
//                   warp phases; lists the nodes whose sibling finishes in
//                   another warp
//   k_lbvh_global   the rest of the climb, one thread per listed node
//
// The climb builds the same logical tree as recurse_morton /
// find_split_morton (src/builder.cpp:2281-2409): ranges of fewer than 8
// triangles become leaf clusters, a range whose first and last codes are
// equal is split after (count >> 1) + 1 triangles, and any other range is
// split where the highest differing code bit flips.  The last rule is the
// binary radix tree over the distinct codes, so runs of equal codes are its
// leaves.  Each run head climbs that tree bottom-up (Apetrei, "Fast and
// Simple Agglomerative LBVH Construction", 2014): the parent of a node over
// [l, r) splits at whichever neighbouring boundary, l or r, has the smaller
// code XOR, and the second thread to reach a parent continues with the union
// of both children.  Records go to the range-tree layout described in
// oracle/sq_oracle.c, so the GPU and the oracle write identical records.
#include "sq_common.cuh"
#include "sq_lbvh_dev.cuh"

#include <algorithm>
#include <cstdio>

namespace {

using namespace sq;

constexpr int kTileTris = 256;  // triangles staged per block iteration

// Stage triangles [first, first + count) of a 16-byte aligned array into
// shared memory with float4 loads (first is a multiple of kTileTris, so the
// tile start is 16-byte aligned: 256 * 36 bytes = 9216 bytes).
__device__ __forceinline__ void stage_tris(const float* __restrict__ tris, uint32_t first, uint32_t count,
                                           float* s, bool aligned)
{
    const uint32_t nf = count * 9u;
    const float* src = tris + 9ull * first;
    if (aligned) {
        const uint32_t nv = nf >> 2;
        const float4* src4 = reinterpret_cast<const float4*>(src);
        float4* s4 = reinterpret_cast<float4*>(s);
        for (uint32_t j = threadIdx.x; j < nv; j += blockDim.x) s4[j] = __ldg(src4 + j);
        for (uint32_t j = (nv << 2) + threadIdx.x; j < nf; j += blockDim.x) s[j] = __ldg(src + j);
    } else {
        for (uint32_t j = threadIdx.x; j < nf; j += blockDim.x) s[j] = __ldg(src + j);
    }
}

// ---------------------------------------------------------------------------
// Bulk-copy staging of triangle tiles (TMA, cp.async.bulk): two shared
// buffers per block, each completed through its own mbarrier, so the copy of
// a block's next tile is in flight while the current one is processed.  A
// tile of kTileTris triangles is 9216 bytes, a multiple of 16, and starts on
// a 16-byte boundary when the array does; the last tile, when partial, is
// read with plain loads.  Waits are bounded: a copy that does not complete
// raises SQ_DEVERR_COPY_TIMEOUT and the block gives up.
constexpr uint32_t kTileBytes = kTileTris * 36u;
constexpr uint32_t kCopySpins = 1u << 22;

struct TileStage {
    float tri[2][kTileTris * 9];
    unsigned long long bar[2];
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// thread 0: start the copy of full tile t into buffer b
__device__ __forceinline__ void stage_issue(TileStage& st, int b, const float* __restrict__ tris, uint32_t t)
{
    const uint32_t bar = smem_addr(&st.bar[b]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kTileBytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(st.tri[b])), "l"(tris + 9ull * kTileTris * t), "r"(kTileBytes), "r"(bar)
                 : "memory");
}

// every thread: wait for phase `parity` of buffer b's barrier (bounded)
__device__ __forceinline__ bool stage_wait(TileStage& st, int b, uint32_t parity)
{
    const uint32_t bar = smem_addr(&st.bar[b]);
    for (uint32_t spins = 0; spins < kCopySpins; ++spins) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// Calls body(s_tri, first, count) for each of this block's tiles (tile
// blockIdx.x + k * gridDim.x), tiles staged as described above; every thread
// of the block must call it.  Falls back to plain staged loads when the
// array is not 16-byte aligned.
template <class Body>
__device__ void for_each_tile(const float* __restrict__ tris, uint32_t n, bool aligned, uint32_t* err, Body body)
{
    __shared__ __align__(128) TileStage st;
    const uint32_t ntiles = (n + kTileTris - 1) / kTileTris, full = n / kTileTris;
    if (!aligned) {
        for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const uint32_t first = t * kTileTris, count = min((uint32_t)kTileTris, n - first);
            __syncthreads();
            stage_tris(tris, first, count, st.tri[0], false);
            __syncthreads();
            body(st.tri[0], first, count);
        }
        return;
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&st.bar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&st.bar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // per buffer: the barrier phase to wait for, and whether a copy into it
    // has been started and not yet waited for (the same in every thread)
    uint32_t parity[2] = {0u, 0u};
    bool pending[2] = {false, false};
    uint32_t t = blockIdx.x;
    if (t < full) {
        if (threadIdx.x == 0) stage_issue(st, 0, tris, t);
        pending[0] = true;
    }
    bool ok = true;
    for (int b = 0; t < ntiles; t += gridDim.x, b ^= 1) {
        const uint32_t next = t + gridDim.x;
        // buffer b ^ 1 was released by the barrier that ended the last tile
        if (next < full) {
            if (threadIdx.x == 0) stage_issue(st, b ^ 1, tris, next);
            pending[b ^ 1] = true;
        }
        const uint32_t first = t * kTileTris, count = min((uint32_t)kTileTris, n - first);
        if (t < full) {
            ok = stage_wait(st, b, parity[b]);
            if (ok) {
                parity[b] ^= 1u;
                pending[b] = false;
            }
        } else {
            stage_tris(tris, first, count, st.tri[b], true);  // the partial last tile
        }
        if (!__syncthreads_and(ok)) break;
        body(st.tri[b], first, count);
        __syncthreads();
    }
    if (!__syncthreads_and(ok)) {
        // give up: wait (bounded) for the copies this block started, so none
        // lands in shared memory after the block has left
        if (threadIdx.x == 0) {
            raise_error(err, SQ_DEVERR_COPY_TIMEOUT);
            for (int b = 0; b < 2; ++b)
                if (pending[b]) stage_wait(st, b, parity[b]);
        }
        __syncthreads();
        return;
    }
    // every copy has completed: retire the barriers before the shared memory
    // is used for anything else
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(&st.bar[0])) : "memory");
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(&st.bar[1])) : "memory");
    }
}

__device__ __forceinline__ float warp_min(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

// box_ord[k] = ordered(-min_k), box_ord[3 + k] = ordered(max_k); zero-initialised.
__global__ void __launch_bounds__(256) k_scene_bounds(const float* __restrict__ tris, uint32_t n, uint32_t mode,
                                                      uint32_t* __restrict__ box_ord, bool aligned, uint32_t* err)
{
    chain_wait();  // a chained launch (the build's kernels follow one another)
    chain_release();
    __shared__ float s_red[8][6];
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for_each_tile(tris, n, aligned, err, [&](const float* s_tri, uint32_t, uint32_t count) {
        if (threadIdx.x < count) {
            Box b = tri_box(s_tri + 9 * threadIdx.x);
            if (mode == SQ_MORTON_BOUNDS_CENTROID) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float c = (b.mn[k] + b.mx[k]) * 0.5f;
                    mn[k] = fminf(mn[k], c);
                    mx[k] = fmaxf(mx[k], c);
                }
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) { mn[k] = fminf(mn[k], b.mn[k]); mx[k] = fmaxf(mx[k], b.mx[k]); }
            }
        }
    });
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) { mn[k] = warp_min(mn[k]); mx[k] = warp_max(mx[k]); }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) { s_red[warp][k] = mn[k]; s_red[warp][3 + k] = mx[k]; }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        float v = s_red[0][k];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = (k < 3) ? fminf(v, s_red[w][k]) : fmaxf(v, s_red[w][k]);
        atomicMax(box_ord + k, float_to_ordered(k < 3 ? -v : v));
    }
}

// Spread the low 10 bits of v to every third bit (bit i -> bit 3i).
__device__ __forceinline__ uint32_t spread10(uint32_t v)
{
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t f2u(float x) { return (x >= 0.0f) ? (uint32_t)x : 0u; }

template <int DB, int PASSES>
__global__ void __launch_bounds__(256) k_morton(const float* __restrict__ tris, uint32_t n, uint32_t mode,
                                                const uint32_t* __restrict__ box_ord, uint32_t* __restrict__ keys,
                                                uint32_t* __restrict__ vals, uint32_t* __restrict__ hist, bool aligned,
                                                uint32_t* err)
{
    chain_wait();  // a chained launch (the build's kernels follow one another)
    chain_release();
    constexpr int RADIX = 1 << DB;
    __shared__ uint32_t s_hist[PASSES * RADIX];
    for (int j = threadIdx.x; j < PASSES * RADIX; j += blockDim.x) s_hist[j] = 0;
    float smin[3], ext[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        smin[k] = -ordered_to_float(box_ord[k]);
        const float smax = ordered_to_float(box_ord[3 + k]);
        ext[k] = smax - smin[k];
    }
    (void)mode;
    for_each_tile(tris, n, aligned, err, [&](const float* s_tri, uint32_t first, uint32_t count) {
        if (threadIdx.x < count) {
            const Box b = tri_box(s_tri + 9 * threadIdx.x);
            uint32_t q[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                // centre = (bb_min + bb_max) * 0.5f; (centre - min) / (max - min); * 0x3FF
                const float c = (b.mn[k] + b.mx[k]) * 0.5f;
                const float u = (c - smin[k]) / ext[k];
                q[k] = f2u(u * 1023.0f);
            }
            const uint32_t code = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
            const uint32_t i = first + threadIdx.x;
            keys[i] = code;
            if (vals) vals[i] = i;  // null when the sort's first pass generates the indices
#pragma unroll
            for (int p = 0; p < PASSES; ++p) atomicAdd(&s_hist[p * RADIX + ((code >> (p * DB)) & (RADIX - 1))], 1u);
        }
    });
    __syncthreads();
    for (int j = threadIdx.x; j < PASSES * RADIX; j += blockDim.x) {
        const uint32_t c = s_hist[j];
        if (c) atomicAdd(hist + j, c);
    }
}

// Spread the low 21 bits of v to every third bit (bit i -> bit 3i).
__device__ __forceinline__ uint64_t spread21(uint64_t v)
{
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x001F00000000FFFFull;
    v = (v | (v << 16)) & 0x001F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// 60-bit codes of build_hierarchy_morton2 (setup_morton2,
// src/builder.cpp:2247-2279: 0xFFFFF steps per axis, x at bit 0), split into
// low and high words, plus the 8-bit digit histograms of both words (four
// passes each: hist[0..4) the low word, hist[4..8) the high word).
__global__ void __launch_bounds__(256) k_morton64(const float* __restrict__ tris, uint32_t n,
                                                  const uint32_t* __restrict__ box_ord, uint32_t* __restrict__ lo,
                                                  uint32_t* __restrict__ hi, uint32_t* __restrict__ vals,
                                                  uint32_t* __restrict__ hist, bool aligned)
{
    __shared__ __align__(16) float s_tri[kTileTris * 9];
    __shared__ uint32_t s_hist[8 * 256];
    for (int j = threadIdx.x; j < 8 * 256; j += blockDim.x) s_hist[j] = 0;
    float smin[3], ext[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        smin[k] = -ordered_to_float(box_ord[k]);
        ext[k] = ordered_to_float(box_ord[3 + k]) - smin[k];
    }
    for (uint32_t first = blockIdx.x * kTileTris; first < n; first += gridDim.x * kTileTris) {
        const uint32_t count = min((uint32_t)kTileTris, n - first);
        __syncthreads();
        stage_tris(tris, first, count, s_tri, aligned);
        __syncthreads();
        if (threadIdx.x < count) {
            const Box b = tri_box(s_tri + 9 * threadIdx.x);
            uint64_t q[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float c = (b.mn[k] + b.mx[k]) * 0.5f;
                const float u = (c - smin[k]) / ext[k];
                q[k] = f2u(u * 1048575.0f);
            }
            const uint64_t code = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
            const uint32_t i = first + threadIdx.x;
            const uint32_t l = (uint32_t)code, h = (uint32_t)(code >> 32);
            lo[i] = l;
            hi[i] = h;
            vals[i] = i;
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                atomicAdd(&s_hist[p * 256 + ((l >> (8 * p)) & 255u)], 1u);
                atomicAdd(&s_hist[(4 + p) * 256 + ((h >> (8 * p)) & 255u)], 1u);
            }
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < 8 * 256; j += blockDim.x) {
        const uint32_t c = s_hist[j];
        if (c) atomicAdd(hist + j, c);
    }
}

// Second sort stage of the 60-bit codes: the high words in the order of the
// first stage, keyed by position.
__global__ void k_gather_high(const uint32_t* __restrict__ hi, const uint32_t* __restrict__ perm1, uint32_t n,
                              uint32_t* __restrict__ hi1, uint32_t* __restrict__ pos)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        hi1[i] = hi[perm1[i]];
        pos[i] = i;
    }
}

// codes64[i] = hi_sorted[i] : lo_sorted[perm2[i]], perm[i] = perm1[perm2[i]]
__global__ void k_combine64(const uint32_t* __restrict__ hi_sorted, const uint32_t* __restrict__ perm2,
                            const uint32_t* __restrict__ lo_sorted, const uint32_t* __restrict__ perm1, uint32_t n,
                            uint64_t* __restrict__ codes64, uint32_t* __restrict__ perm)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j = perm2[i];
        codes64[i] = ((uint64_t)hi_sorted[i] << 32) | lo_sorted[j];
        perm[i] = perm1[j];
    }
}

// ---------------------------------------------------------------------------
// climb

// Sibling record of a node beside its parent boundary p: box, far end,
// split and the code XOR at the far end (left child: slot 2p, right: 2p + 1).
__device__ __forceinline__ void publish_record(float4* __restrict__ info, uint32_t p, bool left, const Box& box,
                                               uint32_t far_end, uint32_t split, uint64_t dfar)
{
    float4* mine = info + 3ull * (2ull * p + (left ? 0u : 1u));
    mine[0] = make_float4(box.mn[0], box.mn[1], box.mn[2], __uint_as_float(far_end));
    mine[1] = make_float4(box.mx[0], box.mx[1], box.mx[2], __uint_as_float(split));
    mine[2] = make_float4(__uint_as_float((uint32_t)dfar), __uint_as_float((uint32_t)(dfar >> 32)), 0.0f, 0.0f);
}

// Leaf and warp phases of the climb.  Nodes still open after the warp phase
// (their sibling finishes in another warp) publish their record and are
// listed as (parent boundary | left << 31) in surv for k_lbvh_global; a
// block takes its slots with one atomic on surv_count.  Splitting the climb
// this way lets these blocks retire at once: waiting out a global climb held
// their SM slots from the blocks still to run.
//
// SEG: positions [off[m], off[m + 1]) hold mesh m of a batch, sorted by
// (mesh, code), and each mesh gets its own tree: runs, parents and the root
// never cross a segment boundary, and mesh m's root record goes to slot
// root0 + m (without SEG the single segment is [0, n) and its root slot 0).
// Parent boundaries of different meshes never coincide: a node's parent
// boundary lies strictly inside its mesh's range.  256 threads and at most
// 40 registers: six blocks per SM, so more blocks overlap their leaf gathers.
template <class Code, bool SEG>
__global__ void __launch_bounds__(256, 6) k_lbvh_climb(const Code* __restrict__ codes, const uint32_t* __restrict__ perm,
                                                    const float* __restrict__ tris, uint32_t n, Node* __restrict__ nodes,
                                                    float4* __restrict__ info, uint32_t* __restrict__ surv,
                                                    uint32_t* __restrict__ surv_count, const uint32_t* __restrict__ off,
                                                    uint32_t M, uint32_t root0, uint32_t* err)
{
    chain_wait();  // a chained launch (the build's kernels follow one another)
    chain_release();
    constexpr uint32_t FULL = 0xFFFFFFFFu;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = (int)(threadIdx.x & 31u);
    const uint32_t leaf0 = 2u * n + 2u;
    // this position's segment [sb, se) and mesh
    uint32_t sb = 0, se = n, m = 0;
    if (SEG && i < n) {
        m = mesh_of(off, M, i);
        sb = __ldg(off + m);
        se = __ldg(off + m + 1);
    }
    // this lane's node: [l, r) with its box and split, while `active`
    bool active = false;
    uint32_t l = 0, r = 0, split = 0;
    Code dl = 0, dr = 0;  // code XOR at boundaries l and r (where they are inside (0, n))
    Box box;
    box_reset(box);
    // codes of this position and its neighbours (shuffled within the warp)
    const uint32_t W = i - (uint32_t)lane;  // the warp's first position
    const Code code = i < n ? codes[i] : Code(0);
    Code prev = __shfl_up_sync(FULL, code, 1), next = __shfl_down_sync(FULL, code, 1);
    if (lane == 0 && i > 0 && i < n) prev = codes[i - 1];
    if (lane == 31 && i + 1 < n) next = codes[i + 1];
    // d_own = code XOR at boundary i (between positions i - 1 and i); d_end =
    // the XOR at boundary W + 32, just past the warp
    const Code d_own = prev ^ code;
    const Code d_end = __shfl_sync(FULL, code ^ next, 31);
    if (i < n) {
        if (i == sb || prev != code) {  // a run head
            uint32_t e = i + 1;
            if (e < se && next == code) {
                ++e;
                while (e < se && e < i + 8 && codes[e] == code) ++e;
            }
            if (e == i + 8 && e < se && codes[e] == code) {
                uint32_t lo = e, hi = se;
                while (lo < hi) {
                    const uint32_t mid = lo + ((hi - lo) >> 1);
                    if (codes[mid] == code) lo = mid + 1; else hi = mid;
                }
                e = lo;
            }
            // leaf records of the run and the run box
            for (uint32_t p = i; p < e; ++p) {
                const uint32_t t = perm[p];
                float tv[9];
                load_tri(tris, t, tv);
                const Box b = tri_box(tv);
                store_node(nodes + leaf0 + p, b, t, 1u, kLeafFlag);
                box_grow(box, b);
            }
            if (e - i >= 8) run_subtree(i, e, leaf0, nodes, box, split, err);
            l = i;
            r = e;
            active = true;
        }
    }
    {
        // the XOR at the run's end comes from the lane that owns it when it is
        // inside the warp
        const bool r_in = active && r - W < 32u;
        const Code dr_in = __shfl_sync(FULL, d_own, r_in ? (int)(r - W) : lane);
        if (active) {
            dl = d_own;
            if (r_in) dr = dr_in;
            else if (r == W + 32u) dr = d_end;
            else if (r < se) dr = codes[r - 1] ^ codes[r];
        }
    }

    // The parent of a node over [l, r) splits at boundary l or r (whichever
    // has the smaller code XOR with its neighbour); the node is its left
    // child when the split is at r.
    auto parent_of = [&](uint32_t& p, bool& left) {
        if (l == sb) { p = r; left = true; }
        else if (r == se) { p = l; left = false; }
        else if (dr < dl) { p = r; left = true; }
        else { p = l; left = false; }
    };
    auto write_root = [&]() {
        Node* root = nodes + (SEG ? root0 + m : 0u);
        if (se - sb >= 8) store_node(root, box, 2u * split, 2u, 0);
        else store_node(root, box, leaf0 + sb, se - sb, 0);
    };
    // Merge this node with its sibling (ending or starting at s_end, with the
    // code XOR s_d at that far boundary): write both children's records when
    // the parent is an inner node, and continue with the parent.
    auto merge = [&](uint32_t p, bool left, uint32_t s_end, const Box& sb, uint32_t s_split, Code s_d) {
        uint32_t ll, rr, lsplit, rsplit;
        Box lb, rb;
        if (left) { ll = l; rr = s_end; lb = box; rb = sb; lsplit = split; rsplit = s_split; dr = s_d; }
        else { ll = s_end; rr = r; lb = sb; rb = box; lsplit = s_split; rsplit = split; dl = s_d; }
        if (rr - ll >= 8) {
            write_child(nodes, 2u * p, ll, p, lb, lsplit, leaf0);
            write_child(nodes, 2u * p + 1u, p, rr, rb, rsplit, leaf0);
        }
        box = lb;
        box_grow(box, rb);
        l = ll;
        r = rr;
        split = p;
    };

    // Warp phase: nodes whose two children both finish inside this warp are
    // merged through shuffles, in rounds, until a round merges nothing; only
    // the nodes left then go to the global protocol (k_lbvh_global).  Most
    // small subtrees never touch the sibling records or the flags.  A node
    // [l, r) is always held by the lane of its first position, l - W (run
    // heads start there, and a merge continues in the left child's lane), so
    // a left child (parent boundary r) finds its sibling in lane r - W: the
    // node there must be active and name boundary r as its own parent, as the
    // right child.  The right child learns that it was merged from an OR of
    // the lanes the left children took.
    for (;;) {
        if (active && l == sb && r == se) { write_root(); active = false; }
        if (!__any_sync(FULL, active)) break;
        uint32_t p = 0;
        bool left = false;
        if (active) parent_of(p, left);
        // (parent boundary, side, active) of every lane; parent boundaries
        // are below 2^30
        const uint32_t me = active ? (p << 2) | (left ? 2u : 0u) | 1u : 0u;
        const bool look = active && left && r - W < 32u;
        const int src = look ? (int)(r - W) : lane;
        const uint32_t other = __shfl_sync(FULL, me, src);
        const bool take = look && other == ((r << 2) | 1u);
        const uint32_t o_r = __shfl_sync(FULL, r, src);
        const Code o_dr = __shfl_sync(FULL, dr, src);
        const uint32_t o_split = __shfl_sync(FULL, split, src);
        Box ob;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            ob.mn[k] = __shfl_sync(FULL, box.mn[k], src);
            ob.mx[k] = __shfl_sync(FULL, box.mx[k], src);
        }
        const uint32_t taken = __reduce_or_sync(FULL, take ? 1u << src : 0u);
        if (take) merge(p, true, o_r, ob, o_split, o_dr);
        if ((taken >> lane) & 1u) active = false;
        if (!taken) break;
    }

    uint32_t p = 0;
    bool left = false;
    if (active) {
        parent_of(p, left);
        publish_record(info, p, left, box, left ? l : r, split, (uint64_t)(left ? dl : dr));
    }
    __shared__ uint32_t s_count, s_base;
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    const uint32_t am = __ballot_sync(FULL, active);
    uint32_t woff = 0;
    if (lane == 0 && am) woff = atomicAdd(&s_count, (uint32_t)__popc(am));
    woff = __shfl_sync(FULL, woff, 0);
    __syncthreads();
    if (threadIdx.x == 0) s_base = s_count ? atomicAdd(surv_count, s_count) : 0u;
    __syncthreads();
    if (active) surv[s_base + woff + __popc(am & ((1u << lane) - 1u))] = p | (left ? 0x80000000u : 0u);
}

// Global phase of the climb (Apetrei's protocol): each listed node counts its
// arrival at its parent boundary (release its record, acquire the sibling's);
// the second arrival merges the two and continues with the parent, whose
// record it publishes first.  Nothing waits: a first arrival stops.
template <class Code, bool SEG>
__global__ void __launch_bounds__(256, 6) k_lbvh_global(const uint32_t* __restrict__ surv,
                                                     const uint32_t* __restrict__ surv_count, uint32_t n,
                                                     Node* __restrict__ nodes, uint32_t* __restrict__ flags,
                                                     float4* __restrict__ info, const uint32_t* __restrict__ off,
                                                     uint32_t M, uint32_t root0, uint32_t* err)
{
    chain_wait();  // a chained launch (the build's kernels follow one another)
    chain_release();
    const uint32_t leaf0 = 2u * n + 2u;
    const uint32_t count = *surv_count;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        const uint32_t e = surv[t];
        uint32_t p = e & 0x7FFFFFFFu;
        bool left = (e >> 31) != 0u;
        // the node's segment: its parent boundary lies inside it
        uint32_t sb = 0, se = n, m = 0;
        if (SEG) {
            m = mesh_of(off, M, p);
            sb = __ldg(off + m);
            se = __ldg(off + m + 1);
        }
        // this node from its own record; the XOR at its near end (boundary p)
        // is not needed: the merge replaces it with the sibling's far XOR
        const float4* mine = info + 3ull * (2ull * p + (left ? 0u : 1u));
        const float4 m0 = __ldcg(mine), m1 = __ldcg(mine + 1), m2 = __ldcg(mine + 2);
        Box box;
        box.mn[0] = m0.x; box.mn[1] = m0.y; box.mn[2] = m0.z;
        box.mx[0] = m1.x; box.mx[1] = m1.y; box.mx[2] = m1.z;
        uint32_t split = __float_as_uint(m1.w);
        const Code dfar = (Code)((uint64_t)__float_as_uint(m2.x) | ((uint64_t)__float_as_uint(m2.y) << 32));
        uint32_t l, r;
        Code dl = 0, dr = 0;
        if (left) { l = __float_as_uint(m0.w); r = p; dl = dfar; }
        else { l = p; r = __float_as_uint(m0.w); dr = dfar; }
        for (bool first = true;; first = false) {
            if (!first) {
                if (l == sb && r == se) {
                    Node* root = nodes + (SEG ? root0 + m : 0u);
                    if (se - sb >= 8) store_node(root, box, 2u * split, 2u, 0);
                    else store_node(root, box, leaf0 + sb, se - sb, 0);
                    break;
                }
                if (l == sb) { p = r; left = true; }
                else if (r == se) { p = l; left = false; }
                else if (dr < dl) { p = r; left = true; }
                else { p = l; left = false; }
                publish_record(info, p, left, box, left ? l : r, split, (uint64_t)(left ? dl : dr));
            }
            const uint32_t old = atomic_add_acq_rel_u32(flags + p, 1u);
            if (old == 0) break;
            if (old != 1) { raise_error(err, SQ_DEVERR_TOPOLOGY); break; }
            const float4* sib = info + 3ull * (2ull * p + (left ? 1u : 0u));
            const float4 s0 = __ldcg(sib), s1 = __ldcg(sib + 1), s2 = __ldcg(sib + 2);
            Box sb;
            sb.mn[0] = s0.x; sb.mn[1] = s0.y; sb.mn[2] = s0.z;
            sb.mx[0] = s1.x; sb.mx[1] = s1.y; sb.mx[2] = s1.z;
            const Code s_d = (Code)((uint64_t)__float_as_uint(s2.x) | ((uint64_t)__float_as_uint(s2.y) << 32));
            const uint32_t s_end = __float_as_uint(s0.w), s_split = __float_as_uint(s1.w);
            uint32_t ll, rr, lsplit, rsplit;
            Box lb, rb;
            if (left) { ll = l; rr = s_end; lb = box; rb = sb; lsplit = split; rsplit = s_split; dr = s_d; }
            else { ll = s_end; rr = r; lb = sb; rb = box; lsplit = s_split; rsplit = split; dl = s_d; }
            if (rr - ll >= 8) {
                write_child(nodes, 2u * p, ll, p, lb, lsplit, leaf0);
                write_child(nodes, 2u * p + 1u, p, rr, rb, rsplit, leaf0);
            }
            box = lb;
            box_grow(box, rb);
            l = ll;
            r = rr;
            split = p;
        }
    }
}

int sms() { return sm_count(); }

}  // namespace

namespace sqk {

// Both streaming kernels run eight blocks per SM (two 9 KB tile buffers each;
// the next tile's bulk copy overlaps the current tile's work).
void scene_bounds(const float* tris, uint32_t n, uint32_t mode, uint32_t* box_ord, uint32_t* err, cudaStream_t s)
{
    if (n == 0) return;
    const bool aligned = (reinterpret_cast<uintptr_t>(tris) & 15u) == 0;
    const uint32_t tiles = (n + kTileTris - 1) / kTileTris;
    const uint32_t grid = min(tiles, (uint32_t)sms() * 8u);
    launch_chained(k_scene_bounds, dim3(grid), dim3(256), 0, s, tris, n, mode, box_ord, aligned, err);
}

void morton_codes(const float* tris, uint32_t n, uint32_t mode, const uint32_t* box_ord, uint32_t* keys, uint32_t* vals,
                  uint32_t* hist, uint32_t digit_bits, uint32_t passes, uint32_t* err, cudaStream_t s)
{
    if (n == 0) return;
    const bool aligned = (reinterpret_cast<uintptr_t>(tris) & 15u) == 0;
    const uint32_t tiles = (n + kTileTris - 1) / kTileTris;
    const uint32_t grid = min(tiles, (uint32_t)sms() * 8u);
    if (digit_bits == 8 && passes == 4)
        launch_chained(k_morton<8, 4>, dim3(grid), dim3(256), 0, s, tris, n, mode, box_ord, keys, vals, hist, aligned, err);
    else if (digit_bits == 10 && passes == 3)
        launch_chained(k_morton<10, 3>, dim3(grid), dim3(256), 0, s, tris, n, mode, box_ord, keys, vals, hist, aligned, err);
    else if (digit_bits == 6 && passes == 5)
        launch_chained(k_morton<6, 5>, dim3(grid), dim3(256), 0, s, tris, n, mode, box_ord, keys, vals, hist, aligned, err);
}

void morton_codes64(const float* tris, uint32_t n, const uint32_t* box_ord, uint32_t* lo, uint32_t* hi,
                    uint32_t* vals, uint32_t* hist, cudaStream_t s)
{
    if (n == 0) return;
    const bool aligned = (reinterpret_cast<uintptr_t>(tris) & 15u) == 0;
    const uint32_t tiles = (n + kTileTris - 1) / kTileTris;
    const uint32_t grid = min(tiles, (uint32_t)sms() * 8u);
    k_morton64<<<grid, 256, 0, s>>>(tris, n, box_ord, lo, hi, vals, hist, aligned);
}

void gather_high(const uint32_t* hi, const uint32_t* perm1, uint32_t n, uint32_t* hi1, uint32_t* pos, cudaStream_t s)
{
    if (n == 0) return;
    k_gather_high<<<min((n + 255) / 256, (uint32_t)sms() * 8u), 256, 0, s>>>(hi, perm1, n, hi1, pos);
}

void combine64(const uint32_t* hi_sorted, const uint32_t* perm2, const uint32_t* lo_sorted, const uint32_t* perm1,
               uint32_t n, uint64_t* codes64, uint32_t* perm, cudaStream_t s)
{
    if (n == 0) return;
    k_combine64<<<min((n + 255) / 256, (uint32_t)sms() * 8u), 256, 0, s>>>(hi_sorted, perm2, lo_sorted, perm1, n,
                                                                            codes64, perm);
}

template <class Code, bool SEG>
void climb_launch(const Code* codes, const uint32_t* perm, const float* tris, uint32_t n, sq::Node* nodes,
                  uint32_t* flags, float4* info, uint32_t* surv, uint32_t* surv_count, const uint32_t* off, uint32_t M,
                  uint32_t root0, uint32_t* err, cudaStream_t s)
{
    if (n == 0) return;
    launch_chained(k_lbvh_climb<Code, SEG>, dim3((n + 255) / 256), dim3(256), 0, s, codes, perm, tris, n, nodes, info, surv,
                   surv_count, off, M, root0, err);
    // one thread per open node, all at once: the climbs are chains of round
    // trips, so running them side by side beats a grid-stride loop over fewer
    // threads.  Their count is on the device; a warp of 32 positions leaves
    // about four open nodes (its subtree's two spines), so n / 6 threads plus
    // a block per SM cover them without launching blocks that find nothing
    // to do (the loop is grid-stride, so any count is processed)
    const uint32_t grid = std::min((n + 255u) / 256u, (n / 6u + 255u) / 256u + (uint32_t)sms());
    launch_chained(k_lbvh_global<Code, SEG>, dim3(grid), dim3(256), 0, s, surv, surv_count, n, nodes, flags, info, off,
                   M, root0, err);
}

void lbvh_climb(const uint32_t* codes, const uint32_t* perm, const float* tris, uint32_t n, sq::Node* nodes,
                uint32_t* flags, float4* info, uint32_t* surv, uint32_t* surv_count, uint32_t* err, cudaStream_t s)
{
    climb_launch<uint32_t, false>(codes, perm, tris, n, nodes, flags, info, surv, surv_count, nullptr, 1u, 0u, err, s);
}

void lbvh_climb_seg(const uint32_t* codes, const uint32_t* perm, const float* tris, uint32_t n, const uint32_t* off,
                    uint32_t M, uint32_t root0, sq::Node* nodes, uint32_t* flags, float4* info, uint32_t* surv,
                    uint32_t* surv_count, uint32_t* err, cudaStream_t s)
{
    climb_launch<uint32_t, true>(codes, perm, tris, n, nodes, flags, info, surv, surv_count, off, M, root0, err, s);
}

void lbvh_climb64(const uint64_t* codes, const uint32_t* perm, const float* tris, uint32_t n, sq::Node* nodes,
                  uint32_t* flags, float4* info, uint32_t* surv, uint32_t* surv_count, uint32_t* err, cudaStream_t s)
{
    climb_launch<uint64_t, false>(codes, perm, tris, n, nodes, flags, info, surv, surv_count, nullptr, 1u, 0u, err, s);
}

}  // namespace sqk
