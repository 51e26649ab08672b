// sq_sah.cu -- binned SAH and grid BVH builders on the GPU.
//
// Same logical tree as the reference's binned SAH build (recurse /
// recurse_omp / build_hierarchy, src/builder.cpp:1053-1156, 1365-1477,
// 1576-1618) and grid build (src/builder.cpp:1665-1753, 2133-2194), with the
// bin count and leaf size as parameters:
//   leaf        count <= leaf_size, or centroid box area <= 0
//   axis        choose_axis (src/builder.cpp:334-345)
//   bins        bin = int(k1 * (c[axis] - cmin)), k1 = bins*(1-2^-23)/extent
//               (src/builder.cpp:372-398)
//   plane       left-to-right unions, right-to-left sweep, score
//               sa(L)*nL + sa(R)*nR, strict <, ties to the higher plane
//               (src/builder.cpp:488-523)
//   partition   bin <= plane goes left.  The reference swaps in place
//               (src/builder.cpp:599-628); this builder partitions stably.
//               Both yield the same two sets, so the same tree.
//   children    their primitive and centroid boxes come from the bins.
// Records are written in the range-tree layout (oracle/sq_oracle.c), so the
// result is record-for-record the oracle's.
//
// Schedule:
//   large nodes (> kSmall triangles): level by level.  Chunks of 256 or
//     2048 triangles (by mesh size) bin into per-warp shared bins (shared-memory atomics on
//     order-preserving integer encodings, or full-warp reductions when a
//     warp's 32 triangles share one bin), then one atomic per bin value and
//     block; one warp per node sweeps the planes; a count / scan / scatter
//     triple partitions stably into the other id buffer.
//   small nodes: one warp per subtree, smaller child first (stack depth
//     O(log n)), binning and partitioning with warp intrinsics only.
#include "sq_common.cuh"

#include <utility>

namespace {

using namespace sq;

// Triangles per chunk of a large level: 2048 from 1M triangles up, 256 below
// (a small mesh then still spreads a level over many blocks; each thread
// handles one triangle of a chunk instead of eight dependent ones).
constexpr uint32_t kChunk = 2048;
constexpr uint32_t kChunkSmall = 256;
constexpr uint32_t kChunkSmallBelow = 1u << 20;
constexpr uint32_t kSmall = 128;
constexpr int kMaxBins = 32;
constexpr int kBinWords = 13;  // -pmin xyz, pmax xyz, -cmin xyz, cmax xyz (ordered ints), count
constexpr int kStackDepth = 24;
// Large-phase levels of the batched build (device-side counts, no host
// round trip): deeper work is finished by the small phase.
constexpr uint32_t kBatchLargeLevels = 24;
// Large-phase levels a single build queues between two host reads of the
// task count (even, so the count read is always the next level's).
constexpr uint32_t kSahLevelsPerCheck = 4;

struct __align__(16) Task {
    uint32_t begin, count, slot, flags;  // flags: bit0 = ids live in buffer B, bit1 = root-like record
    float pmn[3], pmx[3], cmn[3], cmx[3];
};
static_assert(sizeof(Task) == 64, "Task is 64 bytes");

struct LeafRange {
    uint32_t begin, count, slot, flags;
    float pmn[3], pmx[3];
    uint32_t pad[2];
};
static_assert(sizeof(LeafRange) == 48, "LeafRange is 48 bytes");

struct Split {
    int plane;   // -1: no split (leaf)
    int axis;
    float k1, cmin;
    uint32_t nl;
    uint32_t pad[3];
};

// Task counts.  n_large[l & 1] holds the large tasks of level l: level l
// reads it and appends its large children to n_large[(l + 1) & 1], which
// the level's prep kernel clears first; the kernels read the counts on the
// device, so a level needs no host round trip.
struct Ctl {
    uint32_t n_large[2], n_small, n_leaf;
    uint32_t small_pop, err_bits, big_pop, pad;  // pop counters of the staged and the unstaged small kernels
};
static_assert(sizeof(Ctl) == 32, "Ctl is 32 bytes");

__device__ __forceinline__ float box_sa(const float* mn, const float* mx)
{
    const float lx = mx[0] - mn[0], ly = mx[1] - mn[1], lz = mx[2] - mn[2];
    const float xy = lx * ly, xz = lx * lz, yz = ly * lz;
    float s = xy + xz;
    s = s + yz;
    return s * 2.0f;
}

__device__ __forceinline__ int choose_axis(const float* mn, const float* mx)
{
    const float lx = mx[0] - mn[0], ly = mx[1] - mn[1], lz = mx[2] - mn[2];
    int r = 0;
    r += 2 * (lz > lx && lz > ly);
    r += 1 * (ly > lx && ly >= lz);
    return r;
}

__device__ __forceinline__ float bin_k1(int nb, float ext)
{
    const float eps = 1.1920929e-7f;
    const float one_minus = 1.0f - eps;
    const float num = (float)nb * one_minus;
    return num / ext;
}

__device__ __forceinline__ int bin_of(float k1, float c, float cmin, int nb)
{
    const float d = c - cmin;
    const float x = k1 * d;
    int b = (x == x) ? (int)x : 0;  // cvt.rzi saturates; NaN -> 0
    b = b < 0 ? 0 : b;
    return b > nb - 1 ? nb - 1 : b;
}

__device__ __forceinline__ void load_box(const float4* __restrict__ tb, uint32_t id, float* mn, float* mx)
{
    const float4 a = __ldg(tb + 2ull * id), b = __ldg(tb + 2ull * id + 1);
    mn[0] = a.x; mn[1] = a.y; mn[2] = a.z;
    mx[0] = b.x; mx[1] = b.y; mx[2] = b.z;
}

__device__ __forceinline__ float sel(const float* v, int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); }

// ---------------------------------------------------------------------------
// setup: triangle boxes, identity ids, root boxes

__global__ void __launch_bounds__(256) k_sah_setup(const float* __restrict__ tris, uint32_t n, float4* __restrict__ tb,
                                                   uint32_t* __restrict__ ids, uint32_t* __restrict__ root_ord)
{
    float v[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) v[k] = -FLT_MAX;  // max of (-pmin, pmax, -cmin, cmax)
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float t[9];
        load_tri(tris, i, t);
        const Box b = tri_box(t);
        tb[2ull * i] = make_float4(b.mn[0], b.mn[1], b.mn[2], 0.0f);
        tb[2ull * i + 1] = make_float4(b.mx[0], b.mx[1], b.mx[2], 0.0f);
        ids[i] = i;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float c = (b.mn[k] + b.mx[k]) * 0.5f;
            v[k] = fmaxf(v[k], -b.mn[k]);
            v[3 + k] = fmaxf(v[3 + k], b.mx[k]);
            v[6 + k] = fmaxf(v[6 + k], -c);
            v[9 + k] = fmaxf(v[9 + k], c);
        }
    }
#pragma unroll
    for (int k = 0; k < 12; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = fmaxf(v[k], __shfl_xor_sync(0xFFFFFFFFu, v[k], o));
    }
    __shared__ float s[8][12];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 12; ++k) s[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 12) {
        float m = s[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, s[w][threadIdx.x]);
        atomicMax(root_ord + threadIdx.x, float_to_ordered(m));
    }
}

__device__ __forceinline__ float dec_neg(uint32_t u) { return -ordered_to_float(u); }
__device__ __forceinline__ float dec_pos(uint32_t u) { return ordered_to_float(u); }

// Place a task: leaf (recorded in the leaf list), large (appended to
// large_next, counted in *large_cnt), or small.
__device__ void classify(const Task& t, uint32_t leaf_size, Task* __restrict__ large_next, uint32_t* large_cnt,
                         Task* __restrict__ small, LeafRange* __restrict__ leaves, Ctl* ctl)
{
    const bool leaf = t.count <= leaf_size || !(box_sa(t.cmn, t.cmx) > 0.0f);
    if (leaf) {
        const uint32_t k = atomicAdd(&ctl->n_leaf, 1u);
        LeafRange lr;
        lr.begin = t.begin; lr.count = t.count; lr.slot = t.slot; lr.flags = t.flags;
        for (int a = 0; a < 3; ++a) { lr.pmn[a] = t.pmn[a]; lr.pmx[a] = t.pmx[a]; }
        lr.pad[0] = lr.pad[1] = 0;
        leaves[k] = lr;
    } else if (t.count > kSmall) {
        large_next[atomicAdd(large_cnt, 1u)] = t;
    } else {
        small[atomicAdd(&ctl->n_small, 1u)] = t;
    }
}

__global__ void k_root_task(const uint32_t* __restrict__ root_ord, uint32_t n, uint32_t leaf_size, Task* large,
                            Task* small, LeafRange* leaves, Ctl* ctl, float* scene_out)
{
    Task t;
    t.begin = 0; t.count = n; t.slot = 0; t.flags = 2u;
    for (int k = 0; k < 3; ++k) {
        t.pmn[k] = dec_neg(root_ord[k]);
        t.pmx[k] = dec_pos(root_ord[3 + k]);
        t.cmn[k] = dec_neg(root_ord[6 + k]);
        t.cmx[k] = dec_pos(root_ord[9 + k]);
        scene_out[k] = t.pmn[k];
        scene_out[3 + k] = t.pmx[k];
    }
    classify(t, leaf_size, large, &ctl->n_large[0], small, leaves, ctl);
}

// ---------------------------------------------------------------------------
// grid: cells, Morton order, cell tasks

// Morton slot of grid cell (x, y, z) in a 4x4x4 grid: bits x0 y0 z0 x1 y1 z1
// (the inverse of compact_1_by_2, src/builder.cpp:27-35, 1726-1728).
__device__ __forceinline__ uint32_t cell_slot(uint32_t x, uint32_t y, uint32_t z)
{
    return (x & 1u) | ((y & 1u) << 1) | ((z & 1u) << 2) | ((x & 2u) << 2) | ((y & 2u) << 3) | ((z & 2u) << 4);
}

__global__ void __launch_bounds__(256) k_grid_bin(const float4* __restrict__ tb, uint32_t n,
                                                  const uint32_t* __restrict__ root_ord, uint32_t* __restrict__ keys,
                                                  uint32_t* __restrict__ cell_ord, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t s_cell[64 * kBinWords];
    for (int j = threadIdx.x; j < 64 * kBinWords; j += blockDim.x) s_cell[j] = 0;
    __syncthreads();
    float cmn[3], k1[3];
    for (int a = 0; a < 3; ++a) {
        cmn[a] = dec_neg(root_ord[6 + a]);
        const float cmx = dec_pos(root_ord[9 + a]);
        k1[a] = bin_k1(4, cmx - cmn[a]);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float mn[3], mx[3], c[3];
        load_box(tb, i, mn, mx);
        uint32_t g[3];
        for (int a = 0; a < 3; ++a) {
            c[a] = (mn[a] + mx[a]) * 0.5f;
            g[a] = (uint32_t)bin_of(k1[a], c[a], cmn[a], 4);
        }
        const uint32_t m = cell_slot(g[0], g[1], g[2]);
        keys[i] = m;
        uint32_t* cb = s_cell + m * kBinWords;
        for (int a = 0; a < 3; ++a) {
            atomicMax(cb + a, float_to_ordered(-mn[a]));
            atomicMax(cb + 3 + a, float_to_ordered(mx[a]));
            atomicMax(cb + 6 + a, float_to_ordered(-c[a]));
            atomicMax(cb + 9 + a, float_to_ordered(c[a]));
        }
        atomicAdd(cb + 12, 1u);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < 64 * kBinWords; j += blockDim.x) {
        const uint32_t v = s_cell[j];
        if ((j % kBinWords) == 12) {
            if (v) { atomicAdd(cell_ord + j, v); atomicAdd(hist + j / kBinWords, v); }
        } else if (v) {
            atomicMax(cell_ord + j, v);
        }
    }
}

__global__ void k_grid_tasks(const uint32_t* __restrict__ cell_ord, const uint32_t* __restrict__ root_ord, uint32_t n,
                             uint32_t leaf_size, uint32_t scene_box_cells, Task* large, Task* small,
                             LeafRange* leaves, Ctl* ctl, float* scene_out)
{
    // one thread per cell, in Morton order; cell m covers [begin_m, begin_m + count_m)
    __shared__ uint32_t s_begin[65];
    const uint32_t m = threadIdx.x;
    if (m == 0) {
        uint32_t sum = 0;
        for (int j = 0; j < 64; ++j) { s_begin[j] = sum; sum += cell_ord[j * kBinWords + 12]; }
        s_begin[64] = sum;
        for (int k = 0; k < 3; ++k) { scene_out[k] = dec_neg(root_ord[k]); scene_out[3 + k] = dec_pos(root_ord[3 + k]); }
    }
    __syncthreads();
    if (m >= 64) return;
    const uint32_t* cb = cell_ord + m * kBinWords;
    Task t;
    t.begin = s_begin[m];
    t.count = cb[12];
    t.slot = 63u + m;
    t.flags = 2u;
    for (int k = 0; k < 3; ++k) {
        if (t.count) {
            t.pmn[k] = dec_neg(cb[k]); t.pmx[k] = dec_pos(cb[3 + k]);
            t.cmn[k] = dec_neg(cb[6 + k]); t.cmx[k] = dec_pos(cb[9 + k]);
        } else {
            t.pmn[k] = FLT_MAX; t.pmx[k] = -FLT_MAX; t.cmn[k] = FLT_MAX; t.cmx[k] = -FLT_MAX;
        }
    }
    if (scene_box_cells) {
        // the plain grid builder gives every cell node the scene box (src/builder.cpp:2173-2174)
        for (int k = 0; k < 3; ++k) { t.pmn[k] = dec_neg(root_ord[k]); t.pmx[k] = dec_pos(root_ord[3 + k]); }
    }
    classify(t, leaf_size, large, &ctl->n_large[0], small, leaves, ctl);
}

// heap of 63 inner nodes above the 64 cell nodes (src/builder.cpp:2181-2188)
__global__ void k_grid_heap(Node* __restrict__ nodes)
{
    if (threadIdx.x != 0) return;
    for (int i = 62; i >= 0; --i) {
        const Node a = nodes[2 * i + 1], b = nodes[2 * i + 2];
        Box u;
        u.mn[0] = ref_min(a.mnx, b.mnx); u.mn[1] = ref_min(a.mny, b.mny); u.mn[2] = ref_min(a.mnz, b.mnz);
        u.mx[0] = ref_max(a.mxx, b.mxx); u.mx[1] = ref_max(a.mxy, b.mxy); u.mx[2] = ref_max(a.mxz, b.mxz);
        store_node(nodes + i, u, 2u * i + 1u, 2u, 0);
    }
}

// ---------------------------------------------------------------------------
// warp-level binning and plane choice

// Merge one element per lane (bin = nb for inactive lanes) into warp bins.
__device__ __forceinline__ void warp_bin_add(uint32_t* __restrict__ wb, int bin, int nb, const float* mn, const float* mx,
                                             const float* c)
{
    const int lane = threadIdx.x & 31;
    uint32_t e[12];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        e[a] = float_to_ordered(-mn[a]);
        e[3 + a] = float_to_ordered(mx[a]);
        e[6 + a] = float_to_ordered(-c[a]);
        e[9 + a] = float_to_ordered(c[a]);
    }
    const int b0 = __shfl_sync(0xFFFFFFFFu, bin, 0);
    if (__all_sync(0xFFFFFFFFu, bin == b0)) {
        // the whole warp in one bin: full-warp reductions and one writer
        if (b0 < nb) {
#pragma unroll
            for (int k = 0; k < 12; ++k) e[k] = __reduce_max_sync(0xFFFFFFFFu, e[k]);
            if (lane == 0) {
                uint32_t* b = wb + b0 * kBinWords;
#pragma unroll
                for (int k = 0; k < 12; ++k) b[k] = max(b[k], e[k]);
                b[12] += 32u;
            }
        }
    } else if (bin < nb) {
        // lanes spread over bins: shared-memory atomics per lane (reductions
        // with per-bin masks would run once per distinct bin)
        uint32_t* b = wb + bin * kBinWords;
#pragma unroll
        for (int k = 0; k < 12; ++k) atomicMax(b + k, e[k]);
        atomicAdd(b + 12, 1u);
    }
    __syncwarp();
}

struct PlaneResult {
    int plane;  // -1 if none
    uint32_t nl;
    float lp[6], rp[6], lc[6], rc[6];  // min xyz, max xyz
};

// choose_plane (src/builder.cpp:488-523) over nb bins held as encoded words
// (one bin per lane); every lane returns the result.
__device__ PlaneResult warp_choose_plane(const uint32_t* __restrict__ bins, int nb)
{
    const int lane = threadIdx.x & 31;
    float p[6], c[6];
    uint32_t cnt = 0;
    if (lane < nb) {
        const uint32_t* b = bins + lane * kBinWords;
        cnt = b[12];
        if (cnt) {
            for (int a = 0; a < 3; ++a) {
                p[a] = dec_neg(b[a]); p[3 + a] = dec_pos(b[3 + a]);
                c[a] = dec_neg(b[6 + a]); c[3 + a] = dec_pos(b[9 + a]);
            }
        }
    }
    if (lane >= nb || !cnt) {
        for (int a = 0; a < 3; ++a) { p[a] = FLT_MAX; p[3 + a] = -FLT_MAX; c[a] = FLT_MAX; c[3 + a] = -FLT_MAX; }
    }
    // inclusive prefix (l2r) and suffix unions
    float lp[6], lc[6], sp[6], sc[6];
    uint32_t lcnt = cnt, scnt = cnt;
    for (int k = 0; k < 6; ++k) { lp[k] = p[k]; lc[k] = c[k]; sp[k] = p[k]; sc[k] = c[k]; }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float yp[6], yc[6], zp[6], zc[6];
        for (int k = 0; k < 6; ++k) {
            yp[k] = __shfl_up_sync(0xFFFFFFFFu, lp[k], o);
            yc[k] = __shfl_up_sync(0xFFFFFFFFu, lc[k], o);
            zp[k] = __shfl_down_sync(0xFFFFFFFFu, sp[k], o);
            zc[k] = __shfl_down_sync(0xFFFFFFFFu, sc[k], o);
        }
        const uint32_t ycnt = __shfl_up_sync(0xFFFFFFFFu, lcnt, o);
        const uint32_t zcnt = __shfl_down_sync(0xFFFFFFFFu, scnt, o);
        if (lane >= o) {
            for (int k = 0; k < 3; ++k) {
                lp[k] = fminf(lp[k], yp[k]); lp[3 + k] = fmaxf(lp[3 + k], yp[3 + k]);
                lc[k] = fminf(lc[k], yc[k]); lc[3 + k] = fmaxf(lc[3 + k], yc[3 + k]);
            }
            lcnt += ycnt;
        }
        if (lane + o < 32) {
            for (int k = 0; k < 3; ++k) {
                sp[k] = fminf(sp[k], zp[k]); sp[3 + k] = fmaxf(sp[3 + k], zp[3 + k]);
                sc[k] = fminf(sc[k], zc[k]); sc[3 + k] = fmaxf(sc[3 + k], zc[3 + k]);
            }
            scnt += zcnt;
        }
    }
    // right side of plane i = suffix(i + 1)
    float rp[6], rc[6];
    for (int k = 0; k < 6; ++k) {
        rp[k] = __shfl_down_sync(0xFFFFFFFFu, sp[k], 1);
        rc[k] = __shfl_down_sync(0xFFFFFFFFu, sc[k], 1);
    }
    const uint32_t rcnt = __shfl_down_sync(0xFFFFFFFFu, scnt, 1);
    bool valid = false;
    float score = 0.0f;
    if (lane <= nb - 2) {
        const float sl = box_sa(lp, lp + 3) * (float)lcnt;
        const float sr = box_sa(rp, rp + 3) * (float)rcnt;
        score = sl + sr;
        valid = score < FLT_MAX;
    }
    // best: smallest score, ties to the highest plane
    int best = valid ? lane : -1;
    float bs = score;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int ob = __shfl_xor_sync(0xFFFFFFFFu, best, o);
        const float os = __shfl_xor_sync(0xFFFFFFFFu, bs, o);
        if (ob >= 0 && (best < 0 || os < bs || (os == bs && ob > best))) { best = ob; bs = os; }
    }
    PlaneResult r;
    r.plane = best;
    r.nl = 0;
    if (best >= 0) {
        r.nl = __shfl_sync(0xFFFFFFFFu, lcnt, best);
        for (int k = 0; k < 6; ++k) {
            r.lp[k] = __shfl_sync(0xFFFFFFFFu, lp[k], best);
            r.lc[k] = __shfl_sync(0xFFFFFFFFu, lc[k], best);
            r.rp[k] = __shfl_sync(0xFFFFFFFFu, rp[k], best);
            r.rc[k] = __shfl_sync(0xFFFFFFFFu, rc[k], best);
        }
    }
    return r;
}

__device__ __forceinline__ Task child_task(uint32_t begin, uint32_t count, uint32_t slot, uint32_t buf, const float* p,
                                           const float* c)
{
    Task t;
    t.begin = begin; t.count = count; t.slot = slot; t.flags = buf;
    for (int k = 0; k < 3; ++k) { t.pmn[k] = p[k]; t.pmx[k] = p[3 + k]; t.cmn[k] = c[k]; t.cmx[k] = c[3 + k]; }
    return t;
}

// ---------------------------------------------------------------------------
// large phase
//
// Every kernel reads the level's task count *ntp on the device and loops
// over its work (chunks per block, tasks per warp), so the same kernels run
// with an exact grid when the host knows the count and with a fixed grid in
// the graph-captured batch build, where it does not.

__global__ void k_large_zero(uint32_t* __restrict__ bins, const uint32_t* __restrict__ ntp, int nb)
{
    chain_wait();  // a chained launch (enqueue_level_chunks)
    chain_release();
    const size_t per = (size_t)nb * kBinWords;
    const size_t words = (size_t)(*ntp) * per;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        bins[(i / per) * (kMaxBins * kBinWords) + i % per] = 0;
}

template <uint32_t CHUNK>
__global__ void k_large_prep(const Task* __restrict__ tasks, const uint32_t* __restrict__ ntp, uint32_t* next_cnt,
                             int nb, Split* __restrict__ split, uint32_t* __restrict__ chunk_start)
{
    chain_wait();  // a chained launch (enqueue_level_chunks)
    chain_release();
    // single block: chunk counts and their exclusive scan
    __shared__ uint32_t s_sum[1024];
    const uint32_t nt = *ntp;
    if (threadIdx.x == 0) *next_cnt = 0;  // this level's large children are counted from 0
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nt; base += blockDim.x) {
        const uint32_t t = base + threadIdx.x;
        uint32_t ch = 0;
        if (t < nt) {
            const Task& tk = tasks[t];
            ch = (tk.count + CHUNK - 1) / CHUNK;
            Split s;
            s.axis = choose_axis(tk.cmn, tk.cmx);
            s.cmin = sel(tk.cmn, s.axis);
            s.k1 = bin_k1(nb, sel(tk.cmx, s.axis) - s.cmin);
            s.plane = -1;
            s.nl = 0;
            s.pad[0] = s.pad[1] = s.pad[2] = 0;
            split[t] = s;
        }
        s_sum[threadIdx.x] = ch;
        __syncthreads();
        for (uint32_t o = 1; o < blockDim.x; o <<= 1) {
            const uint32_t v = threadIdx.x >= o ? s_sum[threadIdx.x - o] : 0u;
            __syncthreads();
            s_sum[threadIdx.x] += v;
            __syncthreads();
        }
        if (t < nt) chunk_start[t] = carry + s_sum[threadIdx.x] - ch;
        carry += s_sum[blockDim.x - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) chunk_start[nt] = carry;
}

__device__ __forceinline__ uint32_t task_of_chunk(const uint32_t* __restrict__ chunk_start, uint32_t nt, uint32_t c)
{
    uint32_t lo = 0, hi = nt;  // largest t with chunk_start[t] <= c
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(chunk_start + mid) <= c) lo = mid; else hi = mid;
    }
    return lo;
}

template <uint32_t CHUNK>
__global__ void __launch_bounds__(256) k_large_bin(const Task* __restrict__ tasks, const uint32_t* __restrict__ ntp,
                                                   const Split* __restrict__ split, const uint32_t* __restrict__ chunk_start,
                                                   const uint32_t* __restrict__ ids_a, const uint32_t* __restrict__ ids_b,
                                                   const float4* __restrict__ tb, int nb, uint32_t* __restrict__ bins_g)
{
    chain_wait();  // a chained launch (enqueue_level_chunks)
    chain_release();
    __shared__ uint32_t s_wb[8][kMaxBins * kBinWords];
    const uint32_t nt = *ntp;
    const uint32_t chunks = chunk_start[nt];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* wb = s_wb[warp];
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const uint32_t t = task_of_chunk(chunk_start, nt, c);
        const Task tk = tasks[t];
        const Split sp = split[t];
        const uint32_t off = (c - chunk_start[t]) * CHUNK;
        const uint32_t len = min(CHUNK, tk.count - off);
        const uint32_t* ids = (tk.flags & 1u) ? ids_b : ids_a;
        for (int j = lane; j < kMaxBins * kBinWords; j += 32) wb[j] = 0;
        __syncwarp();
        for (uint32_t base = warp * 32; base < len; base += 256) {
            const uint32_t j = base + lane;
            float mn[3], mx[3], cc[3];
            int bin = nb;
            if (j < len) {
                load_box(tb, ids[tk.begin + off + j], mn, mx);
                for (int a = 0; a < 3; ++a) cc[a] = (mn[a] + mx[a]) * 0.5f;
                bin = bin_of(sp.k1, sel(cc, sp.axis), sp.cmin, nb);
            } else {
                for (int a = 0; a < 3; ++a) { mn[a] = mx[a] = cc[a] = 0.0f; }
            }
            warp_bin_add(wb, bin, nb, mn, mx, cc);
        }
        __syncthreads();
        uint32_t* g = bins_g + (size_t)t * kMaxBins * kBinWords;
        for (int j = threadIdx.x; j < nb * kBinWords; j += blockDim.x) {
            uint32_t v = s_wb[0][j];
            const bool is_count = (j % kBinWords) == 12;
            for (int w = 1; w < 8; ++w) v = is_count ? v + s_wb[w][j] : max(v, s_wb[w][j]);
            if (v) {
                if (is_count) atomicAdd(g + j, v); else atomicMax(g + j, v);
            }
        }
        __syncthreads();  // every warp's bins read before the next chunk clears them
    }
}

__global__ void k_large_split(const Task* __restrict__ tasks, const uint32_t* __restrict__ ntp, Split* __restrict__ split,
                              const uint32_t* __restrict__ bins_g, int nb, uint32_t base, uint32_t leaf_size,
                              Node* __restrict__ nodes, Task* large_next, uint32_t* next_cnt, Task* small,
                              LeafRange* leaves, Ctl* ctl)
{
    chain_wait();  // a chained launch (enqueue_level_chunks)
    chain_release();
    const uint32_t nt = *ntp;
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += warps) {
        const Task tk = tasks[t];
        const PlaneResult r = warp_choose_plane(bins_g + (size_t)t * kMaxBins * kBinWords, nb);
        if (lane != 0) continue;
        if (r.plane < 0 || r.nl == 0 || r.nl == tk.count) {
            // no plane scored below FLT_MAX: the node becomes a leaf
            const uint32_t k = atomicAdd(&ctl->n_leaf, 1u);
            LeafRange lr;
            lr.begin = tk.begin; lr.count = tk.count; lr.slot = tk.slot; lr.flags = tk.flags;
            for (int a = 0; a < 3; ++a) { lr.pmn[a] = tk.pmn[a]; lr.pmx[a] = tk.pmx[a]; }
            lr.pad[0] = lr.pad[1] = 0;
            leaves[k] = lr;
            continue;
        }
        Split s = split[t];
        s.plane = r.plane;
        s.nl = r.nl;
        split[t] = s;
        const uint32_t q = tk.begin + r.nl;
        Box pb;
        for (int a = 0; a < 3; ++a) { pb.mn[a] = tk.pmn[a]; pb.mx[a] = tk.pmx[a]; }
        store_node(nodes + tk.slot, pb, base + 2u * q, 2u, 0);
        const uint32_t buf = (tk.flags & 1u) ^ 1u;
        classify(child_task(tk.begin, r.nl, base + 2u * q, buf, r.lp, r.lc), leaf_size, large_next, next_cnt, small,
                 leaves, ctl);
        classify(child_task(q, tk.count - r.nl, base + 2u * q + 1u, buf, r.rp, r.rc), leaf_size, large_next, next_cnt,
                 small, leaves, ctl);
    }
}

template <uint32_t CHUNK>
__global__ void __launch_bounds__(256) k_large_count(const Task* __restrict__ tasks, const uint32_t* __restrict__ ntp,
                                                     const Split* __restrict__ split,
                                                     const uint32_t* __restrict__ chunk_start,
                                                     const uint32_t* __restrict__ ids_a, const uint32_t* __restrict__ ids_b,
                                                     const float4* __restrict__ tb, int nb,
                                                     uint32_t* __restrict__ chunk_left)
{
    chain_wait();  // a chained launch (enqueue_level_chunks)
    chain_release();
    __shared__ uint32_t s[8];
    const uint32_t nt = *ntp;
    const uint32_t chunks = chunk_start[nt];
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const uint32_t t = task_of_chunk(chunk_start, nt, c);
        const Split sp = split[t];
        if (sp.plane < 0) continue;  // block-uniform
        const Task tk = tasks[t];
        const uint32_t off = (c - chunk_start[t]) * CHUNK;
        const uint32_t len = min(CHUNK, tk.count - off);
        const uint32_t* ids = (tk.flags & 1u) ? ids_b : ids_a;
        uint32_t cnt = 0;
        for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) {
            float mn[3], mx[3];
            load_box(tb, ids[tk.begin + off + j], mn, mx);
            const float cc = (sel(mn, sp.axis) + sel(mx, sp.axis)) * 0.5f;
            cnt += bin_of(sp.k1, cc, sp.cmin, nb) <= sp.plane;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, o);
        if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t total = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += s[w];
            chunk_left[c] = total;
        }
        __syncthreads();
    }
}

// exclusive scan of the left counts over each task's chunks (one warp per task)
__global__ void k_large_scan(const Split* __restrict__ split, const uint32_t* __restrict__ ntp,
                             const uint32_t* __restrict__ chunk_start, uint32_t* __restrict__ chunk_left)
{
    chain_wait();  // a chained launch (enqueue_level_chunks)
    chain_release();
    const uint32_t nt = *ntp;
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += warps) {
        if (split[t].plane < 0) continue;  // warp-uniform
        uint32_t carry = 0;
        for (uint32_t c0 = chunk_start[t]; c0 < chunk_start[t + 1]; c0 += 32) {
            const uint32_t c = c0 + lane;
            const uint32_t v = c < chunk_start[t + 1] ? chunk_left[c] : 0u;
            uint32_t x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                if (lane >= o) x += y;
            }
            if (c < chunk_start[t + 1]) chunk_left[c] = carry + x - v;
            carry += __shfl_sync(0xFFFFFFFFu, x, 31);
        }
    }
}

template <uint32_t CHUNK>
__global__ void __launch_bounds__(256) k_large_scatter(const Task* __restrict__ tasks, const uint32_t* __restrict__ ntp,
                                                       const Split* __restrict__ split,
                                                       const uint32_t* __restrict__ chunk_start,
                                                       uint32_t* __restrict__ ids_a, uint32_t* __restrict__ ids_b,
                                                       const float4* __restrict__ tb, int nb,
                                                       const uint32_t* __restrict__ chunk_left)
{
    chain_wait();  // a chained launch (enqueue_level_chunks)
    chain_release();
    constexpr int kPer = CHUNK / 256;  // consecutive elements per thread
    __shared__ uint32_t s_w[8];
    const uint32_t nt = *ntp;
    const uint32_t chunks = chunk_start[nt];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const uint32_t t = task_of_chunk(chunk_start, nt, c);
        const Split sp = split[t];
        if (sp.plane < 0) continue;  // block-uniform
        const Task tk = tasks[t];
        const uint32_t off = (c - chunk_start[t]) * CHUNK;
        const uint32_t len = min(CHUNK, tk.count - off);
        const uint32_t* in = (tk.flags & 1u) ? ids_b : ids_a;
        uint32_t* out = (tk.flags & 1u) ? ids_a : ids_b;
        uint32_t idv[kPer];
        bool left[kPer];
        uint32_t cnt = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const uint32_t j = threadIdx.x * kPer + k;
            left[k] = false;
            idv[k] = 0;
            if (j < len) {
                idv[k] = in[tk.begin + off + j];
                float mn[3], mx[3];
                load_box(tb, idv[k], mn, mx);
                const float cc = (sel(mn, sp.axis) + sel(mx, sp.axis)) * 0.5f;
                left[k] = bin_of(sp.k1, cc, sp.cmin, nb) <= sp.plane;
                cnt += left[k];
            }
        }
        // block exclusive scan of per-thread left counts
        uint32_t x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[warp] = x;
        __syncthreads();
        uint32_t wsum = 0;
        for (int w = 0; w < warp; ++w) wsum += s_w[w];
        uint32_t lrank = wsum + x - cnt;                    // left elements before this thread in the chunk
        const uint32_t left_before = chunk_left[c];          // left elements before this chunk in the task
        const uint32_t lbase = tk.begin + left_before;
        const uint32_t rbase = tk.begin + sp.nl + (off - left_before);
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const uint32_t j = threadIdx.x * kPer + k;
            if (j < len) {
                if (left[k]) { out[lbase + lrank] = idv[k]; lrank++; }
                else out[rbase + (j - lrank)] = idv[k];
            }
        }
        __syncthreads();  // s_w read by every warp before the next chunk writes it
    }
}

// After the last fixed level of the batch build: large tasks still left go
// to the small phase, whose warps split subtrees of any size.
__global__ void k_large_to_small(const Task* __restrict__ large, const uint32_t* __restrict__ ntp,
                                 Task* __restrict__ small, Ctl* ctl)
{
    const uint32_t nt = *ntp;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x)
        small[atomicAdd(&ctl->n_small, 1u)] = large[t];
}

// ---------------------------------------------------------------------------
// leaves

// Leaf-region records for [b, b+c) and the range's own record at its slot.
__device__ void warp_emit_leaf(const uint32_t* __restrict__ ids, uint32_t b, uint32_t c, uint32_t slot, uint32_t flags,
                               const float* pmn, const float* pmx, const float4* __restrict__ tb, Node* __restrict__ nodes,
                               uint32_t leaf0, uint32_t* err)
{
    const int lane = threadIdx.x & 31;
    for (uint32_t j = lane; j < c; j += 32) {
        const uint32_t id = ids[b + j];
        Box bb;
        load_box(tb, id, bb.mn, bb.mx);
        store_node(nodes + leaf0 + b + j, bb, id, 1u, kLeafFlag);
        if (c == 1 && !(flags & 2u)) store_node(nodes + slot, bb, id, 1u, kLeafFlag);
    }
    if (lane == 0 && (c != 1 || (flags & 2u))) {
        if (c > 65535u) { raise_error(err, SQ_DEVERR_NODE_COUNT); return; }
        Box pb;
        for (int a = 0; a < 3; ++a) { pb.mn[a] = pmn[a]; pb.mx[a] = pmx[a]; }
        store_node(nodes + slot, pb, leaf0 + b, c, 0);
    }
}

__global__ void k_emit_leaves(const LeafRange* __restrict__ leaves, const Ctl* __restrict__ ctl,
                              const uint32_t* __restrict__ ids_a, const uint32_t* __restrict__ ids_b,
                              const float4* __restrict__ tb, Node* __restrict__ nodes, uint32_t leaf0, uint32_t* err)
{
    const uint32_t nl = ctl->n_leaf;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nl; w += (gridDim.x * blockDim.x) >> 5) {
        const LeafRange lr = leaves[w];
        const uint32_t* ids = (lr.flags & 1u) ? ids_b : ids_a;
        warp_emit_leaf(ids, lr.begin, lr.count, lr.slot, lr.flags, lr.pmn, lr.pmx, tb, nodes, leaf0, err);
    }
}

// ---------------------------------------------------------------------------
// small phase: one warp per subtree
//
// A subtree of at most kStage triangles (every small task of a single build:
// a task turns small at kSmall or fewer) is staged once in the warp's shared
// memory -- each triangle's box and id -- and its nodes are binned,
// partitioned and emitted from there: only 16-bit local indices move between
// the two orders (the buffer parity of the global ids, which the staged
// subtree no longer writes), and leaves read their boxes from the stage.  A
// node then costs shared-memory latency instead of two dependent global
// round trips per 32 triangles.  Larger small tasks (leftovers of the
// batched build's fixed large levels) read and write the global buffers.
constexpr uint32_t kStage = 128;

struct SmallStage {
    float4 box[kStage][2];      // min xyz, max xyz of local triangle k
    uint32_t gid[kStage];       // its triangle id
    uint16_t loc[2][kStage];    // local triangles in the order of buffer parity p
};

template <bool STAGED>
__device__ void small_subtree(Task cur, SmallStage& sg, Task* st, uint32_t* wb, uint32_t* __restrict__ ids_a,
                              uint32_t* __restrict__ ids_b, const float4* __restrict__ tb, int nb, uint32_t leaf_size,
                              uint32_t base, Node* __restrict__ nodes, uint32_t leaf0, uint32_t* err)
{
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t root_begin = cur.begin;
    // triangle at position `pos` (global) of the order of parity p
    auto get = [&](uint32_t p, uint32_t pos, uint32_t& id, uint16_t& li, float* mn, float* mx) {
        if (STAGED) {
            li = sg.loc[p][pos - root_begin];
            const float4 a = sg.box[li][0], b = sg.box[li][1];
            mn[0] = a.x; mn[1] = a.y; mn[2] = a.z;
            mx[0] = b.x; mx[1] = b.y; mx[2] = b.z;
            id = sg.gid[li];
        } else {
            li = 0;
            id = (p ? ids_b : ids_a)[pos];
            load_box(tb, id, mn, mx);
        }
    };
    auto put = [&](uint32_t p, uint32_t pos, uint32_t id, uint16_t li) {
        if (STAGED) sg.loc[p][pos - root_begin] = li;
        else (p ? ids_b : ids_a)[pos] = id;
    };
    // leaf records of positions [b, b + c) of parity p (warp_emit_leaf's records)
    auto emit_leaf = [&](uint32_t p, uint32_t b, uint32_t c, uint32_t slot, uint32_t flags, const float* pmn,
                         const float* pmx) {
        for (uint32_t j = lane; j < c; j += 32) {
            uint32_t id;
            uint16_t li;
            Box bb;
            get(p, b + j, id, li, bb.mn, bb.mx);
            store_node(nodes + leaf0 + b + j, bb, id, 1u, kLeafFlag);
            if (c == 1 && !(flags & 2u)) store_node(nodes + slot, bb, id, 1u, kLeafFlag);
        }
        if (lane == 0 && (c != 1 || (flags & 2u))) {
            if (c > 65535u) { raise_error(err, SQ_DEVERR_NODE_COUNT); return; }
            Box pb;
            for (int a = 0; a < 3; ++a) { pb.mn[a] = pmn[a]; pb.mx[a] = pmx[a]; }
            store_node(nodes + slot, pb, leaf0 + b, c, 0);
        }
    };
    if (STAGED) {
        const uint32_t* in0 = (cur.flags & 1u) ? ids_b : ids_a;
        for (uint32_t j = lane; j < cur.count; j += 32) {
            const uint32_t id = in0[cur.begin + j];
            sg.box[j][0] = __ldg(tb + 2ull * id);
            sg.box[j][1] = __ldg(tb + 2ull * id + 1);
            sg.gid[j] = id;
            sg.loc[cur.flags & 1u][j] = (uint16_t)j;
        }
        __syncwarp();
    }
    int sp = 0;
    for (;;) {
        // cur is splittable (count > leaf_size, centroid area > 0)
        const uint32_t pin = cur.flags & 1u, pout = pin ^ 1u;
        const int axis = choose_axis(cur.cmn, cur.cmx);
        const float cmin = sel(cur.cmn, axis);
        const float k1 = bin_k1(nb, sel(cur.cmx, axis) - cmin);
        for (int j = lane; j < kMaxBins * kBinWords; j += 32) wb[j] = 0;
        __syncwarp();
        for (uint32_t j0 = 0; j0 < cur.count; j0 += 32) {
            const uint32_t j = j0 + lane;
            float mn[3], mx[3], cc[3];
            int bin = nb;
            if (j < cur.count) {
                uint32_t id;
                uint16_t li;
                get(pin, cur.begin + j, id, li, mn, mx);
                for (int a = 0; a < 3; ++a) cc[a] = (mn[a] + mx[a]) * 0.5f;
                bin = bin_of(k1, sel(cc, axis), cmin, nb);
            } else {
                for (int a = 0; a < 3; ++a) { mn[a] = mx[a] = cc[a] = 0.0f; }
            }
            warp_bin_add(wb, bin, nb, mn, mx, cc);
        }
        const PlaneResult r = warp_choose_plane(wb, nb);
        __syncwarp();
        bool have_next = false;
        if (r.plane < 0 || r.nl == 0 || r.nl == cur.count) {
            // no plane scored below FLT_MAX: leaf
            emit_leaf(pin, cur.begin, cur.count, cur.slot, cur.flags, cur.pmn, cur.pmx);
        } else {
            const uint32_t q = cur.begin + r.nl;
            if (lane == 0) {
                Box pb;
                for (int a = 0; a < 3; ++a) { pb.mn[a] = cur.pmn[a]; pb.mx[a] = cur.pmx[a]; }
                store_node(nodes + cur.slot, pb, base + 2u * q, 2u, 0);
            }
            // stable partition into the other order
            uint32_t lc = 0, rc = 0;
            for (uint32_t j0 = 0; j0 < cur.count; j0 += 32) {
                const uint32_t j = j0 + lane;
                const bool valid = j < cur.count;
                uint32_t id = 0;
                uint16_t li = 0;
                bool left = false;
                if (valid) {
                    float mn[3], mx[3];
                    get(pin, cur.begin + j, id, li, mn, mx);
                    const float cc = (sel(mn, axis) + sel(mx, axis)) * 0.5f;
                    left = bin_of(k1, cc, cmin, nb) <= r.plane;
                }
                const uint32_t lb = __ballot_sync(0xFFFFFFFFu, valid && left);
                const uint32_t rb = __ballot_sync(0xFFFFFFFFu, valid && !left);
                if (valid) {
                    if (left) put(pout, cur.begin + lc + __popc(lb & lt), id, li);
                    else put(pout, q + rc + __popc(rb & lt), id, li);
                }
                lc += __popc(lb);
                rc += __popc(rb);
            }
            __syncwarp();
            Task ch[2] = {child_task(cur.begin, r.nl, base + 2u * q, pout, r.lp, r.lc),
                          child_task(q, cur.count - r.nl, base + 2u * q + 1u, pout, r.rp, r.rc)};
            bool split_ch[2];
            for (int k = 0; k < 2; ++k) {
                split_ch[k] = !(ch[k].count <= leaf_size || !(box_sa(ch[k].cmn, ch[k].cmx) > 0.0f));
                if (!split_ch[k]) emit_leaf(pout, ch[k].begin, ch[k].count, ch[k].slot, ch[k].flags, ch[k].pmn, ch[k].pmx);
            }
            if (split_ch[0] && split_ch[1]) {
                const int small_k = ch[0].count <= ch[1].count ? 0 : 1;
                if (sp >= kStackDepth) {
                    raise_error(err, SQ_DEVERR_SAH_QUEUE);
                    return;
                }
                if (lane == 0) st[sp] = ch[1 - small_k];
                sp++;
                __syncwarp();
                cur = ch[small_k];
                have_next = true;
            } else if (split_ch[0] || split_ch[1]) {
                cur = split_ch[0] ? ch[0] : ch[1];
                have_next = true;
            }
        }
        if (!have_next) {
            if (sp == 0) break;
            --sp;
            __syncwarp();
            cur = st[sp];
            __syncwarp();
        }
    }
    __syncwarp();  // the stage is reused by the warp's next subtree
}

// One warp per small task: STAGED takes the tasks of at most kStage
// triangles (all of a single build's), the other kernel the rest (leftovers
// of the batched build's fixed large levels); each kernel pops the shared
// list with its own counter and skips the other's tasks.  Two kernels, so
// the staged one keeps its own, smaller register count.
template <bool STAGED>
__global__ void __launch_bounds__(128) k_small(const Task* __restrict__ small, Ctl* ctl, uint32_t* __restrict__ ids_a,
                                               uint32_t* __restrict__ ids_b, const float4* __restrict__ tb, int nb,
                                               uint32_t leaf_size, uint32_t base, Node* __restrict__ nodes,
                                               uint32_t leaf0, uint32_t* err)
{
    __shared__ uint32_t s_bins[4][kMaxBins * kBinWords];
    __shared__ Task s_stack[4][kStackDepth];
    __shared__ SmallStage s_stage[STAGED ? 4 : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t total = ctl->n_small;
    uint32_t* pop = STAGED ? &ctl->small_pop : &ctl->big_pop;
    for (;;) {
        uint32_t ti = 0;
        if (lane == 0) ti = atomicAdd(pop, 1u);
        ti = __shfl_sync(0xFFFFFFFFu, ti, 0);
        if (ti >= total) return;
        const Task cur = small[ti];
        if ((cur.count <= kStage) != STAGED) continue;  // warp-uniform
        small_subtree<STAGED>(cur, s_stage[STAGED ? warp : 0], s_stack[warp], s_bins[warp], ids_a, ids_b, tb, nb,
                              leaf_size, base, nodes, leaf0, err);
    }
}

int sms() { return sm_count(); }

// Workspace carving shared by the single and the batched build.
struct SahWs {
    float4* tb;
    uint32_t *ids_a, *ids_b;
    Task *lists[2], *small;
    LeafRange* leaves;
    Split* split;
    uint32_t *chunk_start, *chunk_left, *bins, *cells, *hist, *root_ord;
    Ctl* ctl;
};

size_t sah_tasks(uint32_t n) { return n / kSmall + 2; }

size_t sah_ws_bytes(uint32_t n, uint32_t meshes)
{
    const size_t tasks = sah_tasks(n);
    size_t b = 0;
    auto add = [&](size_t bytes) { b += (bytes + 255) / 256 * 256; };
    add(sizeof(float4) * 2ull * n);               // triangle boxes
    add(sizeof(uint32_t) * (size_t)n);            // ids A
    add(sizeof(uint32_t) * (size_t)n);            // ids B
    add(sizeof(Task) * tasks);                    // large lists (two levels)
    add(sizeof(Task) * tasks);
    add(sizeof(Task) * ((size_t)n / 2 + 2));      // small list
    add(sizeof(LeafRange) * ((size_t)n + 66 + meshes));  // leaf list (+64 empty grid cells, + empty meshes)
    add(sizeof(Split) * tasks);
    add(sizeof(uint32_t) * (tasks + 1));          // chunk starts
    add(sizeof(uint32_t) * ((size_t)n / kChunkSmall + tasks + 1));  // chunk left counts
    add(sizeof(uint32_t) * (size_t)kMaxBins * kBinWords * tasks);  // bins
    add(sizeof(uint32_t) * 64 * kBinWords);       // grid cells
    add(sizeof(uint32_t) * 64);                   // grid histogram
    add(sizeof(uint32_t) * 16ull * (meshes ? meshes : 1));  // root boxes (12 words per mesh)
    add(sizeof(Ctl));
    return b;
}

SahWs carve(void* ws, uint32_t n, uint32_t meshes)
{
    const size_t tasks = sah_tasks(n);
    char* p = static_cast<char*>(ws);
    auto take = [&](size_t bytes) { char* r = p; p += (bytes + 255) / 256 * 256; return r; };
    SahWs w;
    w.tb = reinterpret_cast<float4*>(take(sizeof(float4) * 2ull * n));
    w.ids_a = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t)n));
    w.ids_b = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t)n));
    w.lists[0] = reinterpret_cast<Task*>(take(sizeof(Task) * tasks));
    w.lists[1] = reinterpret_cast<Task*>(take(sizeof(Task) * tasks));
    w.small = reinterpret_cast<Task*>(take(sizeof(Task) * ((size_t)n / 2 + 2)));
    w.leaves = reinterpret_cast<LeafRange*>(take(sizeof(LeafRange) * ((size_t)n + 66 + meshes)));
    w.split = reinterpret_cast<Split*>(take(sizeof(Split) * tasks));
    w.chunk_start = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (tasks + 1)));
    w.chunk_left = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * ((size_t)n / kChunkSmall + tasks + 1)));
    w.bins = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t)kMaxBins * kBinWords * tasks));
    w.cells = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * 64 * kBinWords));
    w.hist = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * 64));
    w.root_ord = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * 16ull * (meshes ? meshes : 1)));
    w.ctl = reinterpret_cast<Ctl*>(take(sizeof(Ctl)));
    return w;
}

// One level of the large phase on the tasks in w.lists[level & 1], whose
// count is ctl->n_large[level & 1] on the device.  chunk_grid / task_blocks:
// exact grids when the host knows the count, fixed ones otherwise (the
// kernels loop over whatever the count holds).
template <uint32_t CHUNK>
void enqueue_level_chunks(const SahWs& w, uint32_t level, int nb, uint32_t base, uint32_t leaf_size, Node* nodes,
                          uint32_t chunk_grid, uint32_t task_blocks, cudaStream_t s)
{
    const Task* proc = w.lists[level & 1];
    Task* outl = w.lists[(level + 1) & 1];
    const uint32_t* ntp = &w.ctl->n_large[level & 1];
    uint32_t* next = &w.ctl->n_large[(level + 1) & 1];
    // seven short kernels per level, chained: each may launch while the one
    // before it runs and waits for it on the device (chain_wait)
    launch_chained(k_large_zero, dim3(task_blocks), dim3(256), 0, s, w.bins, ntp, nb);
    launch_chained(k_large_prep<CHUNK>, dim3(1), dim3(1024), 0, s, proc, ntp, next, nb, w.split, w.chunk_start);
    launch_chained(k_large_bin<CHUNK>, dim3(chunk_grid), dim3(256), 0, s, proc, ntp, (const Split*)w.split,
                   (const uint32_t*)w.chunk_start, (const uint32_t*)w.ids_a, (const uint32_t*)w.ids_b,
                   (const float4*)w.tb, nb, w.bins);
    launch_chained(k_large_split, dim3(task_blocks), dim3(128), 0, s, proc, ntp, w.split, (const uint32_t*)w.bins, nb,
                   base, leaf_size, nodes, outl, next, w.small, w.leaves, w.ctl);
    launch_chained(k_large_count<CHUNK>, dim3(chunk_grid), dim3(256), 0, s, proc, ntp, (const Split*)w.split,
                   (const uint32_t*)w.chunk_start, (const uint32_t*)w.ids_a, (const uint32_t*)w.ids_b,
                   (const float4*)w.tb, nb, w.chunk_left);
    launch_chained(k_large_scan, dim3(task_blocks), dim3(128), 0, s, (const Split*)w.split, ntp,
                   (const uint32_t*)w.chunk_start, w.chunk_left);
    launch_chained(k_large_scatter<CHUNK>, dim3(chunk_grid), dim3(256), 0, s, proc, ntp, (const Split*)w.split,
                   (const uint32_t*)w.chunk_start, w.ids_a, w.ids_b, (const float4*)w.tb, nb,
                   (const uint32_t*)w.chunk_left);
}

// one large level of a build over n triangles (chunk size by n)
void enqueue_large_level(const SahWs& w, uint32_t level, int nb, uint32_t base, uint32_t leaf_size, Node* nodes,
                         uint32_t chunk_grid, uint32_t task_blocks, uint32_t n, cudaStream_t s)
{
    if (n < kChunkSmallBelow)
        enqueue_level_chunks<kChunkSmall>(w, level, nb, base, leaf_size, nodes, chunk_grid, task_blocks, s);
    else
        enqueue_level_chunks<kChunk>(w, level, nb, base, leaf_size, nodes, chunk_grid, task_blocks, s);
}

// ---------------------------------------------------------------------------
// batch: many meshes in one build

// Boxes, ids and every mesh's root boxes (order-preserving words, 12 per
// mesh at a stride of 16): triangle i belongs to the mesh m with
// off[m] <= i < off[m + 1]; lanes of one mesh merge through the warp before
// one atomic per word.
__global__ void __launch_bounds__(256) k_sah_setup_seg(const float* __restrict__ tris, uint32_t n,
                                                       const uint32_t* __restrict__ off, uint32_t M,
                                                       float4* __restrict__ tb, uint32_t* __restrict__ ids,
                                                       uint32_t* __restrict__ root_ord)
{
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t m = 0xFFFFFFFFu;
        uint32_t e[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) e[k] = 0u;
        if (valid) {
            uint32_t lo = 0, hi = M;  // largest m with off[m] <= i
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
            }
            m = lo;
            float t[9];
            load_tri(tris, i, t);
            const Box b = tri_box(t);
            tb[2ull * i] = make_float4(b.mn[0], b.mn[1], b.mn[2], 0.0f);
            tb[2ull * i + 1] = make_float4(b.mx[0], b.mx[1], b.mx[2], 0.0f);
            ids[i] = i;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float c = (b.mn[k] + b.mx[k]) * 0.5f;
                e[k] = float_to_ordered(-b.mn[k]);
                e[3 + k] = float_to_ordered(b.mx[k]);
                e[6 + k] = float_to_ordered(-c);
                e[9 + k] = float_to_ordered(c);
            }
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, m);
#pragma unroll
        for (int k = 0; k < 12; ++k) e[k] = __reduce_max_sync(peers, e[k]);
        if (valid && (threadIdx.x & 31) == (uint32_t)(__ffs(peers) - 1))
            for (int k = 0; k < 12; ++k) atomicMax(root_ord + 16ull * m + k, e[k]);
    }
}

// One root task per mesh: triangles [off[m], off[m + 1]), record root0 + m.
__global__ void k_root_tasks_seg(const uint32_t* __restrict__ root_ord, const uint32_t* __restrict__ off, uint32_t M,
                                 uint32_t leaf_size, uint32_t root0, Task* large, Task* small, LeafRange* leaves,
                                 Ctl* ctl)
{
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        Task t;
        t.begin = off[m];
        t.count = off[m + 1] - off[m];
        t.slot = root0 + m;
        t.flags = 2u;
        const uint32_t* ro = root_ord + 16ull * m;
        for (int k = 0; k < 3; ++k) {
            if (t.count) {
                t.pmn[k] = dec_neg(ro[k]);
                t.pmx[k] = dec_pos(ro[3 + k]);
                t.cmn[k] = dec_neg(ro[6 + k]);
                t.cmx[k] = dec_pos(ro[9 + k]);
            } else {
                t.pmn[k] = t.cmn[k] = FLT_MAX;
                t.pmx[k] = t.cmx[k] = -FLT_MAX;
            }
        }
        classify(t, leaf_size, large, &ctl->n_large[0], small, leaves, ctl);
    }
}

}  // namespace

namespace sqk {

size_t sah_workspace_bytes(uint32_t n) { return sah_ws_bytes(n, 0); }
size_t sah_batch_workspace_bytes(uint32_t n, uint32_t meshes) { return sah_ws_bytes(n, meshes); }

// Builds a SAH (grid = 0) or grid (grid = 1) BVH.  ws: workspace of
// sah_workspace_bytes(n) bytes; keys/vals/alt: 4n-word sort buffers (grid
// only); sort_ws: zeroed onesweep state for one 6-bit pass (grid only).
// host_ctl: pinned 32-byte buffer.  Returns 0 or a cudaError_t.
int build_sah(const float* tris, uint32_t n, uint32_t nb, uint32_t leaf_size, int grid, uint32_t scene_box_cells,
              sq::Node* nodes, float* scene_out, void* ws, uint32_t* sort_keys, uint32_t* sort_vals,
              uint32_t* sort_alt_keys, uint32_t* sort_alt_vals, uint32_t* sort_lookback, uint32_t* sort_counters,
              uint32_t* err, uint32_t* host_ctl, cudaStream_t s)
{
    const SahWs w = carve(ws, n, 0);
    const uint32_t base = grid ? 128u : 0u;
    const uint32_t leaf0 = base + 2u * n + 2u;
    cudaError_t e;
#define SQ_TRY(x) do { if ((e = (x)) != cudaSuccess) return (int)e; } while (0)
    SQ_TRY(cudaMemsetAsync(w.cells, 0, sizeof(uint32_t) * 64 * kBinWords, s));
    SQ_TRY(cudaMemsetAsync(w.hist, 0, sizeof(uint32_t) * 64, s));
    SQ_TRY(cudaMemsetAsync(w.root_ord, 0, sizeof(uint32_t) * 16, s));
    SQ_TRY(cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), s));
    const uint32_t g = min((n + 255) / 256, (uint32_t)sms() * 8u);
    k_sah_setup<<<g, 256, 0, s>>>(tris, n, w.tb, w.ids_a, w.root_ord);
    if (!grid) {
        k_root_task<<<1, 1, 0, s>>>(w.root_ord, n, leaf_size, w.lists[0], w.small, w.leaves, w.ctl, scene_out);
    } else {
        // bin into 64 cells keyed by Morton slot, then stable sort by slot
        k_grid_bin<<<g, 256, 0, s>>>(w.tb, n, w.root_ord, sort_keys, w.cells, w.hist);
        SQ_TRY(cudaMemcpyAsync(sort_vals, w.ids_a, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        const int which = sort_passes(sort_keys, sort_vals, sort_alt_keys, sort_alt_vals, n, w.hist, sort_lookback,
                                      sort_counters, 6, 1, err, s);
        SQ_TRY(cudaMemcpyAsync(w.ids_a, which ? sort_alt_vals : sort_vals, sizeof(uint32_t) * (size_t)n,
                               cudaMemcpyDeviceToDevice, s));
        k_grid_tasks<<<1, 64, 0, s>>>(w.cells, w.root_ord, n, leaf_size, scene_box_cells, w.lists[0], w.small,
                                      w.leaves, w.ctl, scene_out);
    }
    // large phase: the level kernels read their task counts on the device
    // and stride over them with fixed grids, so levels are queued
    // kSahLevelsPerCheck at a time and the host reads a count (and waits)
    // only between such groups; levels past the tree's depth find no tasks
    // and do nothing.  One host round trip per level left the GPU idle for
    // most of a small mesh's build.
    const uint32_t grid_fixed = (uint32_t)sms() * 8u;
    for (uint32_t level = 0;; level += kSahLevelsPerCheck) {
        SQ_TRY(cudaMemcpyAsync(host_ctl, &w.ctl->n_large[level & 1], sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        SQ_TRY(cudaStreamSynchronize(s));
        if (host_ctl[0] == 0) break;
        for (uint32_t j = 0; j < kSahLevelsPerCheck; ++j)
            enqueue_large_level(w, level + j, (int)nb, base, leaf_size, nodes, grid_fixed, grid_fixed, n, s);
    }
    // small phase and leaves
    const uint32_t sg = (uint32_t)sms() * 8u;
    // a single build's small tasks all have at most kSmall = kStage triangles
    static_assert(kSmall <= kStage, "every small task of a single build is staged");
    k_small<true><<<sg, 128, 0, s>>>(w.small, w.ctl, w.ids_a, w.ids_b, w.tb, (int)nb, leaf_size, base, nodes, leaf0,
                                     err);
    k_emit_leaves<<<sg, 256, 0, s>>>(w.leaves, w.ctl, w.ids_a, w.ids_b, w.tb, nodes, leaf0, err);
    if (grid) k_grid_heap<<<1, 32, 0, s>>>(nodes);
    return (int)cudaGetLastError();
#undef SQ_TRY
}

// Binned SAH trees of M meshes at once, with no host synchronisation (a
// fixed number of large-phase levels with device-side task counts, so the
// sequence can be captured in a CUDA graph).  Mesh m holds triangles
// [off[m], off[m + 1]) of the concatenated `tris` (off on the device, M + 1
// words); its root is record root0 + m, inner records at 2q and 2q + 1 for a
// split at q, leaf records at 2n + 2 + position -- the layout of a single
// build, shifted by the mesh's offset.  Large tasks left after the last
// fixed level go to the small phase (same splits, one warp per subtree).
int build_sah_batch(const float* tris, uint32_t n, const uint32_t* off, uint32_t M, uint32_t nb, uint32_t leaf_size,
                    uint32_t root0, sq::Node* nodes, void* ws, uint32_t* err, cudaStream_t s)
{
    const SahWs w = carve(ws, n, M);
    const uint32_t leaf0 = 2u * n + 2u;
    cudaError_t e;
#define SQ_TRY(x) do { if ((e = (x)) != cudaSuccess) return (int)e; } while (0)
    SQ_TRY(cudaMemsetAsync(w.root_ord, 0, sizeof(uint32_t) * 16ull * M, s));
    SQ_TRY(cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), s));
    const uint32_t sm = (uint32_t)sms();
    if (n > 0) {
        const uint32_t g = min((n + 255) / 256, sm * 8u);
        k_sah_setup_seg<<<g, 256, 0, s>>>(tris, n, off, M, w.tb, w.ids_a, w.root_ord);
    }
    k_root_tasks_seg<<<(M + 127) / 128, 128, 0, s>>>(w.root_ord, off, M, leaf_size, root0, w.lists[0], w.small,
                                                      w.leaves, w.ctl);
    for (uint32_t level = 0; level < kBatchLargeLevels; ++level)
        enqueue_large_level(w, level, (int)nb, 0u, leaf_size, nodes, sm * 8u, sm * 8u, n, s);
    k_large_to_small<<<sm, 256, 0, s>>>(w.lists[kBatchLargeLevels & 1], &w.ctl->n_large[kBatchLargeLevels & 1],
                                       w.small, w.ctl);
    k_small<true><<<sm * 8u, 128, 0, s>>>(w.small, w.ctl, w.ids_a, w.ids_b, w.tb, (int)nb, leaf_size, 0u, nodes, leaf0,
                                          err);
    k_small<false><<<sm * 8u, 128, 0, s>>>(w.small, w.ctl, w.ids_a, w.ids_b, w.tb, (int)nb, leaf_size, 0u, nodes, leaf0,
                                           err);
    k_emit_leaves<<<sm * 8u, 256, 0, s>>>(w.leaves, w.ctl, w.ids_a, w.ids_b, w.tb, nodes, leaf0, err);
    return (int)cudaGetLastError();
#undef SQ_TRY
}

}  // namespace sqk
