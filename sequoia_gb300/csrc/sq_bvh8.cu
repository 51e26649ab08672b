// sq_bvh8.cu -- 8-wide BVH with 8-bit quantised child boxes (the precision
// form), built by collapsing a binary range-tree BVH (node layout in
// sq_bvh8_dev.cuh; its traversal is in sq_bvh8_trace.cu).
//
// Child box on axis a: [origin_a + qlo * 2^e_a, origin_a + qhi * 2^e_a], each
// bound computed exactly as the traversal computes it (one rounded add of an
// exact product) and moved outward until it contains the binary node's FP32
// box, so a quantised box is never smaller than the FP32 box it replaces.
// This is the compressed wide BVH idea of Ylitie, Karras and Laine
// ("Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
// BVHs", HPG 2017), laid out our own way.
//
// Collapse: each 8-wide node starts from a binary inner record's two children
// and repeatedly opens the inner child of largest surface area until it has 8
// children or no inner child is left.  Leaf-cluster records (and single leaf
// records) become leaf children; their triangles are copied into a 48-byte
// triangle array in leaf order, with the original triangle index in the
// fourth float of the first vertex.
#include "sq_bvh8_dev.cuh"

#include <algorithm>
#include <type_traits>
#include <utility>

namespace {

using namespace sq;

__device__ __forceinline__ float node_sa(const Node& r)
{
    const float lx = r.mxx - r.mnx, ly = r.mxy - r.mny, lz = r.mxz - r.mnz;
    return lx * ly + lx * lz + ly * lz;
}


// Exponent of the quantisation step so that origin + 255 * 2^e >= hi.
__device__ int quant_exp(float lo, float hi)
{
    const float ext = hi - lo;
    int e = -126;
    if (ext > 0.0f) {
        int ex;
        frexpf(ext, &ex);  // ext in [2^(ex-1), 2^ex)
        e = ex - 8;        // 255 * 2^e >= 2^(ex-1) * 255/128 ... adjusted below
        if (e < -126) e = -126;
        while (e > -126 && fmaf(255.0f, pow2f(e - 1), lo) >= hi) --e;
        while (fmaf(255.0f, pow2f(e), lo) < hi && e < 127) ++e;
    }
    return e;
}

// (v - origin) / 2^e is computed as (v - origin) * 2^-e: both are the
// correctly rounded value of the same real number (2^-e is exact for every
// exponent quant_exp returns), and the multiply is far cheaper.
__device__ __forceinline__ uint8_t quant_lo(float v, float origin, int e)
{
    const float s = pow2f(e);
    float q = floorf((v - origin) * ldexpf(1.0f, -e));
    int qi = q < 0.0f ? 0 : (q > 255.0f ? 255 : (int)q);
    while (qi > 0 && fmaf((float)qi, s, origin) > v) --qi;
    return (uint8_t)qi;
}

__device__ __forceinline__ uint8_t quant_hi(float v, float origin, int e)
{
    const float s = pow2f(e);
    float q = ceilf((v - origin) * ldexpf(1.0f, -e));
    int qi = q < 0.0f ? 0 : (q > 255.0f ? 255 : (int)q);
    while (qi < 255 && fmaf((float)qi, s, origin) < v) ++qi;
    return (uint8_t)qi;
}


// Build 8-wide nodes from binary records, eight lanes per node and four
// nodes per warp.  Lane k of a group holds candidate child slot k (its binary
// record in registers), so the records a step opens are loaded in parallel
// and the six dequantised planes of each slot are computed by the slot's own
// lane.  The decisions are those of a sequential scan over the slots: open
// the first child of largest surface area that still fits, until none does.
// All 32 lanes must call this; a group whose `active` is false only takes
// part in the warp-wide shuffles.  Inner children become nodes
// [child_base, child_base + n) and leaf triangles take the triangle slots
// [tri_base, ...).
// The warp's four groups allocate together: lane 0 calls
// alloc(nodes, tris, node_base, tri_base, task_base) once with the warp's
// totals (one atomic per warp instead of one per node and one per child:
// same-address atomics serialise in L2), and each group takes its share in
// group order.  publish(task, node, record) is called by the child's lane
// with task = task_base + the child's rank in the warp.  sm: this warp's
// staging area (one GroupSmem per warp).
struct GroupSmem {
    Node8 node[4];
    uint32_t off[4][8], cnt[4][8], child[4][8];
};

template <class Alloc, class Publish>
__device__ void collapse_node_group(const Node* __restrict__ rec, uint32_t leaf0, const float* __restrict__ tris,
                                    bool active, uint32_t rec_i, uint32_t node_i, Node8* __restrict__ nodes8,
                                    float4* __restrict__ tris8, uint32_t* err, GroupSmem& sm, Alloc alloc,
                                    Publish publish)
{
    constexpr uint32_t FULL = 0xFFFFFFFFu;
    const int lane = (int)(threadIdx.x & 31u);
    const int k = lane & 7;   // slot of this lane
    const int g = lane >> 3;  // group (node) of this lane
    const int gs = lane & ~7; // first lane of the group
    auto gballot = [&](bool pr) -> uint32_t { return (__ballot_sync(FULL, pr) >> gs) & 0xFFu; };
    Node self;
    uint32_t c0 = 0, cn = 0;
    if (active) {
        self = rec[rec_i];
        c0 = self.child;
        cn = node_count(self.count_flags);
        if (cn > 8) {
            if (k == 0) raise_error(err, SQ_DEVERR_NODE_COUNT);
            active = false;
        }
    }
    // slot state of this lane
    Node e_node;
    e_node.child = 0;
    e_node.count_flags = 0;
    uint32_t e_rec = 0, e_kind = 0, e_cnt = 0;
    float e_sa = 0.0f;
    auto load_entry = [&](uint32_t i) {
        e_node = rec[i];
        e_rec = i;
        e_sa = node_sa(e_node);
        e_cnt = node_count(e_node.count_flags);
        if (node_is_leaf(e_node.count_flags)) e_kind = 2;
        else e_kind = (e_node.child < leaf0 && e_cnt > 0) ? 0u : 1u;
        // the records an opening of this entry would load, towards L2 now:
        // the collapse is a chain of dependent record loads
        if (e_kind != 2 && e_cnt > 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(rec + e_node.child));
    };
    if (active && k < (int)cn) load_entry(c0 + (uint32_t)k);
    // the start set is a binary record's two children or a cluster's leaves;
    // open the child of largest area (a binary record into its two children,
    // a leaf cluster into its single-triangle leaves) while it fits in 8 slots
    int nc = active ? (int)cn : 0;
    bool opening = active;
    for (;;) {
        const bool can = opening && k < nc &&
                         (e_kind == 0 ? (nc + 1 <= 8) : (e_kind == 1 && nc + (int)e_cnt - 1 <= 8));
        const uint32_t canm = gballot(can);
        opening = opening && canm != 0;
        if (!__any_sync(FULL, opening)) break;
        int best = -1;
        float bsa = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float sq = __shfl_sync(FULL, e_sa, q, 8);
            if (((canm >> q) & 1u) && (best < 0 || sq > bsa)) { best = q; bsa = sq; }
        }
        const int bs = best < 0 ? 0 : best;
        const uint32_t bkind = __shfl_sync(FULL, e_kind, bs, 8), bcnt = __shfl_sync(FULL, e_cnt, bs, 8);
        const uint32_t bchild = __shfl_sync(FULL, e_node.child, bs, 8);
        const uint32_t m = bkind == 0 ? 2u : bcnt;
        const bool drop = opening && m == 0;
        if (__any_sync(FULL, drop)) {
            // drop the empty cluster: the group's last slot moves into its place
            const int src = nc > 0 ? nc - 1 : 0;
            Node t;
            t.mnx = __shfl_sync(FULL, e_node.mnx, src, 8); t.mny = __shfl_sync(FULL, e_node.mny, src, 8);
            t.mnz = __shfl_sync(FULL, e_node.mnz, src, 8);
            t.count_flags = __shfl_sync(FULL, e_node.count_flags, src, 8);
            t.mxx = __shfl_sync(FULL, e_node.mxx, src, 8); t.mxy = __shfl_sync(FULL, e_node.mxy, src, 8);
            t.mxz = __shfl_sync(FULL, e_node.mxz, src, 8); t.child = __shfl_sync(FULL, e_node.child, src, 8);
            const uint32_t trec = __shfl_sync(FULL, e_rec, src, 8), tkind = __shfl_sync(FULL, e_kind, src, 8);
            const uint32_t tcnt = __shfl_sync(FULL, e_cnt, src, 8);
            const float tsa = __shfl_sync(FULL, e_sa, src, 8);
            if (drop) {
                if (k == best) { e_node = t; e_rec = trec; e_kind = tkind; e_cnt = tcnt; e_sa = tsa; }
                --nc;
            }
        }
        if (opening && m != 0) {
            if (k == best) load_entry(bchild);
            else if (k >= nc && k < nc + (int)m - 1) load_entry(bchild + 1u + (uint32_t)(k - nc));
            nc += (int)m - 1;
        }
    }
    // a cluster of 2..8 triangles that did not fit becomes a wide child node
    // of its own (its triangles one per slot), so every triangle keeps its own
    // box; larger clusters stay leaf children of up to 15 triangles
    if (k < nc && e_kind == 1 && e_cnt >= 2 && e_cnt <= 8) e_kind = 0;
    // children with an empty box (empty grid cells and subtrees of them) take
    // no slot
    const bool ok = k < nc && e_node.mnx <= e_node.mxx && e_node.mny <= e_node.mxy && e_node.mnz <= e_node.mxz;
    const bool inner = ok && e_kind == 0;
    const bool leafc = ok && e_kind != 0;
    if (gballot(leafc && e_cnt > 15u)) {
        if (active && k == 0) raise_error(err, SQ_DEVERR_NODE_COUNT);
        active = false;
    }
    const uint32_t cntk = leafc ? e_cnt : 0u;
    const uint32_t imask = gballot(inner);
    const uint32_t valid = gballot(ok);
    const uint32_t leafrec = gballot(k < nc && node_is_leaf(e_node.count_flags));
    uint32_t incl = cntk;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o, 8);
        if (k >= o) incl += y;
    }
    const uint32_t n_tris = __shfl_sync(FULL, incl, 7, 8);
    const uint32_t tri_off = incl - cntk;
    const uint32_t n_inner = active ? __popc(imask) : 0u, n_place = active ? n_tris : 0u;
    // the warp's totals and this group's offsets (groups in lane order)
    uint32_t pre_i = 0, pre_t = 0, sum_i = 0, sum_t = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t a = __shfl_sync(FULL, n_inner, 8 * q), b = __shfl_sync(FULL, n_place, 8 * q);
        if (q < g) { pre_i += a; pre_t += b; }
        sum_i += a;
        sum_t += b;
    }
    uint32_t node_base = 0, tri_base = 0, task_base = 0;
    if (lane == 0 && (sum_i | sum_t)) alloc(sum_i, sum_t, node_base, tri_base, task_base);
    const uint32_t child_base = __shfl_sync(FULL, node_base, 0) + pre_i;
    tri_base = __shfl_sync(FULL, tri_base, 0) + pre_t;
    task_base = __shfl_sync(FULL, task_base, 0) + pre_i;
    // quantised child planes, one slot per lane, staged in shared memory
    Node8& sn = sm.node[g];
    int e[3] = {0, 0, 0};
    if (active) {
        const float lo[3] = {self.mnx, self.mny, self.mnz}, hi[3] = {self.mxx, self.mxy, self.mxz};
#pragma unroll
        for (int a = 0; a < 3; ++a) e[a] = quant_exp(lo[a], hi[a]);
        uint32_t ql[3] = {255u, 255u, 255u}, qh[3] = {0u, 0u, 0u};
        if (ok) {
            const float cl[3] = {e_node.mnx, e_node.mny, e_node.mnz}, ch[3] = {e_node.mxx, e_node.mxy, e_node.mxz};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                ql[a] = quant_lo(cl[a], lo[a], e[a]);
                qh[a] = quant_hi(ch[a], lo[a], e[a]);
            }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) { sn.qlo[a][k] = (uint8_t)ql[a]; sn.qhi[a][k] = (uint8_t)qh[a]; }
        sm.off[g][k] = tri_off;
        sm.cnt[g][k] = cntk;
        sm.child[g][k] = e_node.child;
        if (inner) {
            const uint32_t r = __popc(imask & ((1u << k) - 1u));
            publish(task_base + r, child_base + r, e_rec);
        }
    }
    __syncwarp();
    if (active && k == 0) {
        uint32_t counts = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) counts |= sm.cnt[g][q] << (4 * q);
        sn.ox = self.mnx; sn.oy = self.mny; sn.oz = self.mnz;
        sn.exps_imask = (uint32_t)(e[0] + 127) | ((uint32_t)(e[1] + 127) << 8) | ((uint32_t)(e[2] + 127) << 16) |
                        (imask << 24);
        sn.child_base = child_base;
        sn.tri_base = tri_base;
        sn.counts = counts;
        sn.valid = valid;
    }
    __syncwarp();
    if (active) {
        // the node: five 16-byte words
        if (k < 5) reinterpret_cast<float4*>(nodes8 + node_i)[k] = reinterpret_cast<const float4*>(&sn)[k];
        // leaf triangles, spread over the group: triangle t of the node
        // belongs to the leaf slot whose [off, off + cnt) holds it
        for (uint32_t t = (uint32_t)k; t < n_tris; t += 8u) {
            int q = 0;
#pragma unroll
            for (int r = 1; r < 8; ++r)
                if (sm.cnt[g][r] && sm.off[g][r] <= t) q = r;
            const uint32_t j = t - sm.off[g][q], qc = sm.child[g][q];
            // a leaf record is its own triangle; a cluster's are its leaves
            const uint32_t id = ((leafrec >> q) & 1u) ? qc + j : rec[qc + j].child;
            float tv[9];
            load_tri(tris, id, tv);
            float4* d = tris8 + 3ull * (tri_base + t);
            d[0] = make_float4(tv[0], tv[1], tv[2], __uint_as_float(id));
            d[1] = make_float4(tv[3], tv[4], tv[5], 0.0f);
            d[2] = make_float4(tv[6], tv[7], tv[8], 0.0f);
        }
    }
    __syncwarp();  // the staging area is reused by the warp's next nodes
}

// Nodes and triangle slots of one warp from the counter pair at ctr (nodes
// in word 0, triangles in word 1: one 64-bit atomic).  On overflow of the
// node capacity the error word is set and the nodes land at `capacity`, where
// nothing is written.
__device__ __forceinline__ void alloc_nodes_tris(uint32_t* ctr, uint32_t kn, uint32_t kt, uint32_t capacity,
                                                 uint32_t* err, uint32_t& nb, uint32_t& tb)
{
    const unsigned long long v =
        atomicAdd(reinterpret_cast<unsigned long long*>(ctr), ((unsigned long long)kt << 32) | kn);
    nb = (uint32_t)v;
    tb = (uint32_t)(v >> 32);
    if ((unsigned long long)nb + kn > capacity) {
        raise_error(err, SQ_DEVERR_SAH_QUEUE);
        nb = capacity;
    }
}

// One level of the collapse: group i (four per warp) builds node
// task_node[i] from binary record tasks[i]; inner children are allocated
// contiguously from the node counter and appended to the next level's list.
constexpr int kCollapseBlock = 128;

__global__ void __launch_bounds__(kCollapseBlock) k_collapse_level(
    const Node* __restrict__ rec, uint32_t leaf0, const float* __restrict__ tris, const uint32_t* __restrict__ tasks,
    const uint32_t* __restrict__ task_node, uint32_t ntasks, Node8* __restrict__ nodes8, float4* __restrict__ tris8,
    uint32_t* __restrict__ counters, uint32_t* __restrict__ next_tasks, uint32_t* __restrict__ next_node,
    uint32_t capacity, uint32_t* err)
{
    __shared__ GroupSmem s_group[kCollapseBlock / 32];
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (4u * w >= ntasks) return;  // whole warps
    const uint32_t i = 4u * w + ((threadIdx.x & 31u) >> 3);
    const bool active = i < ntasks;
    auto alloc = [&](uint32_t kn, uint32_t kt, uint32_t& nb, uint32_t& tb, uint32_t& jb) {
        alloc_nodes_tris(counters, kn, kt, capacity, err, nb, tb);
        jb = kn ? atomicAdd(counters + 2, kn) : 0u;
    };
    auto publish = [&](uint32_t j, uint32_t node, uint32_t record) {
        if (node >= capacity) return;
        next_tasks[j] = record;
        next_node[j] = node;
    };
    collapse_node_group(rec, leaf0, tris, active, active ? tasks[i] : 0u, active ? task_node[i] : 0u, nodes8, tris8,
                        err, s_group[threadIdx.x >> 5], alloc, publish);
}

// Collapse without host synchronisation (so it can be captured in a CUDA
// graph): a fixed number of level kernels, each a grid-stride loop over the
// task count its predecessor left in device memory (counts[level]); a level
// with no tasks returns at once.  Nothing waits on anything.  If the tree is
// deeper than the launched levels, the last level raises SQ_DEVERR_SAH_QUEUE.
constexpr uint32_t kFixedLevels = 64;

__global__ void __launch_bounds__(128) k_collapse_fixed(const Node* __restrict__ rec, uint32_t leaf0,
                                                        const float* __restrict__ tris, uint32_t level,
                                                        uint32_t* __restrict__ counts, const uint32_t* __restrict__ tasks,
                                                        const uint32_t* __restrict__ task_node,
                                                        uint32_t* __restrict__ next_tasks, uint32_t* __restrict__ next_node,
                                                        uint32_t* __restrict__ counters2, Node8* __restrict__ nodes8,
                                                        float4* __restrict__ tris8, uint32_t capacity, uint32_t* err)
{
    chain_wait();  // a chained launch: the levels follow one another
    chain_release();
    const uint32_t ntasks = counts[level];
    if (ntasks == 0) return;
    if (level + 1 >= kFixedLevels) {
        if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(err, SQ_DEVERR_SAH_QUEUE);
        return;
    }
    __shared__ GroupSmem s_group[4];
    uint32_t* next_count = counts + level + 1;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = 4u * ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); base < ntasks; base += 4u * warps) {
        const uint32_t i = base + ((threadIdx.x & 31u) >> 3);
        const bool active = i < ntasks;
        auto alloc = [&](uint32_t kn, uint32_t kt, uint32_t& nb, uint32_t& tb, uint32_t& jb) {
            alloc_nodes_tris(counters2, kn, kt, capacity, err, nb, tb);
            jb = kn ? atomicAdd(next_count, kn) : 0u;
        };
        auto publish = [&](uint32_t j, uint32_t node, uint32_t record) {
            if (node >= capacity) return;
            next_tasks[j] = record;
            next_node[j] = node;
        };
        collapse_node_group(rec, leaf0, tris, active, active ? tasks[i] : 0u, active ? task_node[i] : 0u, nodes8,
                            tris8, err, s_group[threadIdx.x >> 5], alloc, publish);
    }
}

// All levels in one cooperative launch (every block is resident): a
// grid-stride loop over a level's tasks, a grid barrier, the next level.  No
// host round trip per level.  The barrier's wait is bounded: a block that
// polls more than kBarrierSpins times raises SQ_DEVERR_SAH_QUEUE and returns
// (the other blocks then time out at their next barrier too).  Task lists
// are read through L2 (__ldcg): the same lists are rewritten every other
// level, so an SM's L1 may hold stale lines of them.  The failure-detection
// tests pass a small poll limit and one phantom block (barrier_extra = 1)
// that never arrives: every block then gives up at the first barrier.
constexpr uint32_t kBarrierSpins = 1u << 24;

// Grid barrier; the last block to arrive runs on_last() (thread 0 only)
// after every other block's writes before the barrier are visible to it and
// before any block leaves.
template <class OnLast>
__device__ bool grid_barrier(uint32_t* bar, uint32_t nblocks, uint32_t spin_limit, uint32_t* err, OnLast on_last)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const uint32_t gen = ld_acquire_u32(bar + 1);
        __threadfence();
        if (atomicAdd(bar, 1u) + 1u == nblocks) {
            // last arrival: reset the count, then open the next generation
            __threadfence();
            on_last();
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t spins = 0;
            while (ld_acquire_u32(bar + 1) == gen) {
                if (++spins > spin_limit) {
                    raise_error(err, SQ_DEVERR_SAH_QUEUE);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The tasks of a level are the nodes [lo, hi) that the previous level
// allocated, in allocation order: task j builds node lo + j from the binary
// record in the level's task list at j.  A warp's allocation at node base b
// therefore also places its children's tasks at b - hi in the next list, and
// the next level's end is the node counter once the level is done (read by
// the barrier's last block).
__global__ void __launch_bounds__(256) k_collapse_coop(const Node* __restrict__ rec, uint32_t leaf0,
                                                       const float* __restrict__ tris, uint32_t* __restrict__ ws,
                                                       uint32_t capacity, Node8* __restrict__ nodes8,
                                                       float4* __restrict__ tris8, uint32_t* err,
                                                       uint32_t barrier_extra, uint32_t spin_limit)
{
    // ws: [0] node counter, [1] triangle counter (one 64-bit pair), [2..3]
    // barrier, [4] levels done, [5] end of the next level's nodes, then the
    // task lists of even and odd levels (`capacity` records each, at the
    // offsets the seed uses)
    uint32_t* bar = ws + 2;
    uint32_t* ta = ws + 8 + kFixedLevels + 8;
    uint32_t* tb = ta + 2ull * capacity;
    __shared__ GroupSmem s_group[8];
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lo = 0, hi = 1;  // the root task
    for (uint32_t level = 0;; ++level) {
        const uint32_t ntasks = hi - lo;
        if (ntasks == 0) {
            if (blockIdx.x == 0 && threadIdx.x == 0) ws[4] = level;
            return;
        }
        if (level + 1 >= kFixedLevels) {
            if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(err, SQ_DEVERR_SAH_QUEUE);
            return;
        }
        const uint32_t* tasks = (level & 1) ? tb : ta;
        uint32_t* next_tasks = (level & 1) ? ta : tb;
        for (uint32_t base = 4u * wid; base < ntasks; base += 4u * warps) {
            const uint32_t i = base + ((threadIdx.x & 31u) >> 3);
            const bool active = i < ntasks;
            auto alloc = [&](uint32_t kn, uint32_t kt, uint32_t& nb, uint32_t& tb_, uint32_t& jb) {
                alloc_nodes_tris(ws, kn, kt, capacity, err, nb, tb_);
                jb = nb - hi;
            };
            auto publish = [&](uint32_t j, uint32_t node, uint32_t record) {
                if (node >= capacity) return;
                next_tasks[j] = record;
            };
            collapse_node_group(rec, leaf0, tris, active, active ? __ldcg(tasks + i) : 0u, lo + i, nodes8, tris8, err,
                                s_group[threadIdx.x >> 5], alloc, publish);
        }
        const bool ok = grid_barrier(bar, gridDim.x + barrier_extra, spin_limit, err, [&]() {
            const uint32_t end = ld_acquire_u32(ws);
            st_relaxed_u32(ws + 5, end < capacity ? end : capacity);
        });
        if (!ok) return;
        lo = hi;
        hi = ld_acquire_u32(ws + 5);
    }
}

// Seed of the cooperative collapse: one root task (record `root`, node 0).
__global__ void k_coop_seed(uint32_t* __restrict__ ws, uint32_t root)
{
    ws[0] = 1u;  // node 0 is the root
    ws[8 + kFixedLevels + 8] = root;  // the first task list
}

__global__ void k_fixed_seed(const uint32_t* __restrict__ roots, uint32_t nroots, uint32_t* __restrict__ tasks,
                             uint32_t* __restrict__ task_node, uint32_t* __restrict__ counts,
                             uint32_t* __restrict__ node_counter)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nroots; i += gridDim.x * blockDim.x) {
        tasks[i] = roots[i];
        task_node[i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counts[0] = nroots;
        *node_counter = nroots;
    }
}

}  // namespace

namespace sqk {

int build_bvh8_queue(const Node* rec, const uint32_t* roots_dev, uint32_t nroots, uint32_t leaf0, const float* tris,
                     uint32_t n, void* nodes8, void* tris8, uint32_t* ws, uint32_t* err, cudaStream_t s)
{
    // ws: [0] node counter, [1] triangle counter, [8 .. 8+kFixedLevels] level
    // counts, then two (record, node) task lists of `capacity` entries
    const uint32_t capacity = bvh8_capacity(n) + nroots;
    uint32_t* node_counter = ws;
    uint32_t* counts = ws + 8;
    uint32_t* ta = counts + kFixedLevels + 8;
    uint32_t* na = ta + capacity;
    uint32_t* tb = na + capacity;
    uint32_t* nb = tb + capacity;
    cudaError_t e;
    if ((e = cudaMemsetAsync(ws, 0, sizeof(uint32_t) * (16 + kFixedLevels), s)) != cudaSuccess) return (int)e;
    k_fixed_seed<<<(nroots + 255) / 256, 256, 0, s>>>(roots_dev, nroots, ta, na, counts, node_counter);
    static PerDevice<int> cache;
    const int grid = cache.get([] { return blocks_per_sm(k_collapse_fixed, 128) * sm_count(); });
    for (uint32_t level = 0; level < kFixedLevels; ++level) {
        uint32_t* in_t = (level & 1) ? tb : ta;
        uint32_t* in_n = (level & 1) ? nb : na;
        uint32_t* out_t = (level & 1) ? ta : tb;
        uint32_t* out_n = (level & 1) ? na : nb;
        launch_chained(k_collapse_fixed, dim3(grid), dim3(128), 0, s, rec, leaf0, tris, level, counts,
                       (const uint32_t*)in_t, (const uint32_t*)in_n, out_t, out_n, ws, static_cast<Node8*>(nodes8),
                       static_cast<float4*>(tris8), capacity, err);
    }
    return (int)cudaGetLastError();
}



// A wide node has at least two children except the root and nodes next to
// empty grid cells (at most 64 of those), so n + 130 nodes always suffice.
uint32_t bvh8_capacity(uint32_t n) { return n + 130u; }
size_t bvh8_node_bytes(uint32_t n) { return sizeof(Node8) * (size_t)bvh8_capacity(n); }
size_t bvh8_ws_words(uint32_t n) { return 4ull * bvh8_capacity(n) + 16 + 2 * kFixedLevels; }
size_t bvh8_tri_bytes(uint32_t n) { return sizeof(float4) * 3ull * ((size_t)n + 1); }

// Collapse the binary tree rooted at record `root` (an inner record) into
// nodes8 / tris8, one kernel launch per level of the 8-wide tree (the host
// reads each level's task count from pinned memory).  ws: bvh8_ws_words(n)
// words; host_ctl: pinned, 4 words.  Returns 0 or a cudaError_t; the node
// count is host_ctl[0] and the number of levels host_ctl[3].
static int build_bvh8_levels(const Node* rec, uint32_t root, uint32_t leaf0, const float* tris, uint32_t n, void* nodes8, void* tris8,
               uint32_t* ws, uint32_t* host_ctl, uint32_t* err, cudaStream_t s)
{
    const uint32_t capacity = bvh8_capacity(n);
    uint32_t* counters = ws;  // [0] nodes allocated, [1] triangles placed, [2] next-level tasks
    uint32_t* ta = ws + 8;    // task lists (record, node), two levels
    uint32_t* na = ta + capacity;
    uint32_t* tb = na + capacity;
    uint32_t* nb = tb + capacity;
    cudaError_t e;
    const uint32_t init[4] = {1u, 0u, 0u, 0u};
    if ((e = cudaMemcpyAsync(counters, init, sizeof init, cudaMemcpyHostToDevice, s)) != cudaSuccess) return (int)e;
    const uint32_t first[2] = {root, 0u};
    if ((e = cudaMemcpyAsync(ta, &first[0], 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyAsync(na, &first[1], 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return (int)e;
    uint32_t ntasks = 1, levels = 0;
    while (ntasks) {
        ++levels;
        if ((e = cudaMemsetAsync(counters + 2, 0, 4, s)) != cudaSuccess) return (int)e;
        k_collapse_level<<<(ntasks + 15) / 16, kCollapseBlock, 0, s>>>(rec, leaf0, tris, ta, na, ntasks,
                                                               static_cast<Node8*>(nodes8), static_cast<float4*>(tris8),
                                                               counters, tb, nb, capacity, err);
        if ((e = cudaMemcpyAsync(host_ctl, counters, 12, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return (int)e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return (int)e;
        ntasks = host_ctl[2];
        std::swap(ta, tb);
        std::swap(na, nb);
    }
    host_ctl[3] = levels;
    host_ctl[4] = levels;  // one launch per level
    return (int)cudaGetLastError();
}

int build_bvh8(const Node* rec, uint32_t root, uint32_t leaf0, const float* tris, uint32_t n, void* nodes8, void* tris8,
               uint32_t* ws, uint32_t* host_ctl, uint32_t* err, cudaStream_t s, uint32_t* meta,
               const BarrierStall* stall)
{
    host_ctl[5] = 0;
    // every block of the cooperative collapse must be resident: at most the
    // occupancy limit per SM (0: no cooperative launch, use the per-level
    // path).  From 5M triangles up, four blocks per SM instead of the limit
    // (five): on Gaussian soups the 6M and 8M collapses took 0.61 / 0.76 ms
    // with four against 0.64 / 0.86 ms with five, while at 1-4M (and the 4M
    // terrain) five were as fast or faster.
    static PerDevice<int> cache;
    const int per_sm = cache.get([] {
        int coop = 0, occ = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, current_device());
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_collapse_coop, 256, 0);
        return (coop && occ > 0) ? occ : 0;
    });
    const int grid = (n >= 5000000u && per_sm > 4 ? 4 : per_sm) * sm_count();
    if (grid == 0) return build_bvh8_levels(rec, root, leaf0, tris, n, nodes8, tris8, ws, host_ctl, err, s);
    const uint32_t capacity = bvh8_capacity(n);
    cudaError_t e;
    if ((e = cudaMemsetAsync(ws, 0, sizeof(uint32_t) * (16 + kFixedLevels), s)) != cudaSuccess) return (int)e;
    k_coop_seed<<<1, 1, 0, s>>>(ws, root);
    const uint32_t extra = stall ? 1u : 0u;
    const uint32_t spins = stall ? stall->spin_limit : kBarrierSpins;
    void* args[] = {(void*)&rec, (void*)&leaf0, (void*)&tris, (void*)&ws, (void*)&capacity, (void*)&nodes8,
                    (void*)&tris8, (void*)&err, (void*)&extra, (void*)&spins};
    if ((e = cudaLaunchCooperativeKernel((const void*)k_collapse_coop, dim3(grid), dim3(256), args, 0, s)) !=
        cudaSuccess)
        return (int)e;
    host_ctl[4] = 2;  // the seed and the cooperative kernel
    if (meta) {
        // node count and levels stay on the device until asked for
        if ((e = cudaMemcpyAsync(meta, ws, 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return (int)e;
        if ((e = cudaMemcpyAsync(meta + 1, ws + 4, 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return (int)e;
        host_ctl[5] = 1;
        return (int)cudaGetLastError();
    }
    // node count -> host_ctl[0], levels -> host_ctl[3]
    if ((e = cudaMemcpyAsync(host_ctl, ws, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return (int)e;
    if ((e = cudaMemcpyAsync(host_ctl + 3, ws + 4, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return (int)e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return (int)e;
    return (int)cudaGetLastError();
}

}  // namespace sqk
