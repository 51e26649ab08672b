// sq_coherent.cu -- the reference's packet and bundle tracers on the GPU.
//
// trace_packet<k> (src/tracer.cpp:232-281, traverse_packet_stack 88-123):
// the k = kx * ky rays of a kx x ky pixel block (kx = floor(sqrt(k)), rays in
// row order) traverse together: a node's children are visited when any ray
// of the packet hits the node's box, and the packet counts one test per node
// box.  Every pixel of the packet gets (tests / k) / 200 in the heatmap.  On
// the GPU a packet is k lanes of a warp (32 / k packets per warp); "any ray"
// is a ballot over the packet's lanes, so the lanes of a packet take one path
// and keep identical stacks.
//
// trace_bundle<k> (src/tracer.cpp:292-362, traverse_bundle 126-156,
// intersect_bundle_aabb src/tracer.h:37-80): a tile of k = 16 or 64 rays
// (tw x th pixels, tw = floor(sqrt(k))), ray m * 8 + n at tile position
// morton_lut[m * 8 + n], is tested as one bundle against the box with the
// bundle's direction bounds (min, max and midpoint) while the midpoint
// direction hits; where only the bounds can hit, each packet of 8 rays
// continues alone from that node (the packet tracer above).  A pixel of
// packet m gets bundle_tests / k + packet_tests[m] / 8.  One warp traces one
// tile: the bundle part is the same for every lane, and the packets of 8 are
// 8-lane groups (two rays per lane for k = 64).
//
// Both counts are independent of the visiting order (nothing terminates
// early), so the stack order need not be the reference's.  The heatmap bytes
// are the reference's exactly.
#include "sq_common.cuh"
#include "sq_trace_dev.cuh"

namespace {

using namespace sq;

constexpr int kPacketStack = 128;  // the reference's packet stack (src/tracer.cpp:94)


// traverse_packet_stack from nodes [index, index + count) for the packet of
// lanes `pmask` (all of which call this together): returns the packet's box
// test count; *fault is set on a stack overflow or an index past the array.
__device__ uint32_t packet_tests(const Node* __restrict__ nodes, uint32_t nn, uint32_t index, uint32_t count,
                                 const float* o, const float* inv, uint32_t pmask, bool* fault)
{
    uint32_t st_i[kPacketStack], st_c[kPacketStack];
    int sp = 1;
    uint32_t tests = 0;
    st_i[0] = index;
    st_c[0] = count;
    while (sp > 0) {
        --sp;
        const uint32_t bi = st_i[sp], bc = st_c[sp];
        if ((uint64_t)bi + bc > nn) { *fault = true; break; }
        for (uint32_t c = 0; c < bc; ++c) {
            const NodeRec nd = load_node(nodes, bi + c);
            const bool hit = box_ref(nd, o, inv, 10000.0f);
            const bool any = __ballot_sync(pmask, hit) != 0u;
            tests++;
            if (any && !node_is_leaf(nd.cf)) {
                if (sp >= kPacketStack) { *fault = true; return tests; }
                st_i[sp] = nd.child;
                st_c[sp] = node_count(nd.cf);
                sp++;
            }
        }
    }
    return tests;
}

template <int K>
__global__ void __launch_bounds__(128) k_trace_packet(const sqk::TraceArgs a)
{
    constexpr int KX = (K == 1 || K == 2) ? 1 : 2;  // floor(sqrt(k))
    constexpr int KY = K / KX;
    constexpr int PPW = 32 / K;  // packets per warp
    const int lane = (int)(threadIdx.x & 31u);
    const int m = lane % K;      // ray of the packet (row order in the block)
    const uint32_t pmask = (K == 32 ? 0xFFFFFFFFu : ((1u << K) - 1u)) << (lane - m);
    const uint32_t bw = a.width / KX;
    const uint32_t total = bw * (a.height / KY);
    uint64_t tests_sum = 0;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(a.work, (uint32_t)PPW);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= total) break;
        const uint32_t pk = base + (uint32_t)(lane / K);
        if (pk < total) {
            const uint32_t x = (pk % bw) * KX + (uint32_t)(m % KX);
            const uint32_t y = (pk / bw) * KY + (uint32_t)(m / KX);
            Ray r;
            gen_reference_camera(x, y, a.width, a.height, a.cam, r);
            const float inv[3] = {1.0f / r.d[0], 1.0f / r.d[1], 1.0f / r.d[2]};
            bool fault = false;
            const uint32_t t = packet_tests(a.nodes, a.node_count, a.root, 1u, r.o, inv, pmask, &fault);
            if (fault && m == 0) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
            write_heat(a.heat + 3ull * ((size_t)y * a.width + x), (float)t / (float)K, a.heat_ramp);
            if (m == 0) tests_sum += t;
        }
    }
    if (a.stats) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tests_sum += __shfl_xor_sync(0xFFFFFFFFu, tests_sum, o);
        if (lane == 0) atomicAdd(a.stats, (unsigned long long)tests_sum);
    }
}

// morton_lut (src/tracer.cpp:18-23): k with bits 1 and 2 exchanged
__device__ __forceinline__ uint32_t bundle_lut(uint32_t k) { return (k & ~6u) | ((k & 2u) << 1) | ((k & 4u) >> 1); }

// intersect_bundle_aabb (src/tracer.h:37-80)
__device__ __forceinline__ void bundle_box(const NodeRec& nd, const float* pos, const float* imin, const float* imax,
                                           const float* imid, bool& any_hit, bool& mid_hit)
{
    float tmin_mid[3], tmin_any[3], tmax_mid[3], tmax_any[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float lo = nd.mn[k] - pos[k], hi = nd.mx[k] - pos[k];
        const float t1a = lo * imin[k], t1b = lo * imax[k], t2a = hi * imin[k], t2b = hi * imax[k];
        const float t1 = lo * imid[k], t2 = hi * imid[k];
        const float t1min = ref_min(t1a, t1b), t1max = simd_max(t1a, t1b);
        const float t2min = ref_min(t2a, t2b), t2max = simd_max(t2a, t2b);
        tmin_mid[k] = ref_min(t1, t2);
        tmin_any[k] = ref_min(t1min, t2min);
        tmax_mid[k] = simd_max(t1, t2);
        tmax_any[k] = simd_max(t1max, t2max);
    }
    const float front_mid = ref_max(ref_max(tmin_mid[0], tmin_mid[1]), tmin_mid[2]);
    const float front_any = ref_max(ref_max(tmin_any[0], tmin_any[1]), tmin_any[2]);
    const float back_mid = ref_min(ref_min(tmax_mid[0], tmax_mid[1]), tmax_mid[2]);
    const float back_any = ref_min(ref_min(tmax_any[0], tmax_any[1]), tmax_any[2]);
    mid_hit = back_mid >= front_mid;
    any_hit = back_any >= front_any;
}

template <int K>
__global__ void __launch_bounds__(128) k_trace_bundle(const sqk::TraceArgs a)
{
    constexpr int TW = (K == 16) ? 4 : 8;  // floor(sqrt(k))
    constexpr int TH = K / TW;
    constexpr int SLOTS = (K + 31) / 32;   // rays per lane
    const int lane = (int)(threadIdx.x & 31u);
    const uint32_t gmask = 0xFFu << (lane & 24);  // this lane's 8-lane group (one packet per slot)
    const uint32_t tiles_x = a.width / TW;
    const uint32_t total = tiles_x * (a.height / TH);
    uint64_t tests_sum = 0;
    for (;;) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(a.work, 1u);
        tile = __shfl_sync(0xFFFFFFFFu, tile, 0);
        if (tile >= total) break;
        const uint32_t i0 = (tile % tiles_x) * TW, j0 = (tile / tiles_x) * TH;
        // this lane's rays: r = lane + 32 * s
        float d[SLOTS][3], inv[SLOTS][3];
        uint32_t px[SLOTS];
        bool valid[SLOTS];
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) {
            const uint32_t r = (uint32_t)lane + 32u * (uint32_t)s;
            valid[s] = r < (uint32_t)K;
            const uint32_t v = bundle_lut(valid[s] ? r : 0u);
            const uint32_t x = i0 + v % TW, y = j0 + v / TW;
            Ray ray;
            gen_reference_camera(x, y, a.width, a.height, a.cam, ray);
#pragma unroll
            for (int c = 0; c < 3; ++c) { d[s][c] = ray.d[c]; inv[s][c] = 1.0f / ray.d[c]; }
            px[s] = y * a.width + x;
        }
        // the bundle's direction bounds, accumulated in ray order as the
        // reference does (src/tracer.cpp:331-336)
        float dmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, dmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int r = 0; r < K; ++r) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float v = __shfl_sync(0xFFFFFFFFu, d[0][c], r & 31);
                if (SLOTS > 1) {
                    const float v1 = __shfl_sync(0xFFFFFFFFu, d[SLOTS - 1][c], r & 31);
                    if (r >= 32) v = v1;
                }
                dmin[c] = ref_min(dmin[c], v);
                dmax[c] = ref_max(dmax[c], v);
            }
        }
        float imin[3], imax[3], imid[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            imin[c] = 1.0f / dmin[c];
            imax[c] = 1.0f / dmax[c];
            imid[c] = 1.0f / ((dmin[c] + dmax[c]) * 0.5f);
        }
        // the bundle traversal (the same on every lane)
        uint32_t btests = 0, ptests[SLOTS];
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) ptests[s] = 0;
        uint32_t st_i[kPacketStack], st_c[kPacketStack];
        int sp = 1;
        st_i[0] = a.root;
        st_c[0] = 1;
        bool fault = false;
        while (sp > 0 && !fault) {
            --sp;
            const uint32_t bi = st_i[sp], bc = st_c[sp];
            if ((uint64_t)bi + bc > a.node_count) { fault = true; break; }
            for (uint32_t c = 0; c < bc; ++c) {
                const NodeRec nd = load_node(a.nodes, bi + c);
                bool any_hit, mid_hit;
                bundle_box(nd, a.cam, imin, imax, imid, any_hit, mid_hit);
                btests++;
                if (mid_hit) {
                    if (!node_is_leaf(nd.cf)) {
                        if (sp >= kPacketStack) { fault = true; break; }
                        st_i[sp] = nd.child;
                        st_c[sp] = node_count(nd.cf);
                        sp++;
                    }
                } else if (any_hit) {
                    // each packet of 8 continues alone from this node
#pragma unroll
                    for (int s = 0; s < SLOTS; ++s) {
                        if (valid[s]) ptests[s] += packet_tests(a.nodes, a.node_count, bi + c, 1u, a.cam, inv[s],
                                                                gmask, &fault);
                    }
                }
            }
            fault = __any_sync(0xFFFFFFFFu, fault);
        }
        if (fault && lane == 0) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) {
            if (!valid[s]) continue;
            const float t = (float)btests / (float)K + (float)ptests[s] / 8.0f;
            write_heat(a.heat + 3ull * px[s], t, a.heat_ramp);
            if ((lane & 7) == 0) tests_sum += ptests[s];
        }
        if (lane == 0) tests_sum += btests;
    }
    if (a.stats) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tests_sum += __shfl_xor_sync(0xFFFFFFFFu, tests_sum, o);
        if (lane == 0) atomicAdd(a.stats, (unsigned long long)tests_sum);
    }
}

int sms() { return sm_count(); }

}  // namespace

namespace sqk {

bool coherent_shape_ok(uint32_t bundle, uint32_t k, uint32_t w, uint32_t h)
{
    if (bundle) {
        if (k != 16 && k != 64) return false;
        const uint32_t tw = k == 16 ? 4u : 8u;
        return w % tw == 0 && h % (k / tw) == 0;
    }
    if (k != 1 && k != 2 && k != 4 && k != 8) return false;
    const uint32_t kx = k <= 2 ? 1u : 2u;
    return w % kx == 0 && h % (k / kx) == 0;
}

void trace_coherent(const TraceArgs& a, uint32_t bundle, uint32_t k, cudaStream_t s)
{
    const uint32_t grid = (uint32_t)sms() * 8u;
    if (bundle) {
        if (k == 16) k_trace_bundle<16><<<grid, 128, 0, s>>>(a);
        else k_trace_bundle<64><<<grid, 128, 0, s>>>(a);
        return;
    }
    switch (k) {
    case 1: k_trace_packet<1><<<grid, 128, 0, s>>>(a); break;
    case 2: k_trace_packet<2><<<grid, 128, 0, s>>>(a); break;
    case 4: k_trace_packet<4><<<grid, 128, 0, s>>>(a); break;
    default: k_trace_packet<8><<<grid, 128, 0, s>>>(a); break;
    }
}

}  // namespace sqk
