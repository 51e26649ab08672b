// sq_trace.cu -- ray generation, BVH traversal and heatmap on the GPU.
//
// Replaces trace() / traverse() (src/tracer.cpp:47-65, 195-230) and the
// ray-box / ray-triangle tests (src/tracer.h:12-35, 82-116).
//
// Work distribution: persistent warps.  A warp takes the next batch of 32
// rays from a global counter (8x4 pixel tiles for camera rays, 32
// consecutive rays for explicit ones), traces them, writes the results and
// takes the next batch until the counter passes the end; the counter is
// never waited on.  Each lane runs a stack traversal over Node1 records:
//
//   SQ_TRACE_REF      the reference's semantics: every child box of every hit
//                     inner node is tested and counted, no ordering, no early
//                     exit, Moller-Trumbore hit flag (stack of node groups).
//   SQ_TRACE_CLOSEST  near-child order: all children boxes of a node are
//                     tested (and counted), hits are ordered by entry
//                     distance (ties: slot order), the nearest is visited
//                     next and the others are pushed; popped entries farther
//                     than the current hit are culled without a test; leaf
//                     records run the watertight triangle test (Woop, Benthin,
//                     Wald, JCGT 2013) with an FP64 recomputation only when an
//                     FP32 edge function is exactly zero.
//   SQ_TRACE_ANYHIT   as CLOSEST, stopping at the first accepted hit.
//
// The arithmetic is operation-for-operation that of oracle/sq_oracle.c
// (compiled with -fmad=false), so results are bit-identical to it.
#include "sq_common.cuh"
#include "sq_trace_dev.cuh"

namespace {

using namespace sq;

constexpr float kRobust = 0x1.000008p+0f;  // 1 + 2^-21 > 1 + 2*gamma(3)
constexpr int kStack = 64;

__device__ __forceinline__ void gen_pinhole(uint32_t x, uint32_t y, uint32_t w, uint32_t h, const float* b, Ray& r)
{
    float px = ((float)x + 0.5f) / (float)w;
    px = px * 2.0f;
    px = px - 1.0f;
    float py = ((float)y + 0.5f) / (float)h;
    py = py * 2.0f;
    py = py - 1.0f;
    px = px * b[12];
    py = py * b[13];
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float s = b[3 + k] + px * b[6 + k];
        d[k] = s + py * b[9 + k];
    }
    float l2 = d[0] * d[0] + d[1] * d[1];
    l2 = l2 + d[2] * d[2];
    const float len = sqrtf(l2);
    r.o[0] = b[0]; r.o[1] = b[1]; r.o[2] = b[2];
    r.d[0] = d[0] / len; r.d[1] = d[1] / len; r.d[2] = d[2] / len;
    r.tmin = 0.0f;
    r.tmax = FLT_MAX;
}

// intersect_ray_triangle<1> (src/tracer.h:82-116): hit flag only
__device__ __forceinline__ bool tri_ref(const float* __restrict__ tris, uint32_t id, const float* o, const float* d)
{
    float tv[9];
    load_tri(tris, id, tv);
    const float eps = 0.000000001f;
    float e1[3], e2[3], h[3], s[3], q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { e1[k] = tv[3 + k] - tv[k]; e2[k] = tv[6 + k] - tv[k]; }
    h[0] = d[1] * e2[2] - e2[1] * d[2];
    h[1] = d[2] * e2[0] - e2[2] * d[0];
    h[2] = d[0] * e2[1] - e2[0] * d[1];
    float a = e1[0] * h[0] + e1[1] * h[1];
    a = a + e1[2] * h[2];
    bool miss = (a > -eps) && (a < eps);
    const float f = 1.0f / a;
#pragma unroll
    for (int k = 0; k < 3; ++k) s[k] = o[k] - tv[k];
    float sh = s[0] * h[0] + s[1] * h[1];
    sh = sh + s[2] * h[2];
    const float u = f * sh;
    miss |= (u < 0.0f) || (u > 1.0f);
    q[0] = s[1] * e1[2] - e1[1] * s[2];
    q[1] = s[2] * e1[0] - e1[2] * s[0];
    q[2] = s[0] * e1[1] - e1[0] * s[1];
    float dq = d[0] * q[0] + d[1] * q[1];
    dq = dq + d[2] * q[2];
    const float v = f * dq;
    const float uv = u + v;
    miss |= (v < 0.0f) || (uv > 1.0f);
    float eq = e2[0] * q[0] + e2[1] * q[1];
    eq = eq + e2[2] * q[2];
    const float t = f * eq;
    return (!miss) && (t > eps);
}

struct RayPre {
    float o[3], inv[3], tmin, tmax;
    int kx, ky, kz;
    float sx, sy, sz;
};

__device__ __forceinline__ void ray_prepare(const Ray& r, RayPre& p)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) { p.o[k] = r.o[k]; p.inv[k] = 1.0f / r.d[k]; }
    p.tmin = r.tmin;
    p.tmax = r.tmax;
    const float ax = fabsf(r.d[0]), ay = fabsf(r.d[1]), az = fabsf(r.d[2]);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) { kz = 2; }
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    const float dkz = r.d[kz];
    if (dkz < 0.0f) { const int t = kx; kx = ky; ky = t; }
    p.kx = kx; p.ky = ky; p.kz = kz;
    p.sx = r.d[kx] / dkz;
    p.sy = r.d[ky] / dkz;
    p.sz = 1.0f / dkz;
}

__device__ __forceinline__ bool box_robust(const NodeRec& nd, const RayPre& r, float tclose, float& tn)
{
    const float t0x = (nd.mn[0] - r.o[0]) * r.inv[0];
    const float t1x = (nd.mx[0] - r.o[0]) * r.inv[0];
    const float t0y = (nd.mn[1] - r.o[1]) * r.inv[1];
    const float t1y = (nd.mx[1] - r.o[1]) * r.inv[1];
    const float t0z = (nd.mn[2] - r.o[2]) * r.inv[2];
    const float t1z = (nd.mx[2] - r.o[2]) * r.inv[2];
    const float n = fmaxf(fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z)), r.tmin);
    float f = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    f = f * kRobust;
    const float lim = tclose * kRobust;
    tn = n;
    return (n <= f) && (n <= lim);
}

__device__ __forceinline__ float sel3(const float* v, int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); }

__device__ __forceinline__ bool tri_watertight(const float* __restrict__ tris, uint32_t id, const RayPre& r, float tmax,
                                               float& tout)
{
    float tv[9];
    load_tri(tris, id, tv);
    float A[3], B[3], C[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { A[k] = tv[k] - r.o[k]; B[k] = tv[3 + k] - r.o[k]; C[k] = tv[6 + k] - r.o[k]; }
    const float Akz = sel3(A, r.kz), Bkz = sel3(B, r.kz), Ckz = sel3(C, r.kz);
    const float Ax = sel3(A, r.kx) - r.sx * Akz, Ay = sel3(A, r.ky) - r.sy * Akz;
    const float Bx = sel3(B, r.kx) - r.sx * Bkz, By = sel3(B, r.ky) - r.sy * Bkz;
    const float Cx = sel3(C, r.kx) - r.sx * Ckz, Cy = sel3(C, r.ky) - r.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        const double u = (double)Cx * (double)By - (double)Cy * (double)Bx;
        const double v = (double)Ax * (double)Cy - (double)Ay * (double)Cx;
        const double w = (double)Bx * (double)Ay - (double)By * (double)Ax;
        U = (float)u; V = (float)v; W = (float)w;
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V;
    det = det + W;
    if (det == 0.0f) return false;
    const float Az = r.sz * Akz, Bz = r.sz * Bkz, Cz = r.sz * Ckz;
    float T = U * Az + V * Bz;
    T = T + W * Cz;
    const float t = T / det;
    if (!(t >= r.tmin) || !(t <= tmax)) return false;
    tout = t;
    return true;
}

struct Result {
    uint32_t id;
    float t;
    uint32_t tests;
    uint32_t tri_tests;
    bool overflow;
    bool bad;  // an index outside the node or triangle array
};

// traverse(hierarchy, index, count, ray, attributes) (src/tracer.cpp:47-65)
// from the node group [root, root + group): every node of the group is
// tested in turn, then the groups of the hit inner nodes, depth first.
__device__ Result trace_ref(const Node* __restrict__ nodes, uint32_t nn, uint32_t nt, uint32_t root,
                            const float* __restrict__ tris, const Ray& r, uint32_t group = 1u)
{
    float inv[3] = {1.0f / r.d[0], 1.0f / r.d[1], 1.0f / r.d[2]};
    uint32_t st_child[kStack], st_count[kStack];
    int sp = 0;
    uint32_t cnt = 0, tcnt = 0;
    bool hit = false, overflow = false;
    bool bad = false;
    uint32_t gidx = root, gcnt = group;
    for (;;) {
        if ((uint64_t)gidx + gcnt > nn) { bad = true; break; }
        for (uint32_t i = 0; i < gcnt; ++i) {
            const NodeRec nd = load_node(nodes, gidx + i);
            cnt++;
            if (box_ref(nd, r.o, inv, r.tmax)) {
                if (node_is_leaf(nd.cf)) {
                    const uint32_t c = node_count(nd.cf);
                    if ((uint64_t)nd.child + c > nt) { bad = true; break; }
                    for (uint32_t k = 0; k < c; ++k) hit |= tri_ref(tris, nd.child + k, r.o, r.d);
                    tcnt += c;
                } else {
                    if (sp >= kStack) { overflow = true; break; }
                    st_child[sp] = nd.child;
                    st_count[sp] = node_count(nd.cf);
                    sp++;
                }
            }
        }
        if (overflow || bad || sp == 0) break;
        --sp;
        gidx = st_child[sp];
        gcnt = st_count[sp];
    }
    Result res;
    res.id = hit ? 0u : kNoHit;
    res.t = 0.0f;
    res.tests = cnt;
    res.tri_tests = tcnt;
    res.overflow = overflow;
    res.bad = bad;
    return res;
}

// One ray's closest-hit (or any-hit) traversal, resumable one inner node at
// a time so that a warp can refill a finished lane with a new ray while the
// others continue.  Stack entries: node index, or (triangle index |
// 0x80000000) for a leaf record whose triangle is still to be tested.
struct Lane2 {
    RayPre rp;
    float best_t;
    uint32_t best;
    uint32_t cnt, tcnt;  // box tests, triangle tests
    uint32_t cur;        // inner node to visit next; kNoHit when the ray is done
    int sp;
    bool overflow, bad;
};

template <bool ANY>
__device__ __forceinline__ bool lane2_tri(Lane2& L, const float* __restrict__ tris, uint32_t tri)
{
    float t;
    L.tcnt++;
    if (tri_watertight(tris, tri, L.rp, L.best_t, t)) {
        if (t < L.best_t || (t == L.best_t && tri < L.best)) { L.best_t = t; L.best = tri; }
        if (ANY) return true;
    }
    return false;
}

// The root: its box test, and the triangles of a root that is a leaf record.
template <bool ANY>
__device__ __forceinline__ void lane2_start(Lane2& L, const Node* __restrict__ nodes, uint32_t nn, uint32_t nt,
                                            uint32_t root, const float* __restrict__ tris, const Ray& ray)
{
    ray_prepare(ray, L.rp);
    L.best_t = L.rp.tmax;
    L.best = kNoHit;
    L.cnt = 1;
    L.tcnt = 0;
    L.sp = 0;
    L.overflow = false;
    L.bad = false;
    L.cur = kNoHit;
    float tn;
    if (root >= nn) { L.bad = true; return; }
    const NodeRec rn = load_node(nodes, root);
    if (!box_robust(rn, L.rp, L.best_t, tn)) return;
    if (!node_is_leaf(rn.cf)) { L.cur = root; return; }
    const uint32_t c = node_count(rn.cf);
    if ((uint64_t)rn.child + c > nt) { L.bad = true; return; }
    for (uint32_t k = 0; k < c; ++k)
        if (lane2_tri<ANY>(L, tris, rn.child + k)) return;
}

// Visit L.cur (an inner node that passed its box test and the cull test):
// test all its children's boxes, order the hits by entry distance (ties:
// slot order), push them, then pop until an inner node survives the cull
// test, testing leaf triangles on the way.  Leaves L.cur at that node, or at
// kNoHit when the ray is done.
template <bool ANY>
__device__ __forceinline__ void visit2(Lane2& L, const Node* __restrict__ nodes, uint32_t nn, uint32_t nt,
                                       const float* __restrict__ tris, uint32_t* st_node, float* st_tn)
{
    const NodeRec nd = load_node(nodes, L.cur);
    L.cur = kNoHit;
    const uint32_t c = node_count(nd.cf);
    if ((uint64_t)nd.child + c > nn) { L.bad = true; return; }
    uint32_t hn[8];
    float ht[8];
    int nh = 0;
    for (uint32_t i = 0; i < c; ++i) {
        const NodeRec ch = load_node(nodes, nd.child + i);
        L.cnt++;
        float t;
        if (box_robust(ch, L.rp, L.best_t, t)) {
            if (nh >= 8) { L.overflow = true; return; }
            if (node_is_leaf(ch.cf) && (uint64_t)ch.child + node_count(ch.cf) > nt) { L.bad = true; return; }
            const uint32_t ent = (node_is_leaf(ch.cf) && node_count(ch.cf) == 1u) ? (ch.child | 0x80000000u)
                                                                                  : (nd.child + i);
            // insertion by (tn, slot): equal distances keep slot order
            int b = nh - 1;
            while (b >= 0 && ht[b] > t) { hn[b + 1] = hn[b]; ht[b + 1] = ht[b]; --b; }
            hn[b + 1] = ent;
            ht[b + 1] = t;
            nh++;
        }
    }
    if (L.sp + nh > kStack) { L.overflow = true; return; }
    for (int a = nh - 1; a >= 0; --a) { st_node[L.sp] = hn[a]; st_tn[L.sp] = ht[a]; L.sp++; }
    while (L.sp > 0) {
        --L.sp;
        const uint32_t e = st_node[L.sp];
        if (st_tn[L.sp] > L.best_t * kRobust) continue;
        if (e & 0x80000000u) {
            if (lane2_tri<ANY>(L, tris, e & 0x7FFFFFFFu)) return;
            continue;
        }
        const NodeRec lr = load_node(nodes, e);
        if (node_is_leaf(lr.cf)) {
            // leaf record holding several triangles
            const uint32_t lc = node_count(lr.cf);
            for (uint32_t k = 0; k < lc; ++k)
                if (lane2_tri<ANY>(L, tris, lr.child + k)) return;
            continue;
        }
        L.cur = e;
        return;
    }
}

__device__ __forceinline__ Result lane2_result(const Lane2& L)
{
    Result res;
    res.id = L.best;
    res.t = (L.best == kNoHit) ? 0.0f : L.best_t;
    res.tests = L.cnt;
    res.tri_tests = L.tcnt;
    res.overflow = L.overflow;
    res.bad = L.bad;
    return res;
}

// One ray traced to the end (the tiles kernels): the same traversal as
// lane2_start + visit2 above, written as one loop, which the compiler fits
// in fewer registers (48 against 56) -- the per-lane refill kernel needs the
// resumable form, the tiles kernels do not.  The tests compare the two
// schedules ray for ray (ids, t and box-test counts).
template <bool ANY>
__device__ Result trace_closest(const Node* __restrict__ nodes, uint32_t nn, uint32_t nt, uint32_t root,
                                const float* __restrict__ tris, const Ray& ray)
{
    RayPre rp;
    ray_prepare(ray, rp);
    float best_t = rp.tmax;
    uint32_t best = kNoHit;
    uint32_t cnt = 1, tcnt = 0;
    bool overflow = false, bad = false;
    uint32_t st_node[kStack];
    float st_tn[kStack];
    int sp = 0;
    float tn;
    uint32_t cur = 0;
    bool have = false;
    if (root >= nn) bad = true;
    else {
        const NodeRec rn = load_node(nodes, root);
        if (box_robust(rn, rp, best_t, tn)) {
            if (node_is_leaf(rn.cf)) {
                // a leaf root record: test its triangles
                const uint32_t c = node_count(rn.cf);
                if ((uint64_t)rn.child + c > nt) bad = true;
                for (uint32_t k = 0; k < c && !bad; ++k) {
                    float t;
                    tcnt++;
                    if (tri_watertight(tris, rn.child + k, rp, best_t, t)) {
                        if (t < best_t || (t == best_t && rn.child + k < best)) { best_t = t; best = rn.child + k; }
                        if (ANY) break;
                    }
                }
            } else {
                cur = root;
                have = true;
            }
        }
    }
    while (have) {
        // cur is an inner node that passed its box test and the cull test
        const NodeRec nd = load_node(nodes, cur);
        const uint32_t c = node_count(nd.cf);
        if ((uint64_t)nd.child + c > nn) { bad = true; break; }
        uint32_t hn[8];
        float ht[8];
        int nh = 0;
        for (uint32_t i = 0; i < c; ++i) {
            const NodeRec ch = load_node(nodes, nd.child + i);
            cnt++;
            float t;
            if (box_robust(ch, rp, best_t, t)) {
                if (nh >= 8) { overflow = true; break; }
                if (node_is_leaf(ch.cf) && (uint64_t)ch.child + node_count(ch.cf) > nt) { bad = true; break; }
                const uint32_t ent = (node_is_leaf(ch.cf) && node_count(ch.cf) == 1u) ? (ch.child | 0x80000000u)
                                                                                      : (nd.child + i);
                // insertion by (tn, slot): equal distances keep slot order
                int b = nh - 1;
                while (b >= 0 && ht[b] > t) { hn[b + 1] = hn[b]; ht[b + 1] = ht[b]; --b; }
                hn[b + 1] = ent;
                ht[b + 1] = t;
                nh++;
            }
        }
        if (overflow || bad) break;
        if (sp + nh > kStack) { overflow = true; break; }
        for (int a = nh - 1; a >= 0; --a) { st_node[sp] = hn[a]; st_tn[sp] = ht[a]; sp++; }
        // pop until an inner node survives the cull test
        have = false;
        bool done = false;
        while (sp > 0) {
            --sp;
            const uint32_t e = st_node[sp];
            if (st_tn[sp] > best_t * kRobust) continue;
            if (e & 0x80000000u) {
                const uint32_t tri = e & 0x7FFFFFFFu;
                float t;
                tcnt++;
                if (tri_watertight(tris, tri, rp, best_t, t)) {
                    if (t < best_t || (t == best_t && tri < best)) { best_t = t; best = tri; }
                    if (ANY) { done = true; break; }
                }
                continue;
            }
            {
                const NodeRec lr = load_node(nodes, e);
                if (node_is_leaf(lr.cf)) {
                    // leaf record holding several triangles
                    const uint32_t lc = node_count(lr.cf);
                    for (uint32_t k = 0; k < lc; ++k) {
                        float t;
                        const uint32_t tri = lr.child + k;
                        tcnt++;
                        if (tri_watertight(tris, tri, rp, best_t, t)) {
                            if (t < best_t || (t == best_t && tri < best)) { best_t = t; best = tri; }
                            if (ANY) { done = true; break; }
                        }
                    }
                    if (done) break;
                    continue;
                }
            }
            cur = e;
            have = true;
            break;
        }
        if (done) break;
    }
    Result res;
    res.id = best;
    res.t = (best == kNoHit) ? 0.0f : best_t;
    res.tests = cnt;
    res.tri_tests = tcnt;
    res.overflow = overflow;
    res.bad = bad;
    return res;
}


template <int MODE>
__global__ void __launch_bounds__(128) k_trace(const sqk::TraceArgs a, uint32_t batches)
{
    const uint32_t lane = threadIdx.x & 31u;
    const bool camera = a.ray_kind != SQ_RAYS_EXPLICIT;
    const uint32_t tiles_x = (a.width + 7u) >> 3;
    __shared__ WarpStats s_stats[4];
    WarpStats& ws = s_stats[threadIdx.x >> 5];
    ws.reset(lane);
    for (;;) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(a.work, 1u);
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (b >= batches) break;
        Ray r;
        uint32_t rid = 0;
        bool active;
        if (camera) {
            const uint32_t x = (b % tiles_x) * 8u + (lane & 7u);
            const uint32_t y = (b / tiles_x) * 4u + (lane >> 3);
            active = x < a.width && y < a.height;
            rid = y * a.width + x;
            if (active) {
                if (a.ray_kind == SQ_RAYS_REFERENCE_CAMERA) gen_reference_camera(x, y, a.width, a.height, a.cam, r);
                else gen_pinhole(x, y, a.width, a.height, a.cam, r);
            }
        } else {
            rid = b * 32u + lane;
            active = rid < a.ray_count;
            if (active) {
                const float4* p = reinterpret_cast<const float4*>(a.rays) + 2ull * rid;
                const float4 x0 = __ldg(p), x1 = __ldg(p + 1);
                r.o[0] = x0.x; r.o[1] = x0.y; r.o[2] = x0.z; r.tmin = x0.w;
                r.d[0] = x1.x; r.d[1] = x1.y; r.d[2] = x1.z; r.tmax = x1.w;
            }
        }
        Result res;
        res.tests = 0;
        res.tri_tests = 0;
        if (active) {
            if (MODE == SQ_TRACE_REF) res = trace_ref(a.nodes, a.node_count, a.tri_count, a.root, a.tris, r,
                                                      a.root_group);
            else res = trace_closest<MODE == SQ_TRACE_ANYHIT>(a.nodes, a.node_count, a.tri_count, a.root, a.tris, r);
            if (res.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
            if (res.bad) raise_error(a.err, SQ_DEVERR_TOPOLOGY);
        }
        if (a.stats) {
            // requested bytes: ray in (explicit rays), hit record + heatmap out,
            // 32 B per node record tested, 36 B per triangle tested
            unsigned long long bt = res.tests, tt = res.tri_tests;
            unsigned long long by = active ? (unsigned long long)(camera ? 0u : 32u) + (a.hits ? 12u : 0u) +
                                                 (a.heat ? 3u : 0u) + 32ull * res.tests + 36ull * res.tri_tests
                                           : 0ull;
            ws.add(lane, bt, tt, by, bt);
        }
        if (!active) continue;
        if (a.hits) {
            uint32_t* h = reinterpret_cast<uint32_t*>(a.hits) + 3ull * rid;
            h[0] = res.id;
            h[1] = __float_as_uint(res.t);
            h[2] = res.tests;
        }
        if (a.heat) {
            write_heat(a.heat + 3ull * rid, (float)res.tests, a.heat_ramp);
        }
    }
    if (a.stats) ws.flush(lane, a.stats);
}

// Per-lane ray refill (closest / any-hit): a lane whose ray has finished
// takes the next ray at once (one atomic per warp for all lanes that need
// one) and every iteration visits one node per lane, so a warp does not
// wait for its slowest ray.  Each ray is traced with the same arithmetic and
// visit order as in k_trace, so results are identical; only the assignment
// of rays to lanes changes.  Ray g is explicit ray g, or pixel (g mod 32) of
// 8x4 tile g / 32 for camera rays.
template <int MODE>
__global__ void __launch_bounds__(128) k_trace_refill(const sqk::TraceArgs a, uint32_t total)
{
    constexpr bool ANY = MODE == SQ_TRACE_ANYHIT;
    const uint32_t lane = threadIdx.x & 31u;
    const bool camera = a.ray_kind != SQ_RAYS_EXPLICIT;
    const uint32_t tiles_x = (a.width + 7u) >> 3;
    uint32_t st_node[kStack];
    float st_tn[kStack];
    Lane2 L;
    L.cur = kNoHit;
    bool has = false, exhausted = false;
    uint32_t rid = 0;
    unsigned long long s_bt = 0, s_tt = 0, s_by = 0;
    for (;;) {
        const uint32_t need = __ballot_sync(0xFFFFFFFFu, !has && !exhausted);
        if (need) {
            const uint32_t leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(a.work, __popc(need));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (!has && !exhausted) {
                const uint32_t g = base + __popc(need & ((1u << lane) - 1u));
                if (g >= total) {
                    exhausted = true;
                } else {
                    Ray r;
                    bool ok;
                    if (camera) {
                        const uint32_t b = g >> 5, l = g & 31u;
                        const uint32_t x = (b % tiles_x) * 8u + (l & 7u);
                        const uint32_t y = (b / tiles_x) * 4u + (l >> 3);
                        ok = x < a.width && y < a.height;
                        rid = y * a.width + x;
                        if (ok) {
                            if (a.ray_kind == SQ_RAYS_REFERENCE_CAMERA) gen_reference_camera(x, y, a.width, a.height, a.cam, r);
                            else gen_pinhole(x, y, a.width, a.height, a.cam, r);
                        }
                    } else {
                        rid = g;
                        ok = true;
                        const float4* p = reinterpret_cast<const float4*>(a.rays) + 2ull * rid;
                        const float4 x0 = __ldg(p), x1 = __ldg(p + 1);
                        r.o[0] = x0.x; r.o[1] = x0.y; r.o[2] = x0.z; r.tmin = x0.w;
                        r.d[0] = x1.x; r.d[1] = x1.y; r.d[2] = x1.z; r.tmax = x1.w;
                    }
                    if (ok) {
                        lane2_start<ANY>(L, a.nodes, a.node_count, a.tri_count, a.root, a.tris, r);
                        has = true;
                    }
                }
            }
        }
        const uint32_t busy = __ballot_sync(0xFFFFFFFFu, has);
        if (!busy) {
            if (__all_sync(0xFFFFFFFFu, exhausted)) break;
            continue;
        }
        if (has) {
            if (L.cur != kNoHit) visit2<ANY>(L, a.nodes, a.node_count, a.tri_count, a.tris, st_node, st_tn);
            if (L.cur == kNoHit) {
                has = false;
                const Result res = lane2_result(L);
                if (res.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
                if (res.bad) raise_error(a.err, SQ_DEVERR_TOPOLOGY);
                if (a.stats) {
                    s_bt += res.tests;
                    s_tt += res.tri_tests;
                    s_by += (camera ? 0u : 32u) + (a.hits ? 12u : 0u) + (a.heat ? 3u : 0u) + 32ull * res.tests +
                            36ull * res.tri_tests;
                }
                if (a.hits) {
                    uint32_t* h = reinterpret_cast<uint32_t*>(a.hits) + 3ull * rid;
                    h[0] = res.id;
                    h[1] = __float_as_uint(res.t);
                    h[2] = res.tests;
                }
                if (a.heat) {
                    write_heat(a.heat + 3ull * rid, (float)res.tests, a.heat_ramp);
                }
            }
        }
    }
    if (a.stats) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s_bt += __shfl_xor_sync(0xFFFFFFFFu, s_bt, o);
            s_tt += __shfl_xor_sync(0xFFFFFFFFu, s_tt, o);
            s_by += __shfl_xor_sync(0xFFFFFFFFu, s_by, o);
        }
        if (lane == 0) {
            atomicAdd(a.stats, s_bt); atomicAdd(a.stats + 1, s_tt); atomicAdd(a.stats + 2, s_by); atomicAdd(a.stats + 3, s_bt);
        }
    }
}

template <int MODE>
void launch(const sqk::TraceArgs& a, cudaStream_t s)
{
    uint32_t batches;
    if (a.ray_kind == SQ_RAYS_EXPLICIT) batches = (a.ray_count + 31u) / 32u;
    else batches = ((a.width + 7u) / 8u) * ((a.height + 3u) / 4u);
    if (batches == 0) return;
    const bool refill = a.refill && MODE != SQ_TRACE_REF;
    static PerDevice<std::array<int, 2>> cache;
    const std::array<int, 2> per_sm = cache.get([] {
        return std::array<int, 2>{blocks_per_sm(k_trace<MODE>, 128),
                                  blocks_per_sm(k_trace_refill<MODE == SQ_TRACE_REF ? SQ_TRACE_CLOSEST : MODE>, 128)};
    });
    uint32_t grid = (uint32_t)(per_sm[refill ? 1 : 0] * sm_count());
    const uint32_t need = (batches + 3u) / 4u;
    if (grid > need) grid = need;
    if (refill) {
        const uint32_t total = a.ray_kind == SQ_RAYS_EXPLICIT ? a.ray_count : batches * 32u;
        k_trace_refill<MODE == SQ_TRACE_REF ? SQ_TRACE_CLOSEST : MODE><<<grid, 128, 0, s>>>(a, total);
    } else {
        k_trace<MODE><<<grid, 128, 0, s>>>(a, batches);
    }
}

// Batched trace: warps take 32-ray batches of any job (a mesh's BVH and its
// ray tile) from one counter; each job names its root and ray source.
template <int MODE>
__global__ void __launch_bounds__(256) k_trace_batch(const sqk::BatchTraceArgs a)
{
    const uint32_t lane = threadIdx.x & 31u;
    __shared__ WarpStats s_stats[8];
    WarpStats& ws = s_stats[threadIdx.x >> 5];
    ws.reset(lane);
    for (;;) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(a.work, 1u);
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (b >= a.total_batches) break;
        const uint32_t j = find_job(a.jobs, a.njobs, b);
        const sqk::BatchJob& job = a.jobs[j];
        const uint32_t lb = b - job.batch_begin;
        Ray r;
        uint32_t rid = 0;
        bool active;
        if (job.ray_kind != SQ_RAYS_EXPLICIT) {
            const uint32_t tiles_x = (job.width + 7u) >> 3;
            const uint32_t x = (lb % tiles_x) * 8u + (lane & 7u);
            const uint32_t y = (lb / tiles_x) * 4u + (lane >> 3);
            active = x < job.width && y < job.height;
            rid = y * job.width + x;
            if (active) {
                if (job.ray_kind == SQ_RAYS_REFERENCE_CAMERA) gen_reference_camera(x, y, job.width, job.height, job.cam, r);
                else gen_pinhole(x, y, job.width, job.height, job.cam, r);
            }
        } else {
            rid = lb * 32u + lane;
            active = rid < job.ray_count;
            if (active) {
                const float4* p = reinterpret_cast<const float4*>(job.rays ? job.rays : a.rays) + 2ull * (job.ray_offset + rid);
                const float4 x0 = __ldg(p), x1 = __ldg(p + 1);
                r.o[0] = x0.x; r.o[1] = x0.y; r.o[2] = x0.z; r.tmin = x0.w;
                r.d[0] = x1.x; r.d[1] = x1.y; r.d[2] = x1.z; r.tmax = x1.w;
            }
        }
        Result res;
        res.tests = 0;
        res.tri_tests = 0;
        if (active) {
            if (MODE == SQ_TRACE_REF) res = trace_ref(a.nodes, a.node_count, a.tri_count, job.root, a.tris, r);
            else res = trace_closest<MODE == SQ_TRACE_ANYHIT>(a.nodes, a.node_count, a.tri_count, job.root, a.tris, r);
            if (res.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
            if (res.bad) raise_error(a.err, SQ_DEVERR_TOPOLOGY);
            if (MODE != SQ_TRACE_REF && res.id != kNoHit) res.id -= job.tri_offset;
        }
        if (a.stats) {
            unsigned long long bt = res.tests, tt = res.tri_tests;
            unsigned long long by = active ? (unsigned long long)(job.ray_kind == SQ_RAYS_EXPLICIT ? 32u : 0u) +
                                                 (a.hits ? 12u : 0u) + (a.heat ? 3u : 0u) + 32ull * res.tests +
                                                 36ull * res.tri_tests
                                           : 0ull;
            ws.add(lane, bt, tt, by, bt);
        }
        if (!active) continue;
        const uint64_t out = (uint64_t)job.out_offset + rid;
        if (a.hits) {
            uint32_t* h = reinterpret_cast<uint32_t*>(a.hits) + 3ull * out;
            h[0] = res.id;
            h[1] = __float_as_uint(res.t);
            h[2] = res.tests;
        }
        if (a.heat) {
            write_heat(a.heat + 3ull * out, (float)res.tests, a.heat_ramp);
        }
    }
    if (a.stats) ws.flush(lane, a.stats);
}

// Batched trace with per-lane ray refill (closest / any-hit): as
// k_trace_refill over the job table's ray slots (slot g: lane g mod 32 of
// the job's 32-ray batch g / 32); a lane keeps its current job's batch range
// and searches the table only when a slot leaves it.
template <int MODE>
__global__ void __launch_bounds__(256) k_trace_batch_refill(const sqk::BatchTraceArgs a)
{
    constexpr bool ANY = MODE == SQ_TRACE_ANYHIT;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t total = a.total_batches * 32u;
    uint32_t st_node[kStack];
    float st_tn[kStack];
    Lane2 L;
    L.cur = kNoHit;
    bool has = false, exhausted = false, explicit_rays = false;
    uint32_t out = 0, tri_offset = 0;
    uint32_t cj = 0, jlo = 1, jhi = 0;
    unsigned long long s_bt = 0, s_tt = 0, s_by = 0;
    for (;;) {
        const uint32_t need = __ballot_sync(0xFFFFFFFFu, !has && !exhausted);
        if (need) {
            const uint32_t leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(a.work, __popc(need));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (!has && !exhausted) {
                const uint32_t g = base + __popc(need & ((1u << lane) - 1u));
                if (g >= total) {
                    exhausted = true;
                } else {
                    const uint32_t b = g >> 5, l = g & 31u;
                    if (b < jlo || b >= jhi) {
                        cj = find_job(a.jobs, a.njobs, b);
                        jlo = __ldg(&a.jobs[cj].batch_begin);
                        jhi = cj + 1 < a.njobs ? __ldg(&a.jobs[cj + 1].batch_begin) : a.total_batches;
                    }
                    const sqk::BatchJob& job = a.jobs[cj];
                    const uint32_t lb = b - jlo;
                    Ray r;
                    bool ok;
                    uint32_t rid;
                    explicit_rays = job.ray_kind == SQ_RAYS_EXPLICIT;
                    if (!explicit_rays) {
                        const uint32_t tiles_x = (job.width + 7u) >> 3;
                        const uint32_t x = (lb % tiles_x) * 8u + (l & 7u);
                        const uint32_t y = (lb / tiles_x) * 4u + (l >> 3);
                        ok = x < job.width && y < job.height;
                        rid = y * job.width + x;
                        if (ok) {
                            if (job.ray_kind == SQ_RAYS_REFERENCE_CAMERA) gen_reference_camera(x, y, job.width, job.height, job.cam, r);
                            else gen_pinhole(x, y, job.width, job.height, job.cam, r);
                        }
                    } else {
                        rid = lb * 32u + l;
                        ok = rid < job.ray_count;
                        if (ok) {
                            const float4* p = reinterpret_cast<const float4*>(job.rays ? job.rays : a.rays) +
                                              2ull * (job.ray_offset + rid);
                            const float4 x0 = __ldg(p), x1 = __ldg(p + 1);
                            r.o[0] = x0.x; r.o[1] = x0.y; r.o[2] = x0.z; r.tmin = x0.w;
                            r.d[0] = x1.x; r.d[1] = x1.y; r.d[2] = x1.z; r.tmax = x1.w;
                        }
                    }
                    if (ok) {
                        out = job.out_offset + rid;
                        tri_offset = job.tri_offset;
                        lane2_start<ANY>(L, a.nodes, a.node_count, a.tri_count, job.root, a.tris, r);
                        has = true;
                    }
                }
            }
        }
        const uint32_t busy = __ballot_sync(0xFFFFFFFFu, has);
        if (!busy) {
            if (__all_sync(0xFFFFFFFFu, exhausted)) break;
            continue;
        }
        if (has) {
            if (L.cur != kNoHit) visit2<ANY>(L, a.nodes, a.node_count, a.tri_count, a.tris, st_node, st_tn);
            if (L.cur == kNoHit) {
                has = false;
                Result res = lane2_result(L);
                if (res.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
                if (res.bad) raise_error(a.err, SQ_DEVERR_TOPOLOGY);
                if (res.id != kNoHit) res.id -= tri_offset;
                if (a.stats) {
                    s_bt += res.tests;
                    s_tt += res.tri_tests;
                    s_by += (explicit_rays ? 32u : 0u) + (a.hits ? 12u : 0u) + (a.heat ? 3u : 0u) +
                            32ull * res.tests + 36ull * res.tri_tests;
                }
                if (a.hits) {
                    uint32_t* h = reinterpret_cast<uint32_t*>(a.hits) + 3ull * out;
                    h[0] = res.id;
                    h[1] = __float_as_uint(res.t);
                    h[2] = res.tests;
                }
                if (a.heat) write_heat(a.heat + 3ull * out, (float)res.tests, a.heat_ramp);
            }
        }
    }
    if (a.stats) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s_bt += __shfl_xor_sync(0xFFFFFFFFu, s_bt, o);
            s_tt += __shfl_xor_sync(0xFFFFFFFFu, s_tt, o);
            s_by += __shfl_xor_sync(0xFFFFFFFFu, s_by, o);
        }
        if (lane == 0) {
            atomicAdd(a.stats, s_bt); atomicAdd(a.stats + 1, s_tt); atomicAdd(a.stats + 2, s_by); atomicAdd(a.stats + 3, s_bt);
        }
    }
}

template <int MODE>
void launch_batch(const sqk::BatchTraceArgs& a, int block, cudaStream_t s)
{
    if (a.total_batches == 0) return;
    constexpr int RM = MODE == SQ_TRACE_REF ? SQ_TRACE_CLOSEST : MODE;  // refill: closest / any-hit only
    static PerDevice<std::array<int, 6>> cache;
    const std::array<int, 6> per_sm = cache.get([] {
        return std::array<int, 6>{blocks_per_sm(k_trace_batch<MODE>, 64), blocks_per_sm(k_trace_batch<MODE>, 128),
                                  blocks_per_sm(k_trace_batch<MODE>, 256), blocks_per_sm(k_trace_batch_refill<RM>, 64),
                                  blocks_per_sm(k_trace_batch_refill<RM>, 128),
                                  blocks_per_sm(k_trace_batch_refill<RM>, 256)};
    });
    const bool refill = a.refill && MODE != SQ_TRACE_REF;
    const int bi = block <= 64 ? 0 : (block <= 128 ? 1 : 2);
    uint32_t grid = (uint32_t)(per_sm[(refill ? 3 : 0) + bi] * sm_count());
    const uint32_t need = (a.total_batches + (uint32_t)(block / 32) - 1) / (uint32_t)(block / 32);
    if (grid > need) grid = need;
    if (refill) k_trace_batch_refill<RM><<<grid, block, 0, s>>>(a);
    else k_trace_batch<MODE><<<grid, block, 0, s>>>(a);
}

}  // namespace

namespace sqk {

void trace_batch(const BatchTraceArgs& a, int block, cudaStream_t s)
{
    if (block != 64 && block != 128 && block != 256) block = 128;
    if (a.mode == SQ_TRACE_REF) launch_batch<SQ_TRACE_REF>(a, block, s);
    else if (a.mode == SQ_TRACE_CLOSEST) launch_batch<SQ_TRACE_CLOSEST>(a, block, s);
    else launch_batch<SQ_TRACE_ANYHIT>(a, block, s);
}

void trace(const TraceArgs& a, cudaStream_t s)
{
    if (a.mode == SQ_TRACE_REF) launch<SQ_TRACE_REF>(a, s);
    else if (a.mode == SQ_TRACE_CLOSEST) launch<SQ_TRACE_CLOSEST>(a, s);
    else launch<SQ_TRACE_ANYHIT>(a, s);
}

}  // namespace sqk
