// sq_bvh8_trace.cu -- traversal of the 8-wide quantised BVH (node layout in
// sq_bvh8_dev.cuh; built by sq_bvh8.cu).
//
// Traversal (closest / any-hit): the node's eight child boxes are decoded and
// tested with the same conservative slab test as the FP32 traversal; hits are
// ordered by entry distance; inner children are pushed, leaf children are
// pushed as triangle ranges; the nearest is taken next.  Because every
// quantised box contains its FP32 box and the slab test is monotone in the
// box, this traversal visits every triangle the FP32 2-wide traversal visits,
// so both report the same closest hit (id and t, same watertight test).
#include "sq_bvh8_dev.cuh"

#include <array>
#include <type_traits>

namespace {

using namespace sq;

constexpr float kRobust = 0x1.000008p+0f;  // same factor as the FP32 traversal
constexpr int kStack8 = 64;

// ---------------------------------------------------------------------------
// traversal

struct Ray8 {
    float o[3], d[3], tmin, tmax;
};

struct Pre8 {
    float o[3], inv[3], tmin, tmax;
    int kx, ky, kz;
    float sx, sy, sz;
};

__device__ __forceinline__ void prep8(const Ray8& r, Pre8& p)
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

__device__ __forceinline__ float sel3(const float* v, int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); }

// Camera rays, same arithmetic as the FP32 traversal: the reference camera
// (src/tracer.cpp:207-216) or the pinhole basis.
__device__ __forceinline__ void camera_ray8(uint32_t kind, uint32_t x, uint32_t y, uint32_t w, uint32_t h,
                                            const float* cam, Ray8& r)
{
    if (kind == SQ_RAYS_REFERENCE_CAMERA) {
        const float aspect = (float)w / (float)h;
        float nx = ((float)x + 0.5f) / (float)w;
        nx = nx * 2.0f;
        nx = nx - 1.0f;
        float ny = ((float)y + 0.5f) / (float)h;
        ny = ny * 2.0f;
        ny = ny - 1.0f;
        nx = nx * aspect;
        float l2 = nx * nx + ny * ny;
        l2 = l2 + 1.0f * 1.0f;
        const float len = sqrtf(l2);
        r.o[0] = cam[0]; r.o[1] = cam[1]; r.o[2] = cam[2];
        r.d[0] = nx / len; r.d[1] = ny / len; r.d[2] = 1.0f / len;
        r.tmin = 0.0f;
        r.tmax = 10000.0f;
        return;
    }
    float px = ((float)x + 0.5f) / (float)w;
    px = px * 2.0f;
    px = px - 1.0f;
    float py = ((float)y + 0.5f) / (float)h;
    py = py * 2.0f;
    py = py - 1.0f;
    px = px * cam[12];
    py = py * cam[13];
    float d[3];
    for (int k = 0; k < 3; ++k) {
        const float s = cam[3 + k] + px * cam[6 + k];
        d[k] = s + py * cam[9 + k];
    }
    float l2 = d[0] * d[0] + d[1] * d[1];
    l2 = l2 + d[2] * d[2];
    const float len = sqrtf(l2);
    r.o[0] = cam[0]; r.o[1] = cam[1]; r.o[2] = cam[2];
    r.d[0] = d[0] / len; r.d[1] = d[1] / len; r.d[2] = d[2] / len;
    r.tmin = 0.0f;
    r.tmax = FLT_MAX;
}

// watertight test (same operations as the FP32 traversal)
__device__ __forceinline__ bool tri8(const float4* __restrict__ t8, uint32_t k, const Pre8& r, float tmax, float& tout,
                                     uint32_t& id)
{
    const float4 a = __ldg(t8 + 3ull * k), b = __ldg(t8 + 3ull * k + 1), c = __ldg(t8 + 3ull * k + 2);
    id = __float_as_uint(a.w);
    float A[3] = {a.x - r.o[0], a.y - r.o[1], a.z - r.o[2]};
    float B[3] = {b.x - r.o[0], b.y - r.o[1], b.z - r.o[2]};
    float C[3] = {c.x - r.o[0], c.y - r.o[1], c.z - r.o[2]};
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


// Quantised coordinate j (0..3) of a packed word as an exact float: the byte
// is placed in the mantissa of 2^23 (one byte permute) and 2^23 subtracted.
__device__ __forceinline__ float qbyte(uint32_t word, uint32_t j)
{
    return __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7440u | j)) - 8388608.0f;
}

// A ray for which no slab distance can be NaN: finite origin and finite,
// non-zero reciprocal direction (so bound - origin is finite or +-inf and its
// product with the reciprocal is never 0 * inf).  For such a ray the near
// plane of each axis is known from the sign of the direction, and the
// near/far distances are exactly what the min/max form of the slab test
// computes (min(t0, t1) is t0 when the reciprocal is positive, because the
// rounded product is monotone in the bound); so the test can pick the near
// and far byte once per node instead of taking min and max per child.
__device__ __forceinline__ bool no_nan_slabs(const Pre8& r)
{
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) ok = ok && isfinite(r.o[a]) && isfinite(r.inv[a]) && r.inv[a] != 0.0f;
    return ok;
}

// Affine child-box distances.  For a NaN-free ray the distance to a child's
// plane on axis a is, in exact arithmetic,
//     (org + q * 2^e - o) * inv = q * A + C,  A = 2^e * inv,  C = (org - o) * inv,
// so each of a child's six planes costs one fma once A and C are known for
// the node.  A is exact (a power of two times inv).  The rounded results
// differ from the exact form (dequantise, subtract, multiply: three
// roundings), so the near distance is computed from C - E and the far from
// C + E, with the margin E = 2^-19 * M + 2^-125 where
//     M = (|org| + 255 * 2^e + |o| + 2^-126) * |inv|
// bounds every term whose rounding matters (|q A|, |C|, the plane and the
// slab distance themselves).  The worst case of the roundings sums to about
// 8 * 2^-24 * M (plus subnormal absolute errors well under 2^-125), so the
// affine near distance is never above, and the far never below, what the
// exact form computes for the same quantised box, which in turn is never
// tighter than the FP32 box.
//
// Two more terms are folded into the per-node constants:
//   - the byte enters as the float x = 1 + q * 2^-15 (one byte permute into
//     the mantissa), so t = x * A' + (C - A') with A' = 2^15 * A (exact).
//     C - A' is rounded down for the near constant and up for the far one,
//     which only widens the box (by at most 2^-8 of a quantisation step);
//   - the traversal's robust factor on the far distance (f * (1 + 2^-21))
//     becomes D = 2^-20 * (M + E) added to the far constant: every far
//     distance is at most M + E plus roundings, so D covers f * 2^-21 and
//     the rounding of the product with room to spare.  The far constant
//     takes E + D <= 1.5625 * 2^-19 * M + 2^-123 in one term.
// The test therefore passes for every child the exact test passes (it may
// pass a few more), and the hits are unchanged.  A node whose constants are
// not all finite (coordinates near FLT_MAX) uses the exact form.
__device__ __forceinline__ bool node_affine(const float* org, const float* sc, const Pre8& rp, float* A, float* Cn,
                                            float* Cf)
{
    float msum = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float A1 = sc[a] * rp.inv[a];
        const float C = (org[a] - rp.o[a]) * rp.inv[a];
        const float M = (fmaf(255.0f, sc[a], fabsf(org[a]) + fabsf(rp.o[a])) + 0x1p-126f) * fabsf(rp.inv[a]);
        const float E = fmaf(M, 0x1p-19f, 0x1p-125f);
        const float ED = fmaf(M, 0x1.9p-19f, 0x1p-123f);
        A[a] = A1 * 32768.0f;
        Cn[a] = __fsub_rd(C - E, A[a]);
        Cf[a] = __fsub_ru(__fadd_ru(C, ED), A[a]);
        // an infinite or NaN M, A or C reaches one of these two
        msum += fabsf(Cn[a]) + fabsf(Cf[a]);
    }
    return isfinite(msum);
}

// x = 1 + q * 2^-15 for byte j of a word of quantised planes
__device__ __forceinline__ float qunit(uint32_t word, uint32_t j)
{
    return __uint_as_float(__byte_perm(word, 0x3F800000u, 0x7604u | (j << 4)));
}

__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Sum of the 4-bit triangle counts of slots [0, k) of a node's count word.
__device__ __forceinline__ uint32_t slots_below(uint32_t counts, int k)
{
    const uint32_t x = k >= 8 ? counts : counts & ((1u << (4 * k)) - 1u);
    const uint32_t s = (x & 0x0F0F0F0Fu) + ((x >> 4) & 0x0F0F0F0Fu);
    return (s * 0x01010101u) >> 24;
}

// Stack entry of child slot k: an inner child's node index, or a leaf
// child's triangle range (bit 31, count in bits 27-30, first triangle).
// Computed only for children that pass their box test.
__device__ __forceinline__ uint32_t child_entry(uint32_t imask, uint32_t child_base, uint32_t counts, uint32_t tri_base,
                                                int k)
{
    if ((imask >> k) & 1u) return child_base + __popc(imask & ((1u << k) - 1u));
    return 0x80000000u | (((counts >> (4 * k)) & 0xFu) << 27) | (tri_base + slots_below(counts, k));
}

// Entry and exit distances of child slot k (word w = k / 4, byte j = k % 4).
// The affine form's exit already carries the robust factor; the exact forms
// apply it here.  PAIR: the near and far planes of an axis in one paired
// fp32 fma (fma.rn.f32x2: two independent IEEE fmas, one issue slot), which
// pays in the per-ray tiles loop; the refill loop keeps scalar fmas (the
// pairs raise its register count past its occupancy step).
template <bool AFF, bool SIGNED, bool PAIR = false>
__device__ __forceinline__ void child_span(const uint32_t* qa, const uint32_t* qb, int w, uint32_t j, const float* A,
                                           const float* Cn, const float* Cf, const float* sc, const float* org,
                                           const Pre8& rp, float& n, float& f)
{
    float ta[3], tb[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (AFF && PAIR) {
            unsigned long long X, AA, CC, R;
            asm("mov.b64 %0, {%1, %2};" : "=l"(X) : "f"(qunit(qa[a * 2 + w], j)), "f"(qunit(qb[a * 2 + w], j)));
            asm("mov.b64 %0, {%1, %2};" : "=l"(AA) : "f"(A[a]), "f"(A[a]));
            asm("mov.b64 %0, {%1, %2};" : "=l"(CC) : "f"(Cn[a]), "f"(Cf[a]));
            asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(R) : "l"(X), "l"(AA), "l"(CC));
            asm("mov.b64 {%0, %1}, %2;" : "=f"(ta[a]), "=f"(tb[a]) : "l"(R));
        } else if (AFF) {
            ta[a] = fmaf(qunit(qa[a * 2 + w], j), A[a], Cn[a]);
            tb[a] = fmaf(qunit(qb[a * 2 + w], j), A[a], Cf[a]);
        } else {
            const float ba = fmaf(qbyte(qa[a * 2 + w], j), sc[a], org[a]);
            const float bb = fmaf(qbyte(qb[a * 2 + w], j), sc[a], org[a]);
            ta[a] = (ba - rp.o[a]) * rp.inv[a];
            tb[a] = (bb - rp.o[a]) * rp.inv[a];
        }
    }
    if (AFF) {
        n = fmaxf(max3f(ta[0], ta[1], ta[2]), rp.tmin);
        f = min3f(tb[0], tb[1], tb[2]);
    } else if (SIGNED) {
        n = fmaxf(fmaxf(fmaxf(ta[0], ta[1]), ta[2]), rp.tmin);
        f = fminf(fminf(tb[0], tb[1]), tb[2]) * kRobust;
    } else {
        n = fmaxf(fmaxf(fmaxf(fminf(ta[0], tb[0]), fminf(ta[1], tb[1])), fminf(ta[2], tb[2])), rp.tmin);
        f = fminf(fminf(fmaxf(ta[0], tb[0]), fmaxf(ta[1], tb[1])), fmaxf(ta[2], tb[2])) * kRobust;
    }
}

struct Res8 {
    uint32_t id;
    float t;
    uint32_t tests, tri_tests, nodes;
    bool overflow;
};

// One ray from the root to the end: the nearest hit child is taken next,
// the other hits are pushed far to near (popped entries are culled against
// the current closest distance).
template <bool ANY, bool SIGNED>
__device__ Res8 trace8_impl(const Node8* __restrict__ nodes, uint32_t root, const float4* __restrict__ t8,
                            const Pre8& rp)
{
    float best_t = rp.tmax;
    uint32_t best = kNoHit;
    uint32_t tests = 0, ttests = 0, nvis = 0;
    bool overflow = false;
    uint32_t st_e[kStack8];
    float st_t[kStack8];
    int sp = 0;
    uint32_t cur = root;
    bool have = true;
    // SIGNED: which of the (lo, hi) word pairs holds the near plane, per axis
    const bool neg[3] = {rp.inv[0] < 0.0f, rp.inv[1] < 0.0f, rp.inv[2] < 0.0f};
    while (have) {
        const float4* p = reinterpret_cast<const float4*>(nodes + cur);
        const float4 w0 = __ldg(p), w1 = __ldg(p + 1), w2 = __ldg(p + 2), w3 = __ldg(p + 3), w4 = __ldg(p + 4);
        nvis++;
        const float org[3] = {w0.x, w0.y, w0.z};
        const uint32_t ei = __float_as_uint(w0.w);
        const float sc[3] = {pow2f((int)(ei & 0xFFu) - 127), pow2f((int)((ei >> 8) & 0xFFu) - 127),
                             pow2f((int)((ei >> 16) & 0xFFu) - 127)};
        const uint32_t imask = ei >> 24;
        const uint32_t child_base = __float_as_uint(w1.x), tri_base = __float_as_uint(w1.y);
        const uint32_t counts = __float_as_uint(w1.z), valid = __float_as_uint(w1.w);
        // q words: qlo x (2 words: slots 0-3, 4-7), qlo y, qlo z, qhi x, qhi y, qhi z
        const uint32_t q[12] = {__float_as_uint(w2.x), __float_as_uint(w2.y), __float_as_uint(w2.z), __float_as_uint(w2.w),
                                __float_as_uint(w3.x), __float_as_uint(w3.y), __float_as_uint(w3.z), __float_as_uint(w3.w),
                                __float_as_uint(w4.x), __float_as_uint(w4.y), __float_as_uint(w4.z), __float_as_uint(w4.w)};
        uint32_t qa[6], qb[6];  // SIGNED: near and far words; otherwise lo and hi
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                const uint32_t lo = q[a * 2 + w], hi = q[6 + a * 2 + w];
                qa[a * 2 + w] = (SIGNED && neg[a]) ? hi : lo;
                qb[a * 2 + w] = (SIGNED && neg[a]) ? lo : hi;
            }
        }
        uint32_t hn[8];
        float ht[8];
        int nh = 0;
        float A[3], Cn[3], Cf[3];
        const bool aff = SIGNED && node_affine(org, sc, rp, A, Cn, Cf);
        // the child loop, compiled once per distance form (branching per node,
        // not per child, keeps one form's registers live at a time).  Every
        // slot is tested without a branch (lanes at different nodes have
        // different valid masks); the valid bit joins the hit condition.
        auto scan = [&](auto form) {
            constexpr bool AFF = decltype(form)::value;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                {
                    float n, f;
                    child_span<AFF, SIGNED, true>(qa, qb, k >> 2, (uint32_t)(k & 3), A, Cn, Cf, sc, org, rp, n, f);
                    if (((valid >> k) & 1u) && n <= f && n <= best_t * kRobust) {
                        const uint32_t ent = child_entry(imask, child_base, counts, tri_base, k);
                        int b = nh - 1;
                        while (b >= 0 && ht[b] > n) { hn[b + 1] = hn[b]; ht[b + 1] = ht[b]; --b; }
                        hn[b + 1] = ent;
                        ht[b + 1] = n;
                        nh++;
                    }
                }
            }
        };
        tests += __popc(valid);
        if (aff) scan(std::true_type{});
        else scan(std::false_type{});
        if (sp + nh > kStack8) { overflow = true; break; }
        for (int a = nh - 1; a >= 0; --a) { st_e[sp] = hn[a]; st_t[sp] = ht[a]; sp++; }
        have = false;
        bool done = false;
        while (sp > 0) {
            --sp;
            const uint32_t e = st_e[sp];
            if (st_t[sp] > best_t * kRobust) continue;
            if (e & 0x80000000u) {
                const uint32_t cnt = (e >> 27) & 0xFu, first = e & 0x07FFFFFFu;
                for (uint32_t j = 0; j < cnt; ++j) {
                    float t;
                    uint32_t id;
                    ttests++;
                    if (tri8(t8, first + j, rp, best_t, t, id)) {
                        if (t < best_t || (t == best_t && id < best)) { best_t = t; best = id; }
                        if (ANY) { done = true; break; }
                    }
                }
                if (done) break;
                continue;
            }
            cur = e;
            have = true;
            break;
        }
        if (done) break;
    }
    Res8 r;
    r.id = best;
    r.t = best == kNoHit ? 0.0f : best_t;
    r.tests = tests;
    r.tri_tests = ttests;
    r.nodes = nvis;
    r.overflow = overflow;
    return r;
}

template <bool ANY>
__device__ Res8 trace8(const Node8* __restrict__ nodes, uint32_t root, const float4* __restrict__ t8, const Ray8& ray)
{
    Pre8 rp;
    prep8(ray, rp);
    if (no_nan_slabs(rp)) return trace8_impl<ANY, true>(nodes, root, t8, rp);
    return trace8_impl<ANY, false>(nodes, root, t8, rp);
}


// ---------------------------------------------------------------------------
// Persistent traversal kernels hand out rays in one of two ways (persistent
// threads, Aila and Laine, HPG 2009):
//   tiles    a warp takes a whole 32-ray batch (an 8x4 pixel tile of a
//            camera) and each lane runs its ray to the end (trace8); the
//            warp takes the next batch when all its lanes are done.  This
//            keeps neighbouring primary rays in one warp and their node
//            fetches shared -- the choice for camera rays;
//   refill   one ray per lane as a state machine that visits one wide node
//            per loop iteration (visit8); a lane whose ray has finished takes
//            the next unprocessed ray at once (one atomic per warp for all
//            lanes that need one), so a warp never idles behind its slowest
//            ray -- the choice for explicit (typically incoherent) rays.
// Both visit children in the same order (ascending entry distance, then
// slot), so they count the same box tests for the same ray.

struct Lane8 {
    Pre8 rp;
    float best_t;
    uint32_t best, tests, ttests, nvis;
    uint32_t cur;  // next wide node to visit, or kNoHit when the ray is finished
    int sp;
    bool overflow;
};

__device__ __forceinline__ void lane_start(Lane8& L, const Ray8& ray, uint32_t root)
{
    prep8(ray, L.rp);
    L.best_t = L.rp.tmax;
    L.best = kNoHit;
    L.tests = L.ttests = L.nvis = 0;
    L.cur = root;
    L.sp = 0;
    L.overflow = false;
}

// Test a leaf entry's triangles; returns true when an any-hit ray is done.
template <bool ANY>
__device__ __forceinline__ bool leaf8(Lane8& L, const float4* __restrict__ t8, uint32_t e)
{
    const uint32_t cnt = (e >> 27) & 0xFu, first = e & 0x07FFFFFFu;
    for (uint32_t j = 0; j < cnt; ++j) {
        float t;
        uint32_t id;
        L.ttests++;
        if (tri8(t8, first + j, L.rp, L.best_t, t, id)) {
            if (t < L.best_t || (t == L.best_t && id < L.best)) { L.best_t = t; L.best = id; }
            if (ANY) return true;
        }
    }
    return false;
}

// Visit node L.cur; afterwards L.cur is the next node, or kNoHit when the
// ray has finished (stack empty, any-hit found, or stack overflow).
template <bool ANY, bool SIGNED>
__device__ __forceinline__ void visit8(Lane8& L, const Node8* __restrict__ nodes, const float4* __restrict__ t8,
                                       uint32_t* st_e, float* st_t)
{
    const Pre8& rp = L.rp;
    const float4* p = reinterpret_cast<const float4*>(nodes + L.cur);
    const float4 w0 = __ldg(p), w1 = __ldg(p + 1), w2 = __ldg(p + 2), w3 = __ldg(p + 3), w4 = __ldg(p + 4);
    L.nvis++;
    const float org[3] = {w0.x, w0.y, w0.z};
    const uint32_t ei = __float_as_uint(w0.w);
    const float sc[3] = {pow2f((int)(ei & 0xFFu) - 127), pow2f((int)((ei >> 8) & 0xFFu) - 127),
                         pow2f((int)((ei >> 16) & 0xFFu) - 127)};
    const uint32_t imask = ei >> 24;
    const uint32_t child_base = __float_as_uint(w1.x), tri_base = __float_as_uint(w1.y);
    const uint32_t counts = __float_as_uint(w1.z), valid = __float_as_uint(w1.w);
    const uint32_t q[12] = {__float_as_uint(w2.x), __float_as_uint(w2.y), __float_as_uint(w2.z), __float_as_uint(w2.w),
                            __float_as_uint(w3.x), __float_as_uint(w3.y), __float_as_uint(w3.z), __float_as_uint(w3.w),
                            __float_as_uint(w4.x), __float_as_uint(w4.y), __float_as_uint(w4.z), __float_as_uint(w4.w)};
    uint32_t qa[6], qb[6];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const bool ng = SIGNED && rp.inv[a] < 0.0f;
#pragma unroll
        for (int w = 0; w < 2; ++w) {
            const uint32_t lo = q[a * 2 + w], hi = q[6 + a * 2 + w];
            qa[a * 2 + w] = ng ? hi : lo;
            qb[a * 2 + w] = ng ? lo : hi;
        }
    }
    const float lim = L.best_t * kRobust;
    // nearest hit child (kept in registers) and the others pushed onto the
    // stack, sorted far (bottom) to near (top) within this node's pushes
    uint32_t near_e = kNoHit;
    float near_t = 0.0f;
    const int seg = L.sp;
    float A[3], Cn[3], Cf[3];
    const bool aff = SIGNED && node_affine(org, sc, rp, A, Cn, Cf);
    // the child loop, compiled once per distance form (see the tiles path)
    auto scan = [&](auto form) {
        constexpr bool AFF = decltype(form)::value;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            {
                float n, f;
                child_span<AFF, SIGNED>(qa, qb, k >> 2, (uint32_t)(k & 3), A, Cn, Cf, sc, org, rp, n, f);
                if (((valid >> k) & 1u) && n <= f && n <= lim) {
                    uint32_t ent = child_entry(imask, child_base, counts, tri_base, k);
                    float et = n;
                    if (near_e == kNoHit) {
                        near_e = ent;
                        near_t = n;
                    } else {
                        // Children are visited in ascending (entry distance, slot)
                        // order.  The pushed entries keep that order from the top;
                        // a new child has the largest slot so far and goes below
                        // entries of equal distance, a displaced nearest has the
                        // smallest and goes above them.
                        bool displaced = false;
                        if (n < near_t) {
                            const uint32_t te = near_e; const float tt = near_t;
                            near_e = ent; near_t = n;
                            ent = te; et = tt;
                            displaced = true;
                        }
                        if (L.sp >= kStack8) {
                            L.overflow = true;
                        } else {
                            int b = L.sp - 1;
                            while (b >= seg && (st_t[b] < et || (!displaced && st_t[b] == et))) {
                                st_e[b + 1] = st_e[b]; st_t[b + 1] = st_t[b]; --b;
                            }
                            st_e[b + 1] = ent;
                            st_t[b + 1] = et;
                            L.sp++;
                        }
                    }
                }
            }
        }
    };
    L.tests += __popc(valid);
    if (aff) scan(std::true_type{});
    else scan(std::false_type{});
    if (L.overflow) { L.cur = kNoHit; return; }
    // the next node: the nearest child, else the stack (leaves tested on the way)
    uint32_t e = near_e;
    for (;;) {
        if (e == kNoHit) {
            if (L.sp == 0) { L.cur = kNoHit; return; }
            --L.sp;
            if (st_t[L.sp] > L.best_t * kRobust) continue;
            e = st_e[L.sp];
        }
        if (e & 0x80000000u) {
            if (leaf8<ANY>(L, t8, e)) { L.cur = kNoHit; return; }
            e = kNoHit;
            continue;
        }
        L.cur = e;
        return;
    }
}

// Camera rays, tiles: a warp takes one 8x4 pixel tile, each lane runs its
// ray to the end (trace8), then the warp takes the next tile.
template <int MODE>
__global__ void __launch_bounds__(128) k_trace8_tiles(const sqk::Trace8Args a, uint32_t batches)
{
    const uint32_t lane = threadIdx.x & 31u;
    const bool camera = a.ray_kind != SQ_RAYS_EXPLICIT;
    const uint32_t tiles_x = (a.width + 7u) >> 3;
    __shared__ WarpStats s_stats[4];
    WarpStats& ws = s_stats[threadIdx.x >> 5];
    ws.reset(lane);
    for (;;) {
        uint32_t b = 0;
        if (lane == 0) b = a.tile0 + atomicAdd(a.work, 1u);
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (b >= batches) break;
        Ray8 r;
        uint32_t rid = 0;
        bool active;
        if (camera) {
            const uint32_t x = (b % tiles_x) * 8u + (lane & 7u);
            const uint32_t y = (b / tiles_x) * 4u + (lane >> 3);
            active = x < a.width && y < a.height;
            rid = y * a.width + x;
            if (active && a.ray_kind == SQ_RAYS_REFERENCE_CAMERA) {
                // src/tracer.cpp:207-216 (same arithmetic as the FP32 traversal)
                const float aspect = (float)a.width / (float)a.height;
                float nx = ((float)x + 0.5f) / (float)a.width;
                nx = nx * 2.0f;
                nx = nx - 1.0f;
                float ny = ((float)y + 0.5f) / (float)a.height;
                ny = ny * 2.0f;
                ny = ny - 1.0f;
                nx = nx * aspect;
                float l2 = nx * nx + ny * ny;
                l2 = l2 + 1.0f * 1.0f;
                const float len = sqrtf(l2);
                r.o[0] = a.cam[0]; r.o[1] = a.cam[1]; r.o[2] = a.cam[2];
                r.d[0] = nx / len; r.d[1] = ny / len; r.d[2] = 1.0f / len;
                r.tmin = 0.0f;
                r.tmax = 10000.0f;
            } else if (active) {
                // pinhole camera (same arithmetic as the FP32 traversal)
                const float* bs = a.cam;
                float px = ((float)x + 0.5f) / (float)a.width;
                px = px * 2.0f;
                px = px - 1.0f;
                float py = ((float)y + 0.5f) / (float)a.height;
                py = py * 2.0f;
                py = py - 1.0f;
                px = px * bs[12];
                py = py * bs[13];
                float d[3];
                for (int k = 0; k < 3; ++k) {
                    const float s = bs[3 + k] + px * bs[6 + k];
                    d[k] = s + py * bs[9 + k];
                }
                float l2 = d[0] * d[0] + d[1] * d[1];
                l2 = l2 + d[2] * d[2];
                const float len = sqrtf(l2);
                r.o[0] = bs[0]; r.o[1] = bs[1]; r.o[2] = bs[2];
                r.d[0] = d[0] / len; r.d[1] = d[1] / len; r.d[2] = d[2] / len;
                r.tmin = 0.0f;
                r.tmax = FLT_MAX;
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
        Res8 res;
        res.tests = 0;
        res.tri_tests = 0;
        res.nodes = 0;
        if (active) {
            res = trace8<MODE == SQ_TRACE_ANYHIT>(static_cast<const Node8*>(a.nodes), 0u, a.tris8, r);
            if (res.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
        }
        if (a.stats) {
            // requested bytes: ray in (explicit rays), hit record + heatmap out,
            // 80 B per wide node visited, 48 B per triangle tested
            unsigned long long bt = res.tests, tt = res.tri_tests, nv = res.nodes;
            unsigned long long by = active ? (unsigned long long)(camera ? 0u : 32u) + (a.hits ? 12u : 0u) +
                                                 (a.heat ? 3u : 0u) + 80ull * res.nodes + 48ull * res.tri_tests
                                           : 0ull;
            ws.add(lane, bt, tt, by, nv);
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

// Launch bounds of six blocks per SM: the register count stays at 72 (seven
// blocks resident), but the code scheduled under this cap runs 2-3% faster
// on incoherent rays than under the default.
template <int MODE>
__global__ void __launch_bounds__(128, 6) k_trace8_refill(const sqk::Trace8Args a, uint32_t total)
{
    constexpr bool ANY = MODE == SQ_TRACE_ANYHIT;
    const uint32_t lane = threadIdx.x & 31u;
    const bool camera = a.ray_kind != SQ_RAYS_EXPLICIT;
    const uint32_t tiles_x = (a.width + 7u) >> 3;
    const Node8* nodes = static_cast<const Node8*>(a.nodes);
    uint32_t st_e[kStack8];
    float st_t[kStack8];
    Lane8 L;
    L.cur = kNoHit;
    bool has = false, exhausted = false;
    uint32_t rid = 0;
    unsigned long long s_bt = 0, s_tt = 0, s_by = 0, s_nv = 0;
    for (;;) {
        // refill: every lane without a ray takes the next one
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
                    Ray8 r;
                    bool ok;
                    if (camera) {
                        // ray g: pixel (g mod 32) of 8x4 tile g / 32, tiles in row order
                        const uint32_t b = g >> 5, l = g & 31u;
                        const uint32_t x = (b % tiles_x) * 8u + (l & 7u);
                        const uint32_t y = (b / tiles_x) * 4u + (l >> 3);
                        ok = x < a.width && y < a.height;
                        rid = y * a.width + x;
                        if (ok) camera_ray8(a.ray_kind, x, y, a.width, a.height, a.cam, r);
                    } else {
                        rid = g;
                        ok = true;
                        const float4* p = reinterpret_cast<const float4*>(a.rays) + 2ull * rid;
                        const float4 x0 = __ldg(p), x1 = __ldg(p + 1);
                        r.o[0] = x0.x; r.o[1] = x0.y; r.o[2] = x0.z; r.tmin = x0.w;
                        r.d[0] = x1.x; r.d[1] = x1.y; r.d[2] = x1.z; r.tmax = x1.w;
                    }
                    if (ok) {
                        lane_start(L, r, 0u);
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
            // slab form chosen per ray, as trace8 does (sign-selected planes
            // for a ray that cannot produce NaN), so a ray's box tests do not
            // depend on the rays it shares a warp with
            if (no_nan_slabs(L.rp)) visit8<ANY, true>(L, nodes, a.tris8, st_e, st_t);
            else visit8<ANY, false>(L, nodes, a.tris8, st_e, st_t);
            if (L.cur == kNoHit) {
                has = false;
                if (L.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
                if (a.stats) {
                    s_bt += L.tests;
                    s_tt += L.ttests;
                    s_nv += L.nvis;
                    s_by += (camera ? 0u : 32u) + (a.hits ? 12u : 0u) + (a.heat ? 3u : 0u) + 80ull * L.nvis +
                            48ull * L.ttests;
                }
                if (a.hits) {
                    uint32_t* h = reinterpret_cast<uint32_t*>(a.hits) + 3ull * rid;
                    h[0] = L.best;
                    h[1] = __float_as_uint(L.best == kNoHit ? 0.0f : L.best_t);
                    h[2] = L.tests;
                }
                if (a.heat) {
                    write_heat(a.heat + 3ull * rid, (float)L.tests, a.heat_ramp);
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
            s_nv += __shfl_xor_sync(0xFFFFFFFFu, s_nv, o);
        }
        if (lane == 0) {
            atomicAdd(a.stats, s_bt); atomicAdd(a.stats + 1, s_tt); atomicAdd(a.stats + 2, s_by); atomicAdd(a.stats + 3, s_nv);
        }
    }
}

template <int MODE>
void launch8(const sqk::Trace8Args& a, cudaStream_t s)
{
    uint32_t batches;
    if (a.ray_kind == SQ_RAYS_EXPLICIT) batches = (a.ray_count + 31u) / 32u;
    else batches = ((a.width + 7u) / 8u) * ((a.height + 3u) / 4u);
    if (batches == 0) return;
    // The tiles kernel runs one warp per block: a block's SM slot is free as
    // soon as its warp finds no tile left, so the next kernel on the GPU (the
    // next band of a banded image) fills it at once instead of waiting for
    // the slowest of four warps.
    constexpr int kTilesBlock = 32;
    static PerDevice<std::array<int, 2>> cache;
    const std::array<int, 2> per_sm = cache.get([] {
        return std::array<int, 2>{blocks_per_sm(k_trace8_tiles<MODE>, kTilesBlock),
                                  blocks_per_sm(k_trace8_refill<MODE>, 128)};
    });
    const int v = a.refill ? 1 : 0;
    uint32_t grid = (uint32_t)(per_sm[v] * sm_count());
    if (!v && a.tile_end && a.tile_end < batches) batches = a.tile_end;  // a band of the image
    const uint32_t first = v ? 0u : min(a.tile0, batches);
    const uint32_t need = v ? (batches + 3u) / 4u : batches - first;
    if (grid > need) grid = need;
    if (grid == 0) return;
    if (v) k_trace8_refill<MODE><<<grid, 128, 0, s>>>(a, a.ray_kind == SQ_RAYS_EXPLICIT ? a.ray_count : batches * 32u);
    else k_trace8_tiles<MODE><<<grid, kTilesBlock, 0, s>>>(a, batches);
}

// Batch, tiles: as k_trace8_tiles over the job table's 32-ray batches.
template <int MODE>
__global__ void __launch_bounds__(256) k_trace8_batch_tiles(const sqk::BatchTraceArgs a)
{
    const uint32_t lane = threadIdx.x & 31u;
    const Node8* nodes = static_cast<const Node8*>(a.nodes8);
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
        Ray8 r;
        uint32_t rid = 0;
        bool active;
        if (job.ray_kind != SQ_RAYS_EXPLICIT) {
            const uint32_t tiles_x = (job.width + 7u) >> 3;
            const uint32_t x = (lb % tiles_x) * 8u + (lane & 7u);
            const uint32_t y = (lb / tiles_x) * 4u + (lane >> 3);
            active = x < job.width && y < job.height;
            rid = y * job.width + x;
            if (active) camera_ray8(job.ray_kind, x, y, job.width, job.height, job.cam, r);
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
        Res8 res;
        res.tests = 0;
        res.tri_tests = 0;
        res.nodes = 0;
        if (active) {
            res = trace8<MODE == SQ_TRACE_ANYHIT>(nodes, job.root, a.tris8, r);
            if (res.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
            if (res.id != kNoHit) res.id -= job.tri_offset;
        }
        if (a.stats) {
            unsigned long long bt = res.tests, tt = res.tri_tests, nv = res.nodes;
            unsigned long long by = active ? (unsigned long long)(job.ray_kind == SQ_RAYS_EXPLICIT ? 32u : 0u) +
                                                 (a.hits ? 12u : 0u) + (a.heat ? 3u : 0u) + 80ull * res.nodes +
                                                 48ull * res.tri_tests
                                           : 0ull;
            ws.add(lane, bt, tt, by, nv);
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

// Launch bounds of 28 warps per SM whatever the block shape: the same
// register budget (72) as k_trace8_refill, whose occupancy it needs.
template <int MODE, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 896 / BLOCK) k_trace8_batch_refill(const sqk::BatchTraceArgs a)
{
    constexpr bool ANY = MODE == SQ_TRACE_ANYHIT;
    const uint32_t lane = threadIdx.x & 31u;
    const Node8* nodes = static_cast<const Node8*>(a.nodes8);
    const uint32_t total = a.total_batches * 32u;
    uint32_t st_e[kStack8];
    float st_t[kStack8];
    Lane8 L;
    L.cur = kNoHit;
    bool has = false, exhausted = false, explicit_rays = false;
    uint32_t out = 0, tri_offset = 0;
    // the lane's current job and its 32-ray batch range [jlo, jhi): a lane
    // takes consecutive slots, so the job search runs only when a slot
    // leaves the range
    uint32_t cj = 0, jlo = 1, jhi = 0;
    unsigned long long s_bt = 0, s_tt = 0, s_by = 0, s_nv = 0;
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
                    // ray slot g: lane g mod 32 of the job's 32-ray batch g / 32
                    const uint32_t b = g >> 5, l = g & 31u;
                    if (b < jlo || b >= jhi) {
                        cj = find_job(a.jobs, a.njobs, b);
                        jlo = __ldg(&a.jobs[cj].batch_begin);
                        jhi = cj + 1 < a.njobs ? __ldg(&a.jobs[cj + 1].batch_begin) : a.total_batches;
                    }
                    const sqk::BatchJob& job = a.jobs[cj];
                    const uint32_t lb = b - jlo;
                    Ray8 r;
                    bool ok;
                    uint32_t rid;
                    explicit_rays = job.ray_kind == SQ_RAYS_EXPLICIT;
                    if (!explicit_rays) {
                        const uint32_t tiles_x = (job.width + 7u) >> 3;
                        const uint32_t x = (lb % tiles_x) * 8u + (l & 7u);
                        const uint32_t y = (lb / tiles_x) * 4u + (l >> 3);
                        ok = x < job.width && y < job.height;
                        rid = y * job.width + x;
                        if (ok) camera_ray8(job.ray_kind, x, y, job.width, job.height, job.cam, r);
                    } else {
                        rid = lb * 32u + l;
                        ok = rid < job.ray_count;
                        if (ok) {
                            const float4* p = reinterpret_cast<const float4*>(job.rays ? job.rays : a.rays) + 2ull * (job.ray_offset + rid);
                            const float4 x0 = __ldg(p), x1 = __ldg(p + 1);
                            r.o[0] = x0.x; r.o[1] = x0.y; r.o[2] = x0.z; r.tmin = x0.w;
                            r.d[0] = x1.x; r.d[1] = x1.y; r.d[2] = x1.z; r.tmax = x1.w;
                        }
                    }
                    if (ok) {
                        out = job.out_offset + rid;
                        tri_offset = job.tri_offset;
                        lane_start(L, r, job.root);
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
            if (no_nan_slabs(L.rp)) visit8<ANY, true>(L, nodes, a.tris8, st_e, st_t);
            else visit8<ANY, false>(L, nodes, a.tris8, st_e, st_t);
            if (L.cur == kNoHit) {
                has = false;
                if (L.overflow) raise_error(a.err, SQ_DEVERR_STACK_OVERFLOW);
                if (a.stats) {
                    s_bt += L.tests;
                    s_tt += L.ttests;
                    s_nv += L.nvis;
                    s_by += (explicit_rays ? 32u : 0u) + (a.hits ? 12u : 0u) + (a.heat ? 3u : 0u) + 80ull * L.nvis +
                            48ull * L.ttests;
                }
                const uint32_t id = L.best == kNoHit ? kNoHit : L.best - tri_offset;
                if (a.hits) {
                    uint32_t* h = reinterpret_cast<uint32_t*>(a.hits) + 3ull * out;
                    h[0] = id;
                    h[1] = __float_as_uint(L.best == kNoHit ? 0.0f : L.best_t);
                    h[2] = L.tests;
                }
                if (a.heat) {
                    write_heat(a.heat + 3ull * out, (float)L.tests, a.heat_ramp);
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
            s_nv += __shfl_xor_sync(0xFFFFFFFFu, s_nv, o);
        }
        if (lane == 0) {
            atomicAdd(a.stats, s_bt); atomicAdd(a.stats + 1, s_tt); atomicAdd(a.stats + 2, s_by); atomicAdd(a.stats + 3, s_nv);
        }
    }
}

template <int MODE>
void launch8_batch(const sqk::BatchTraceArgs& a, int block, cudaStream_t s)
{
    if (a.total_batches == 0) return;
    static PerDevice<std::array<int, 6>> cache;
    const std::array<int, 6> per_sm = cache.get([] {
        return std::array<int, 6>{blocks_per_sm(k_trace8_batch_tiles<MODE>, 64),
                                  blocks_per_sm(k_trace8_batch_tiles<MODE>, 128),
                                  blocks_per_sm(k_trace8_batch_tiles<MODE>, 256),
                                  blocks_per_sm(k_trace8_batch_refill<MODE, 64>, 64),
                                  blocks_per_sm(k_trace8_batch_refill<MODE, 128>, 128),
                                  blocks_per_sm(k_trace8_batch_refill<MODE, 256>, 256)};
    });
    const int bi = block <= 64 ? 0 : (block <= 128 ? 1 : 2);
    const int v = a.refill ? 1 : 0;
    uint32_t grid = (uint32_t)(per_sm[3 * v + bi] * sm_count());
    const uint32_t need = (a.total_batches + (uint32_t)(block / 32) - 1) / (uint32_t)(block / 32);
    if (grid > need) grid = need;
    if (v && bi == 0) k_trace8_batch_refill<MODE, 64><<<grid, 64, 0, s>>>(a);
    else if (v && bi == 1) k_trace8_batch_refill<MODE, 128><<<grid, 128, 0, s>>>(a);
    else if (v) k_trace8_batch_refill<MODE, 256><<<grid, 256, 0, s>>>(a);
    else k_trace8_batch_tiles<MODE><<<grid, block, 0, s>>>(a);
}

}  // namespace

namespace sqk {

void trace8_batch(const BatchTraceArgs& a, int block, cudaStream_t s)
{
    if (block != 64 && block != 128 && block != 256) block = 128;
    if (a.mode == SQ_TRACE_ANYHIT) launch8_batch<SQ_TRACE_ANYHIT>(a, block, s);
    else launch8_batch<SQ_TRACE_CLOSEST>(a, block, s);
}

void trace8(const Trace8Args& a, cudaStream_t s)
{
    if (a.mode == SQ_TRACE_ANYHIT) launch8<SQ_TRACE_ANYHIT>(a, s);
    else launch8<SQ_TRACE_CLOSEST>(a, s);
}

}  // namespace sqk
