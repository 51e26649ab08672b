/*
 * sq_oracle.c -- CPU restatement of Sequoia's BVH build and trace path.
 *
 * TEST INFRASTRUCTURE ONLY (see sq_oracle.h).  Compiled with
 * -ffp-contract=off so that every a*b+c is two rounded operations, as in the
 * GPU kernels.
 *
 * Range-tree layout.  Every tree built here (and by the GPU library) is a
 * top-down tree over a final triangle order perm[0..n): each node covers a
 * contiguous range [b, e) of perm.  With L = base + 2n + 2 (the leaf region):
 *   - slot L + p holds the leaf record of the triangle at position p, for
 *     every p (written whether or not a cluster references it);
 *   - a binary node whose split boundary is q (left = [b, q), right = [q, e))
 *     stores its two child records in slots base + 2q and base + 2q + 1;
 *   - a leaf cluster over [b, b + c) is an inner record {child = L + b,
 *     count = c}: its leaves are the leaf-region records, contiguous;
 *   - a child range of one triangle is a copy of its leaf record stored in
 *     the parent's slot;
 *   - the root record is slot 0 (it is always an inner record, as in the
 *     reference: src/builder.cpp:1604-1609, 2498-2501).
 * The position of every record follows from the logical tree alone, so two
 * builds of the same logical tree write identical records whatever order
 * they run in.  Morton and SAH trees use base 0 and 3n + 2 slots; the grid
 * tree puts its 63-node heap in slots 0..62, its 64 cell nodes in 63..126
 * and the cell subtrees at base 128.
 */
#include "sq_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* threads                                                                   */

static int g_threads = 0;

void sqo_set_threads(int n) { g_threads = n; }

int sqo_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* the reference's min/max                                                   */

/* std::min(a, b) == (b < a) ? b : a   (vec3f1 min, src/vec3.h:179; simd min,
 * src/simd_generic.h:164-168)                                               */
static inline float rmin(float a, float b) { return (b < a) ? b : a; }
/* std::max(a, b) == (a < b) ? b : a   (vec3f1 max, src/vec3.h:180)          */
static inline float rmax(float a, float b) { return (a < b) ? b : a; }
/* simd max: a > b ? a : b              (src/simd_generic.h:170-174)          */
static inline float smax(float a, float b) { return (a > b) ? a : b; }

/* float -> uint32 truncation; NaN and negatives give 0 (matching x86-64
 * cvttss2si through a 64-bit register and the GPU's cvt.rzi.u32.f32).      */
static inline uint32_t f2u(float x) { return (x >= 0.0f) ? (uint32_t)x : 0u; }

/* float -> int truncation as int(x) in the reference; out-of-range clamps. */
static inline int f2i(float x)
{
    if (!(x == x)) return 0;
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}

typedef struct box { float mn[3], mx[3]; } box;

static inline void box_reset(box* b)
{
    for (int k = 0; k < 3; ++k) { b->mn[k] = FLT_MAX; b->mx[k] = -FLT_MAX; }
}

/* AABB1::grow(AABB1) (src/aabb.h:114) */
static inline void box_grow_box(box* b, const box* o)
{
    for (int k = 0; k < 3; ++k) { b->mn[k] = rmin(b->mn[k], o->mn[k]); b->mx[k] = rmax(b->mx[k], o->mx[k]); }
}

/* AABB1::grow(vec3f1) (src/aabb.h:113) */
static inline void box_grow_pt(box* b, const float* p)
{
    for (int k = 0; k < 3; ++k) { b->mn[k] = rmin(b->mn[k], p[k]); b->mx[k] = rmax(b->mx[k], p[k]); }
}

/* AABB1::sa() (src/aabb.h:120-123): (x*y + x*z + y*z) * 2 */
static inline float box_sa(const box* b)
{
    float lx = b->mx[0] - b->mn[0], ly = b->mx[1] - b->mn[1], lz = b->mx[2] - b->mn[2];
    float xy = lx * ly, xz = lx * lz, yz = ly * lz;
    float s = xy + xz;
    s = s + yz;
    return s * 2.0f;
}

/* triangle AABB: min(min(v0,v1),v2), max(max(v0,v1),v2) (src/builder.cpp:130-131) */
static inline void tri_box(const float* t, box* b)
{
    for (int k = 0; k < 3; ++k) {
        b->mn[k] = rmin(rmin(t[k], t[3 + k]), t[6 + k]);
        b->mx[k] = rmax(rmax(t[k], t[3 + k]), t[6 + k]);
    }
}

/* centroid (a.min + a.max) * 0.5f (src/builder.cpp:134) */
static inline void box_centre(const box* b, float* c)
{
    for (int k = 0; k < 3; ++k) { float s = b->mn[k] + b->mx[k]; c[k] = s * 0.5f; }
}

void sqo_tri_aabbs(const float* tris, uint32_t n, float* aabbs, float* scene)
{
    box s;
    box_reset(&s);
    for (uint32_t i = 0; i < n; ++i) {
        box b;
        tri_box(tris + 9 * (size_t)i, &b);
        if (aabbs) {
            memcpy(aabbs + 6 * (size_t)i, b.mn, 12);
            memcpy(aabbs + 6 * (size_t)i + 3, b.mx, 12);
        }
        box_grow_box(&s, &b);
    }
    if (scene) { memcpy(scene, s.mn, 12); memcpy(scene + 3, s.mx, 12); }
}

/* ------------------------------------------------------------------------- */
/* Morton codes                                                              */

/* Deposit the low 10 bits of v at every third bit starting at `first`,
 * the effect of _pdep_u32 with masks 0x49249249 / 0x92492492 / 0x24924924
 * (src/algorithms.cpp:10-12) on a 10-bit input.                             */
static inline uint32_t spread3(uint32_t v, int first)
{
    uint32_t r = 0;
    for (int i = 0; i < 11; ++i)
        if ((v >> i) & 1u) {
            int pos = first + 3 * i;
            if (pos < 32) r |= 1u << pos;
        }
    return r;
}

uint32_t sqo_bit_interleave_32(uint32_t x, uint32_t y, uint32_t z)
{
    return spread3(x, 0) | spread3(y, 1) | spread3(z, 2);
}

void sqo_morton_codes(const float* tris, uint32_t n, int bounds_mode,
                      uint32_t* codes, float* scene_box)
{
    /* scene_aabb over the triangle AABBs, serially (src/builder.cpp:2206-2215) */
    box s;
    box_reset(&s);
    for (uint32_t i = 0; i < n; ++i) {
        box b;
        tri_box(tris + 9 * (size_t)i, &b);
        if (bounds_mode == 1) {
            float c[3];
            box_centre(&b, c);
            box_grow_pt(&s, c);
        } else {
            box_grow_box(&s, &b);
        }
    }
    if (scene_box) { memcpy(scene_box, s.mn, 12); memcpy(scene_box + 3, s.mx, 12); }
    float ext[3];
    for (int k = 0; k < 3; ++k) ext[k] = s.mx[k] - s.mn[k];

    /* per-triangle code (src/builder.cpp:2217-2236) */
#pragma omp parallel for schedule(static) num_threads(sqo_get_threads())
    for (long long i = 0; i < (long long)n; ++i) {
        box b;
        tri_box(tris + 9 * (size_t)i, &b);
        float c[3];
        box_centre(&b, c);
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            float u = (c[k] - s.mn[k]) / ext[k];
            q[k] = f2u(u * 1023.0f);
        }
        codes[i] = sqo_bit_interleave_32(q[0], q[1], q[2]);
    }
}

/* 64-bit codes (build_hierarchy_morton2): _pdep_u64 with masks
 * 0x9249249249249249 / 0x2492492492492492 / 0x4924924924924924
 * (src/algorithms.cpp:16-22) on 20-bit inputs.                             */
static inline uint64_t spread3_64(uint64_t v, int first)
{
    uint64_t r = 0;
    for (int i = 0; i < 22; ++i)
        if ((v >> i) & 1u) {
            int pos = first + 3 * i;
            if (pos < 64) r |= (uint64_t)1 << pos;
        }
    return r;
}

uint64_t sqo_bit_interleave_64(uint64_t x, uint64_t y, uint64_t z)
{
    return spread3_64(x, 0) | spread3_64(y, 1) | spread3_64(z, 2);
}

/* setup_morton2 (src/builder.cpp:2247-2279): as sqo_morton_codes with
 * 0xFFFFF steps per axis */
void sqo_morton_codes64(const float* tris, uint32_t n, int bounds_mode, uint64_t* codes, float* scene_box)
{
    box s;
    box_reset(&s);
    for (uint32_t i = 0; i < n; ++i) {
        box b;
        tri_box(tris + 9 * (size_t)i, &b);
        if (bounds_mode == 1) {
            float c[3];
            box_centre(&b, c);
            box_grow_pt(&s, c);
        } else {
            box_grow_box(&s, &b);
        }
    }
    if (scene_box) { memcpy(scene_box, s.mn, 12); memcpy(scene_box + 3, s.mx, 12); }
    float ext[3];
    for (int k = 0; k < 3; ++k) ext[k] = s.mx[k] - s.mn[k];
#pragma omp parallel for schedule(static) num_threads(sqo_get_threads())
    for (long long i = 0; i < (long long)n; ++i) {
        box b;
        tri_box(tris + 9 * (size_t)i, &b);
        float c[3];
        box_centre(&b, c);
        uint64_t q[3];
        for (int k = 0; k < 3; ++k) {
            float u = (c[k] - s.mn[k]) / ext[k];
            q[k] = f2u(u * 1048575.0f);
        }
        codes[i] = sqo_bit_interleave_64(q[0], q[1], q[2]);
    }
}

/* ------------------------------------------------------------------------- */
/* stable LSD radix sort (src/algorithms.h:41-113)                           */

void sqo_sort_pairs(uint32_t* keys, uint32_t* values, uint32_t n,
                    uint32_t key_bits, uint32_t digit_bits)
{
    if (n < 2) return;
    if (digit_bits < 1) digit_bits = 8;
    if (digit_bits > 16) digit_bits = 16;
    uint32_t* k2 = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    uint32_t* v2 = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    uint32_t radix = 1u << digit_bits;
    uint32_t* cnt = (uint32_t*)malloc(sizeof(uint32_t) * radix);
    uint32_t *ks = keys, *vs = values, *kd = k2, *vd = v2;
    for (uint32_t shift = 0; shift < key_bits; shift += digit_bits) {
        uint32_t mask = radix - 1u;
        memset(cnt, 0, sizeof(uint32_t) * radix);
        for (uint32_t i = 0; i < n; ++i) cnt[(ks[i] >> shift) & mask]++;
        uint32_t sum = 0;
        for (uint32_t d = 0; d < radix; ++d) { uint32_t c = cnt[d]; cnt[d] = sum; sum += c; }
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t p = cnt[(ks[i] >> shift) & mask]++;
            kd[p] = ks[i];
            vd[p] = vs[i];
        }
        uint32_t* t;
        t = ks; ks = kd; kd = t;
        t = vs; vs = vd; vd = t;
    }
    if (ks != keys) {
        memcpy(keys, ks, sizeof(uint32_t) * (size_t)n);
        memcpy(values, vs, sizeof(uint32_t) * (size_t)n);
    }
    free(k2);
    free(v2);
    free(cnt);
}

/* radix_sort<uint64_t, RadixInput64>(..., 8): stable LSD over 64-bit keys */
void sqo_sort_pairs64(uint64_t* keys, uint32_t* values, uint32_t n)
{
    if (n < 2) return;
    uint64_t* k2 = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
    uint32_t* v2 = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    uint32_t cnt[256];
    uint64_t *ks = keys, *kd = k2;
    uint32_t *vs = values, *vd = v2;
    for (uint32_t shift = 0; shift < 64; shift += 8) {
        memset(cnt, 0, sizeof cnt);
        for (uint32_t i = 0; i < n; ++i) cnt[(ks[i] >> shift) & 255u]++;
        uint32_t sum = 0;
        for (uint32_t d = 0; d < 256; ++d) { uint32_t c = cnt[d]; cnt[d] = sum; sum += c; }
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t p = cnt[(ks[i] >> shift) & 255u]++;
            kd[p] = ks[i];
            vd[p] = vs[i];
        }
        uint64_t* tk = ks; ks = kd; kd = tk;
        uint32_t* tv = vs; vs = vd; vd = tv;
    }
    /* eight passes: the result is back in the caller's arrays */
    free(k2);
    free(v2);
}

/* ------------------------------------------------------------------------- */
/* Morton topology                                                           */

static inline int lzcnt32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

uint32_t sqo_find_split_morton(const uint32_t* codes, uint32_t count)
{
    uint32_t first = codes[0];
    uint32_t last_code = codes[count - 1];
    if (first == last_code) return count >> 1;
    int common = lzcnt32(first ^ last_code);
    int split = 0;
    int last = (int)count - 1;
    int step = last;
    do {
        step = (step + 1) >> 1;
        int ns = split + step;
        if (ns < last) {
            int sp = lzcnt32(first ^ codes[ns]);
            if (sp > common) split = ns;
        }
    } while (step > 1);
    return (uint32_t)split;
}

static inline int lzcnt64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

/* find_split_morton2 (src/builder.cpp:2316-2349) */
uint32_t sqo_find_split_morton64(const uint64_t* codes, uint32_t count)
{
    uint64_t first = codes[0];
    uint64_t last_code = codes[count - 1];
    if (first == last_code) return count >> 1;
    int common = lzcnt64(first ^ last_code);
    int split = 0;
    int last = (int)count - 1;
    int step = last;
    do {
        step = (step + 1) >> 1;
        int ns = split + step;
        if (ns < last) {
            int sp = lzcnt64(first ^ codes[ns]);
            if (sp > common) split = ns;
        }
    } while (step > 1);
    return (uint32_t)split;
}

uint32_t sqo_node_capacity(uint32_t n, int kind)
{
    return (kind == 2 ? 128u : 0u) + 3u * n + 2u;
}

static inline void write_leaf(sqo_node1* nd, const box* b, uint32_t tri)
{
    memcpy(nd->min, b->mn, 12);
    memcpy(nd->max, b->mx, 12);
    nd->count = 1;
    nd->flags = SQO_LEAF;
    nd->child = tri;
}

static inline void write_inner(sqo_node1* nd, const box* b, uint32_t child, uint32_t count)
{
    memcpy(nd->min, b->mn, 12);
    memcpy(nd->max, b->mx, 12);
    nd->count = (uint16_t)count;
    nd->flags = 0;
    nd->child = child;
}

/* Leaf-region records of every triangle: slot base + 2n + 2 + p */
static void emit_leaves(const box* tb, const uint32_t* perm, uint32_t base, uint32_t n,
                        sqo_node1* nodes)
{
    for (uint32_t p = 0; p < n; ++p) write_leaf(&nodes[base + 2u * n + 2u + p], &tb[perm[p]], perm[p]);
}

static inline void range_box(const box* tb, const uint32_t* perm, uint32_t b, uint32_t c, box* out)
{
    box_reset(out);
    for (uint32_t k = 0; k < c; ++k) box_grow_box(out, &tb[perm[b + k]]);
}

typedef struct morton_job {
    const uint32_t* codes;    /* 30-bit codes, or NULL when codes64 is used */
    const uint64_t* codes64;  /* 60-bit codes (build_hierarchy_morton2)     */
    const uint32_t* perm;
    const box* tb;
    sqo_node1* nodes;
    uint32_t leaf0;
} morton_job;

/* recurse_morton (src/builder.cpp:2351-2409): writes the record of range
 * [b, e) into `slot` and its subtree below; returns the range bounds.       */
static void morton_range(const morton_job* j, uint32_t b, uint32_t e, uint32_t slot, box* out)
{
    uint32_t c = e - b;
    if (c == 1) {
        uint32_t t = j->perm[b];
        write_leaf(&j->nodes[slot], &j->tb[t], t);
        *out = j->tb[t];
        return;
    }
    if (c < 8) {
        range_box(j->tb, j->perm, b, c, out);
        write_inner(&j->nodes[slot], out, j->leaf0 + b, c);
        return;
    }
    uint32_t s = j->codes64 ? sqo_find_split_morton64(j->codes64 + b, c) : sqo_find_split_morton(j->codes + b, c);
    uint32_t q = b + s + 1u;
    box bl, br;
    if (c > 4096) {
#pragma omp task shared(bl) firstprivate(j, b, q)
        morton_range(j, b, q, 2u * q, &bl);
        morton_range(j, q, e, 2u * q + 1u, &br);
#pragma omp taskwait
    } else {
        morton_range(j, b, q, 2u * q, &bl);
        morton_range(j, q, e, 2u * q + 1u, &br);
    }
    *out = bl;
    box_grow_box(out, &br);
    write_inner(&j->nodes[slot], out, 2u * q, 2u);
}

uint32_t sqo_build_morton(const float* tris, uint32_t n, int bounds_mode,
                          sqo_node1* nodes, uint32_t* codes_out,
                          uint32_t* perm_out)
{
    uint32_t* codes = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    box* tb = (box*)malloc(sizeof(box) * ((size_t)n + 1));
    sqo_morton_codes(tris, n, bounds_mode, codes, NULL);
    for (uint32_t i = 0; i < n; ++i) {
        perm[i] = i;
        tri_box(tris + 9 * (size_t)i, &tb[i]);
    }
    sqo_sort_pairs(codes, perm, n, 32, 8);
    morton_job j = {codes, NULL, perm, tb, nodes, 2u * n + 2u};
    emit_leaves(tb, perm, 0, n, nodes);
    box root;
    if (n < 8) {
        /* the root is always an inner record (src/builder.cpp:2498-2501) */
        range_box(tb, perm, 0, n, &root);
        write_inner(&nodes[0], &root, j.leaf0, n);
    } else {
#pragma omp parallel num_threads(sqo_get_threads())
#pragma omp single
        morton_range(&j, 0, n, 0, &root);
    }
    if (codes_out) memcpy(codes_out, codes, sizeof(uint32_t) * (size_t)n);
    if (perm_out) memcpy(perm_out, perm, sizeof(uint32_t) * (size_t)n);
    free(codes);
    free(perm);
    free(tb);
    return 0;
}

/* build_hierarchy_morton2 (src/builder.cpp:2510-2544): the same range tree
 * over 60-bit codes (recurse_morton2, src/builder.cpp:2413-2472) */
uint32_t sqo_build_morton64(const float* tris, uint32_t n, int bounds_mode, sqo_node1* nodes, uint64_t* codes_out,
                            uint32_t* perm_out)
{
    uint64_t* codes = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)n + 1));
    uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    box* tb = (box*)malloc(sizeof(box) * ((size_t)n + 1));
    sqo_morton_codes64(tris, n, bounds_mode, codes, NULL);
    for (uint32_t i = 0; i < n; ++i) {
        perm[i] = i;
        tri_box(tris + 9 * (size_t)i, &tb[i]);
    }
    sqo_sort_pairs64(codes, perm, n);
    morton_job j = {NULL, codes, perm, tb, nodes, 2u * n + 2u};
    emit_leaves(tb, perm, 0, n, nodes);
    box root;
    if (n < 8) {
        range_box(tb, perm, 0, n, &root);
        write_inner(&nodes[0], &root, j.leaf0, n);
    } else {
#pragma omp parallel num_threads(sqo_get_threads())
#pragma omp single
        morton_range(&j, 0, n, 0, &root);
    }
    if (codes_out) memcpy(codes_out, codes, sizeof(uint64_t) * (size_t)n);
    if (perm_out) memcpy(perm_out, perm, sizeof(uint32_t) * (size_t)n);
    free(codes);
    free(perm);
    free(tb);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* binned SAH                                                                */

typedef struct bin { box p, c; int count; } bin;

static inline void bin_reset(bin* b) { box_reset(&b->p); box_reset(&b->c); b->count = 0; }

/* Bin::combine (src/builder.h:25) */
static inline bin bin_combine(const bin* a, const bin* b)
{
    bin r = *a;
    box_grow_box(&r.p, &b->p);
    box_grow_box(&r.c, &b->c);
    r.count = a->count + b->count;
    return r;
}

typedef struct sah_job {
    const box* tb;      /* triangle boxes                  */
    const float* cen;   /* centroids, 3 per triangle       */
    uint32_t* ids;      /* working order                   */
    uint32_t* tmp;      /* partition scratch               */
    sqo_node1* nodes;
    uint32_t base;
    uint32_t leaf0;     /* first leaf-region slot          */
    uint32_t bins;
    uint32_t leaf;
    int fail;
} sah_job;

/* choose_axis (src/builder.cpp:334-345) */
static inline int choose_axis(const box* c)
{
    float lx = c->mx[0] - c->mn[0], ly = c->mx[1] - c->mn[1], lz = c->mx[2] - c->mn[2];
    int r = 0;
    r += 2 * (lz > lx && lz > ly);
    r += 1 * (ly > lx && ly >= lz);
    return r;
}

/* bin index of a centroid coordinate (src/builder.cpp:380-391) */
static inline int bin_of(float k1, float c, float cmin, int nb)
{
    float d = c - cmin;
    int b = f2i(k1 * d);
    if (b < 0) b = 0;
    if (b > nb - 1) b = nb - 1;
    return b;
}

static inline float bin_k1(int nb, float ext)
{
    float eps = 1.1920929e-7f;
    float one_minus = 1.0f - eps;
    float num = (float)nb * one_minus;
    return num / ext;
}

/* leaf creation (src/builder.cpp:1075-1089): a cluster record over the
 * leaf region, or the leaf record itself for one triangle below the root */
static void sah_leaf(sah_job* j, uint32_t b, uint32_t cnt, const box* p, uint32_t slot, int is_root)
{
    if (cnt > 65535u) { j->fail = 1; return; }
    if (cnt == 1 && !is_root) {
        uint32_t t = j->ids[b];
        write_leaf(&j->nodes[slot], &j->tb[t], t);
        return;
    }
    write_inner(&j->nodes[slot], p, j->leaf0 + b, cnt);
}

/* recurse (src/builder.cpp:1053-1156): node over ids[b, e) with primitive box
 * p and centroid box c; writes its record into `slot`.  The partition is
 * stable; the reference's in-place swap partition (src/builder.cpp:599-628)
 * yields the same two sets in another order.                               */
static void sah_range(sah_job* j, uint32_t b, uint32_t e, const box* p, const box* c,
                      uint32_t slot, int is_root)
{
    uint32_t cnt = e - b;
    if (cnt <= j->leaf || box_sa(c) <= 0.0f) {
        sah_leaf(j, b, cnt, p, slot, is_root);
        return;
    }
    int nb = (int)j->bins;
    int axis = choose_axis(c);
    float k1 = bin_k1(nb, c->mx[axis] - c->mn[axis]);
    float cmin = c->mn[axis];
    bin bins[32];
    for (int i = 0; i < nb; ++i) bin_reset(&bins[i]);
    for (uint32_t i = b; i < e; ++i) {
        uint32_t t = j->ids[i];
        const float* ct = j->cen + 3 * (size_t)t;
        int bi = bin_of(k1, ct[axis], cmin, nb);
        box_grow_box(&bins[bi].p, &j->tb[t]);
        box_grow_pt(&bins[bi].c, ct);
        bins[bi].count += 1;
    }
    /* choose_plane (src/builder.cpp:488-523) */
    bin l2r[32];
    l2r[0] = bins[0];
    for (int i = 1; i < nb - 1; ++i) l2r[i] = bin_combine(&l2r[i - 1], &bins[i]);
    bin r2l = bins[nb - 1];
    float best = FLT_MAX;
    int plane = 0, chosen = 0;
    box lp, rp, lc, rc;
    box_reset(&lp); box_reset(&rp); box_reset(&lc); box_reset(&rc);
    for (int i = nb - 2; i >= 0; --i) {
        float sl = box_sa(&l2r[i].p) * (float)l2r[i].count;
        float sr = box_sa(&r2l.p) * (float)r2l.count;
        float score = sl + sr;
        if (score < best) {
            best = score;
            plane = i;
            chosen = 1;
            lp = l2r[i].p; rp = r2l.p; lc = l2r[i].c; rc = r2l.c;
        }
        r2l = bin_combine(&r2l, &bins[i]);
    }
    if (!chosen) {
        /* no plane scored below FLT_MAX (only with coordinates near the float
         * range); the reference would split with unset child boxes here.  Both
         * this oracle and the GPU builder make the node a leaf instead. */
        sah_leaf(j, b, cnt, p, slot, is_root);
        return;
    }
    /* stable partition by bin <= plane */
    uint32_t nl = 0, nr = 0;
    for (uint32_t i = b; i < e; ++i) {
        uint32_t t = j->ids[i];
        int bi = bin_of(k1, j->cen[3 * (size_t)t + axis], cmin, nb);
        if (bi <= plane) j->ids[b + nl++] = t;
        else j->tmp[b + nr++] = t;
    }
    memcpy(j->ids + b + nl, j->tmp + b, sizeof(uint32_t) * nr);
    if (nl == 0 || nr == 0) {
        /* cannot happen for a plane with a finite score */
        j->fail = 1;
        return;
    }
    uint32_t q = b + nl;
    uint32_t ls = j->base + 2u * q, rs = ls + 1u;
    if (nl > 10000) {
#pragma omp task firstprivate(j, b, q, ls, lp, lc)
        sah_range(j, b, q, &lp, &lc, ls, 0);
        sah_range(j, q, e, &rp, &rc, rs, 0);
#pragma omp taskwait
    } else {
        sah_range(j, b, q, &lp, &lc, ls, 0);
        sah_range(j, q, e, &rp, &rc, rs, 0);
    }
    write_inner(&j->nodes[slot], p, ls, 2u);
}

static void sah_setup(const float* tris, uint32_t n, box* tb, float* cen, box* p, box* c)
{
    box_reset(p);
    box_reset(c);
    for (uint32_t i = 0; i < n; ++i) {
        tri_box(tris + 9 * (size_t)i, &tb[i]);
        box_centre(&tb[i], cen + 3 * (size_t)i);
        box_grow_box(p, &tb[i]);
        box_grow_pt(c, cen + 3 * (size_t)i);
    }
}

uint32_t sqo_build_sah(const float* tris, uint32_t n, uint32_t bins,
                       uint32_t leaf_size, sqo_node1* nodes, uint32_t* perm_out)
{
    if (bins < 2) bins = 8;
    if (bins > 32) bins = 32;
    if (leaf_size < 1) leaf_size = 8;
    box* tb = (box*)malloc(sizeof(box) * ((size_t)n + 1));
    float* cen = (float*)malloc(sizeof(float) * 3 * ((size_t)n + 1));
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    box p, c;
    sah_setup(tris, n, tb, cen, &p, &c);
    for (uint32_t i = 0; i < n; ++i) ids[i] = i;
    sah_job j = {tb, cen, ids, tmp, nodes, 0, 2u * n + 2u, bins, leaf_size, 0};
#pragma omp parallel num_threads(sqo_get_threads())
#pragma omp single
    sah_range(&j, 0, n, &p, &c, 0, 1);
    emit_leaves(tb, ids, 0, n, nodes);
    if (perm_out) memcpy(perm_out, ids, sizeof(uint32_t) * (size_t)n);
    free(tb); free(cen); free(ids); free(tmp);
    return j.fail ? 0xFFFFFFFFu : 0u;
}

/* ------------------------------------------------------------------------- */
/* grid builder                                                              */

/* compact_1_by_2 (src/builder.cpp:27-35): every third bit of x */
static inline uint32_t compact3(uint32_t x)
{
    uint32_t r = 0;
    for (int i = 0; i < 11; ++i) r |= ((x >> (3 * i)) & 1u) << i;
    return r;
}

uint32_t sqo_build_grid(const float* tris, uint32_t n, uint32_t bins,
                        uint32_t leaf_size, int scene_bounds_cells,
                        sqo_node1* nodes, uint32_t* perm_out)
{
    if (bins < 2) bins = 8;
    if (bins > 32) bins = 32;
    if (leaf_size < 1) leaf_size = 8;
    box* tb = (box*)malloc(sizeof(box) * ((size_t)n + 1));
    float* cen = (float*)malloc(sizeof(float) * 3 * ((size_t)n + 1));
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    int* cell_of = (int*)malloc(sizeof(int) * ((size_t)n + 1));
    box p, c;
    sah_setup(tris, n, tb, cen, &p, &c);
    /* bin_centroids_to_grid (src/builder.cpp:1665-1753) */
    float k1[3];
    for (int a = 0; a < 3; ++a) k1[a] = bin_k1(4, c.mx[a] - c.mn[a]);
    bin cells[64];
    for (int i = 0; i < 64; ++i) bin_reset(&cells[i]);
    for (uint32_t i = 0; i < n; ++i) {
        int g[3];
        for (int a = 0; a < 3; ++a) g[a] = bin_of(k1[a], cen[3 * (size_t)i + a], c.mn[a], 4);
        int cell = (g[2] * 4 + g[1]) * 4 + g[0];
        cell_of[i] = cell;
        box_grow_box(&cells[cell].p, &tb[i]);
        box_grow_pt(&cells[cell].c, cen + 3 * (size_t)i);
        cells[cell].count += 1;
    }
    /* cells in Morton order: cell slot m holds grid cell (kx, ky, kz) */
    uint32_t begin[65];
    int cell_at[64];
    uint32_t sum = 0;
    for (int m = 0; m < 64; ++m) {
        uint32_t kx = compact3((uint32_t)m), ky = compact3((uint32_t)m >> 1), kz = compact3((uint32_t)m >> 2);
        int cell = (int)((kz * 4 + ky) * 4 + kx);
        cell_at[m] = cell;
        begin[m] = sum;
        sum += (uint32_t)cells[cell].count;
    }
    begin[64] = n;
    int slot_of_cell[64];
    for (int m = 0; m < 64; ++m) slot_of_cell[cell_at[m]] = m;
    uint32_t fill[64];
    for (int m = 0; m < 64; ++m) fill[m] = begin[m];
    for (uint32_t i = 0; i < n; ++i) ids[fill[slot_of_cell[cell_of[i]]]++] = i;

    sah_job j = {tb, cen, ids, tmp, nodes, 128u, 128u + 2u * n + 2u, bins, leaf_size, 0};
#pragma omp parallel for schedule(dynamic, 1) num_threads(sqo_get_threads())
    for (int m = 0; m < 64; ++m) {
        const bin* cb = &cells[cell_at[m]];
        sah_range(&j, begin[m], begin[m + 1], &cb->p, &cb->c, 63u + (uint32_t)m, 1);
        if (scene_bounds_cells) {
            memcpy(nodes[63 + m].min, p.mn, 12);
            memcpy(nodes[63 + m].max, p.mx, 12);
        }
    }
    emit_leaves(tb, ids, 128u, n, nodes);
    /* heap above the cells (src/builder.cpp:2181-2188) */
    for (int i = 62; i >= 0; --i) {
        box u;
        for (int k = 0; k < 3; ++k) {
            u.mn[k] = rmin(nodes[2 * i + 1].min[k], nodes[2 * i + 2].min[k]);
            u.mx[k] = rmax(nodes[2 * i + 1].max[k], nodes[2 * i + 2].max[k]);
        }
        write_inner(&nodes[i], &u, 2u * (uint32_t)i + 1u, 2u);
    }
    if (perm_out) memcpy(perm_out, ids, sizeof(uint32_t) * (size_t)n);
    free(tb); free(cen); free(ids); free(tmp); free(cell_of);
    return j.fail ? 0xFFFFFFFFu : 0u;
}

/* ------------------------------------------------------------------------- */
/* rays                                                                      */

void sqo_rays_reference_camera(uint32_t w, uint32_t h, const float origin[3], float* rays)
{
    float aspect = (float)w / (float)h;
#pragma omp parallel for schedule(static) num_threads(sqo_get_threads())
    for (long long jj = 0; jj < (long long)h; ++jj) {
        uint32_t j = (uint32_t)jj;
        for (uint32_t i = 0; i < w; ++i) {
            /* src/tracer.cpp:207-216 */
            float nx = (((float)i + 0.5f) / (float)w) * 2.0f - 1.0f;
            float ny = (((float)j + 0.5f) / (float)h) * 2.0f - 1.0f;
            nx = nx * aspect;
            float px = nx, py = ny, pz = 1.0f;
            float l2 = px * px + py * py;
            l2 = l2 + pz * pz;
            float len = sqrtf(l2);
            float* r = rays + 8 * ((size_t)j * w + i);
            r[0] = origin[0]; r[1] = origin[1]; r[2] = origin[2]; r[3] = 0.0f;
            r[4] = px / len; r[5] = py / len; r[6] = pz / len; r[7] = 10000.0f;
        }
    }
}

void sqo_pinhole_basis(const float eye[3], const float target[3], const float up[3],
                       float vfov_deg, uint32_t w, uint32_t h, float basis[14])
{
    double f[3], r[3], u[3];
    for (int k = 0; k < 3; ++k) f[k] = (double)target[k] - (double)eye[k];
    double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (int k = 0; k < 3; ++k) f[k] /= fl;
    double up_[3] = {up[0], up[1], up[2]};
    r[0] = f[1] * up_[2] - f[2] * up_[1];
    r[1] = f[2] * up_[0] - f[0] * up_[2];
    r[2] = f[0] * up_[1] - f[1] * up_[0];
    double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int k = 0; k < 3; ++k) r[k] /= rl;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    double th = tan((double)vfov_deg * 3.14159265358979323846 / 360.0);
    for (int k = 0; k < 3; ++k) {
        basis[k] = eye[k];
        basis[3 + k] = (float)f[k];
        basis[6 + k] = (float)r[k];
        basis[9 + k] = (float)u[k];
    }
    basis[12] = (float)(th * (double)w / (double)h);
    basis[13] = (float)th;
}

void sqo_rays_pinhole(uint32_t w, uint32_t h, const float b[14], float* rays)
{
#pragma omp parallel for schedule(static) num_threads(sqo_get_threads())
    for (long long jj = 0; jj < (long long)h; ++jj) {
        uint32_t j = (uint32_t)jj;
        for (uint32_t i = 0; i < w; ++i) {
            float px = (((float)i + 0.5f) / (float)w) * 2.0f - 1.0f;
            float py = (((float)j + 0.5f) / (float)h) * 2.0f - 1.0f;
            px = px * b[12];
            py = py * b[13];
            float d[3];
            for (int k = 0; k < 3; ++k) {
                float s = b[3 + k] + px * b[6 + k];
                d[k] = s + py * b[9 + k];
            }
            float l2 = d[0] * d[0] + d[1] * d[1];
            l2 = l2 + d[2] * d[2];
            float len = sqrtf(l2);
            float* r = rays + 8 * ((size_t)j * w + i);
            r[0] = b[0]; r[1] = b[1]; r[2] = b[2]; r[3] = 0.0f;
            r[4] = d[0] / len; r[5] = d[1] / len; r[6] = d[2] / len; r[7] = FLT_MAX;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* traversal                                                                 */

/* Conservative factor on the exit distance of the closest/any-hit box test:
 * 1 + 2^-21 exceeds 1 + 2*gamma(3) = 1 + 6*2^-24/(1 - 3*2^-24), the bound on
 * the relative error of a slab distance (two roundings plus the reciprocal). */
#define SQ_ROBUST 0x1.000008p+0f

/* intersect_ray_aabb<1> (src/tracer.h:12-35): reference semantics */
static inline int box_ref(const sqo_node1* nd, const float* o, const float* inv, float tmax)
{
    float t1x = (nd->min[0] - o[0]) * inv[0];
    float t2x = (nd->max[0] - o[0]) * inv[0];
    float t1y = (nd->min[1] - o[1]) * inv[1];
    float t2y = (nd->max[1] - o[1]) * inv[1];
    float t1z = (nd->min[2] - o[2]) * inv[2];
    float t2z = (nd->max[2] - o[2]) * inv[2];
    float nx = rmin(t1x, t2x), ny = rmin(t1y, t2y), nz = rmin(t1z, t2z);
    float fx = smax(t1x, t2x), fy = smax(t1y, t2y), fz = smax(t1z, t2z);
    float front = smax(smax(nx, ny), nz);
    float back = rmin(rmin(fx, fy), fz);
    return (back >= front) && (back <= tmax);
}

/* intersect_ray_triangle<1> (src/tracer.h:82-116): Moller-Trumbore hit flag */
static inline int tri_ref(const float* tv, const float* o, const float* d)
{
    const float eps = 0.000000001f;
    float e1[3], e2[3], h[3], s[3], q[3];
    for (int k = 0; k < 3; ++k) { e1[k] = tv[3 + k] - tv[k]; e2[k] = tv[6 + k] - tv[k]; }
    h[0] = d[1] * e2[2] - e2[1] * d[2];
    h[1] = d[2] * e2[0] - e2[2] * d[0];
    h[2] = d[0] * e2[1] - e2[0] * d[1];
    float a = e1[0] * h[0] + e1[1] * h[1];
    a = a + e1[2] * h[2];
    int miss = (a > -eps) && (a < eps);
    float f = 1.0f / a;
    for (int k = 0; k < 3; ++k) s[k] = o[k] - tv[k];
    float sh = s[0] * h[0] + s[1] * h[1];
    sh = sh + s[2] * h[2];
    float u = f * sh;
    miss |= (u < 0.0f) || (u > 1.0f);
    q[0] = s[1] * e1[2] - e1[1] * s[2];
    q[1] = s[2] * e1[0] - e1[2] * s[0];
    q[2] = s[0] * e1[1] - e1[0] * s[1];
    float dq = d[0] * q[0] + d[1] * q[1];
    dq = dq + d[2] * q[2];
    float v = f * dq;
    float uv = u + v;
    miss |= (v < 0.0f) || (uv > 1.0f);
    float eq = e2[0] * q[0] + e2[1] * q[1];
    eq = eq + e2[2] * q[2];
    float t = f * eq;
    return (!miss) && (t > eps);
}

/* per-ray constants of the closest / any-hit tests */
typedef struct ray_pre {
    float o[3], d[3], inv[3], tmin, tmax;
    int kx, ky, kz;
    float sx, sy, sz;
} ray_pre;

static inline void ray_prepare(const float* r, ray_pre* p)
{
    for (int k = 0; k < 3; ++k) { p->o[k] = r[k]; p->d[k] = r[4 + k]; p->inv[k] = 1.0f / r[4 + k]; }
    p->tmin = r[3];
    p->tmax = r[7];
    /* Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1)
     * 2013: shear/scale so the ray runs along +z of a permuted frame. */
    float ax = fabsf(p->d[0]), ay = fabsf(p->d[1]), az = fabsf(p->d[2]);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) { kz = 2; }
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (p->d[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
    p->kx = kx; p->ky = ky; p->kz = kz;
    p->sx = p->d[kx] / p->d[kz];
    p->sy = p->d[ky] / p->d[kz];
    p->sz = 1.0f / p->d[kz];
}

/* slab test for the closest / any-hit modes: near distance in *tn */
static inline int box_robust(const sqo_node1* nd, const ray_pre* r, float tclose, float* tn)
{
    float t0x = (nd->min[0] - r->o[0]) * r->inv[0];
    float t1x = (nd->max[0] - r->o[0]) * r->inv[0];
    float t0y = (nd->min[1] - r->o[1]) * r->inv[1];
    float t1y = (nd->max[1] - r->o[1]) * r->inv[1];
    float t0z = (nd->min[2] - r->o[2]) * r->inv[2];
    float t1z = (nd->max[2] - r->o[2]) * r->inv[2];
    float n = fmaxf(fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z)), r->tmin);
    float f = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    f = f * SQ_ROBUST;
    float lim = tclose * SQ_ROBUST;
    *tn = n;
    return (n <= f) && (n <= lim);
}

/* watertight test; returns 1 and *t when the ray hits in [tmin, tmax] */
static inline int tri_watertight(const float* tv, const ray_pre* r, float tmax, float* tout)
{
    float A[3], B[3], C[3];
    for (int k = 0; k < 3; ++k) { A[k] = tv[k] - r->o[k]; B[k] = tv[3 + k] - r->o[k]; C[k] = tv[6 + k] - r->o[k]; }
    const int kx = r->kx, ky = r->ky, kz = r->kz;
    float Ax = A[kx] - r->sx * A[kz], Ay = A[ky] - r->sy * A[kz];
    float Bx = B[kx] - r->sx * B[kz], By = B[ky] - r->sy * B[kz];
    float Cx = C[kx] - r->sx * C[kz], Cy = C[ky] - r->sy * C[kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double u = (double)Cx * (double)By - (double)Cy * (double)Bx;
        double v = (double)Ax * (double)Cy - (double)Ay * (double)Cx;
        double w = (double)Bx * (double)Ay - (double)By * (double)Ax;
        U = (float)u; V = (float)v; W = (float)w;
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
    float det = U + V;
    det = det + W;
    if (det == 0.0f) return 0;
    float Az = r->sz * A[kz], Bz = r->sz * B[kz], Cz = r->sz * C[kz];
    float T = U * Az + V * Bz;
    T = T + W * Cz;
    float t = T / det;
    if (!(t >= r->tmin) || !(t <= tmax)) return 0;
    *tout = t;
    return 1;
}

#define SQO_STACK 4096

typedef struct se { uint32_t node; float tn; } se;

/* reference traverse() (src/tracer.cpp:47-65) as an explicit stack; the
 * test count and hit flag do not depend on the visit order.               */
static int trace_ref_one(const sqo_node1* nodes, uint32_t root, const float* tris,
                         const float* r, uint32_t* id, uint32_t* tests)
{
    float o[3] = {r[0], r[1], r[2]}, d[3] = {r[4], r[5], r[6]};
    float inv[3] = {1.0f / d[0], 1.0f / d[1], 1.0f / d[2]};
    float tmax = r[7];
    uint32_t stack[SQO_STACK];
    int sp = 0;
    uint32_t cnt = 0;
    int hit = 0;
    /* the root group: traverse(h, root_index, 1, ...) */
    uint32_t gidx = root, gcnt = 1;
    for (;;) {
        for (uint32_t i = 0; i < gcnt; ++i) {
            const sqo_node1* nd = &nodes[gidx + i];
            cnt++;
            if (box_ref(nd, o, inv, tmax)) {
                if (nd->flags & SQO_LEAF) {
                    for (uint32_t k = 0; k < nd->count; ++k)
                        hit |= tri_ref(tris + 9 * (size_t)(nd->child + k), o, d);
                } else {
                    if (sp >= SQO_STACK) { *tests = cnt; *id = hit ? 0u : SQO_NO_HIT; return 1; }
                    stack[sp++] = gidx + i;
                }
            }
        }
        if (sp == 0) break;
        const sqo_node1* g = &nodes[stack[--sp]];
        gidx = g->child;
        gcnt = g->count;
    }
    *tests = cnt;
    *id = hit ? 0u : SQO_NO_HIT;
    return 0;
}

/* Closest / any-hit traversal in near-child order.  A popped node is culled
 * (no test) when its near distance exceeds the current t limit; an internal
 * node tests all its children's boxes in slot order (one test each), sorts
 * the hits by (near distance, slot) and pushes them far to near; a leaf
 * node runs the watertight test on its triangles.  The root box is tested
 * first.                                                                     */
static int trace_closest_one(const sqo_node1* nodes, uint32_t root, const float* tris,
                             const float* r, int anyhit, uint32_t* id, float* tout,
                             uint32_t* tests)
{
    ray_pre rp;
    ray_prepare(r, &rp);
    float best_t = rp.tmax;
    uint32_t best = SQO_NO_HIT;
    uint32_t cnt = 1;
    se stack[SQO_STACK];
    int sp = 0;
    int err = 0;
    float tn;
    if (box_robust(&nodes[root], &rp, best_t, &tn)) { stack[sp].node = root; stack[sp].tn = tn; sp++; }
    while (sp > 0) {
        se e = stack[--sp];
        if (e.tn > best_t * SQ_ROBUST) continue;
        const sqo_node1* nd = &nodes[e.node];
        if (nd->flags & SQO_LEAF) {
            for (uint32_t k = 0; k < nd->count; ++k) {
                uint32_t tri = nd->child + k;
                float t;
                if (tri_watertight(tris + 9 * (size_t)tri, &rp, best_t, &t)) {
                    if (t < best_t || (t == best_t && tri < best)) { best_t = t; best = tri; }
                    if (anyhit) goto done;
                }
            }
            continue;
        }
        se hits[8];
        int nh = 0;
        for (uint32_t i = 0; i < nd->count; ++i) {
            uint32_t c = nd->child + i;
            cnt++;
            if (box_robust(&nodes[c], &rp, best_t, &tn)) {
                if (nh < 8) { hits[nh].node = c; hits[nh].tn = tn; nh++; }
                else { err = 1; break; }
            }
        }
        /* insertion sort by (tn, slot): stable on slot order */
        for (int a = 1; a < nh; ++a) {
            se x = hits[a];
            int b = a - 1;
            while (b >= 0 && hits[b].tn > x.tn) { hits[b + 1] = hits[b]; b--; }
            hits[b + 1] = x;
        }
        if (err) break;
        if (sp + nh > SQO_STACK) { err = 1; break; }
        for (int a = nh - 1; a >= 0; --a) stack[sp++] = hits[a];
    }
done:
    *id = best;
    *tout = (best == SQO_NO_HIT) ? 0.0f : best_t;
    *tests = cnt;
    return err;
}

int sqo_trace(const sqo_node1* nodes, uint32_t root, const float* tris,
              const float* rays, uint32_t nrays, int mode, uint32_t* ids,
              float* ts, uint32_t* tests)
{
    int err = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : err) num_threads(sqo_get_threads())
    for (long long i = 0; i < (long long)nrays; ++i) {
        uint32_t id = SQO_NO_HIT, cnt = 0;
        float t = 0.0f;
        const float* r = rays + 8 * (size_t)i;
        if (mode == SQO_TRACE_REF) err |= trace_ref_one(nodes, root, tris, r, &id, &cnt);
        else err |= trace_closest_one(nodes, root, tris, r, mode == SQO_TRACE_ANYHIT, &id, &t, &cnt);
        if (ids) ids[i] = id;
        if (ts) ts[i] = t;
        if (tests) tests[i] = cnt;
    }
    return err;
}

/* ---------------------------------------------------------------- packets */

/* The reference camera ray through pixel (x, y), src/tracer.cpp:207-216
 * (the same per-pixel arithmetic as trace_packet / trace_bundle,
 * src/tracer.cpp:246-256, 323-329). */
static inline void camera_dir(uint32_t x, uint32_t y, uint32_t w, uint32_t h, float d[3])
{
    float aspect = (float)w / (float)h;
    float nx = (((float)x + 0.5f) / (float)w) * 2.0f - 1.0f;
    float ny = (((float)y + 0.5f) / (float)h) * 2.0f - 1.0f;
    nx = nx * aspect;
    float l2 = nx * nx + ny * ny;
    l2 = l2 + 1.0f * 1.0f;
    float len = sqrtf(l2);
    d[0] = nx / len;
    d[1] = ny / len;
    d[2] = 1.0f / len;
}

#define SQO_PACKET_STACK 128 /* src/tracer.cpp:94 */

/* traverse_packet_stack (src/tracer.cpp:88-123) for a packet of k rays
 * sharing origin o, starting at nodes [index, index + count): a node's
 * children are visited when any ray of the packet hits the node's box; the
 * packet counts one test per node box.  Triangle tests do not change the
 * count.  Returns the count (or UINT32_MAX on a stack overflow). */
static uint32_t packet_tests(const sqo_node1* nodes, uint32_t index, uint32_t count, const float* o,
                             const float (*inv)[3], uint32_t k)
{
    uint32_t st_i[SQO_PACKET_STACK], st_c[SQO_PACKET_STACK];
    uint32_t sp = 1, tests = 0;
    st_i[0] = index;
    st_c[0] = count;
    while (sp > 0) {
        --sp;
        uint32_t bi = st_i[sp], bc = st_c[sp];
        for (uint32_t c = 0; c < bc; ++c) {
            const sqo_node1* nd = &nodes[bi + c];
            int any = 0;
            for (uint32_t r = 0; r < k; ++r) any |= box_ref(nd, o, inv[r], 10000.0f);
            tests++;
            if (any && !(nd->flags & 1u)) {
                if (sp >= SQO_PACKET_STACK) return UINT32_MAX;
                st_i[sp] = nd->child;
                st_c[sp] = nd->count;
                sp++;
            }
        }
    }
    return tests;
}

static inline uint8_t heat_byte(float tests)
{
    float x = tests / 200.0f;
    float m = (x < 1.0f) ? x : 1.0f;
    return (uint8_t)f2u(m * 255.0f);
}

/* trace_packet<k> (src/tracer.cpp:232-281): packets of k = kx * ky rays in
 * kx x ky pixel blocks (kx = floor(sqrt(k))), rays in row order within the
 * block; every pixel of a packet gets (tests / k) / 200 of the packet. */
static int trace_packet_img(const sqo_node1* nodes, uint32_t root, uint32_t w, uint32_t h, const float o[3],
                            uint32_t k, uint8_t* rgb)
{
    uint32_t kx = (uint32_t)floor(sqrt((double)k)), ky = k / kx;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4) num_threads(sqo_get_threads())
    for (long long jj = 0; jj < (long long)h; jj += ky) {
        uint32_t j = (uint32_t)jj;
        float inv[8][3];
        for (uint32_t i = 0; i < w; i += kx) {
            for (uint32_t m = 0; m < k; ++m) {
                float d[3];
                camera_dir(i + m % kx, j + m / kx, w, h, d);
                for (int a = 0; a < 3; ++a) inv[m][a] = 1.0f / d[a];
            }
            uint32_t t = packet_tests(nodes, root, 1, o, (const float (*)[3])inv, k);
            if (t == UINT32_MAX) bad = 1;
            uint8_t b = heat_byte((float)t / (float)k);
            for (uint32_t m = 0; m < k; ++m) {
                size_t px = (size_t)(j + m / kx) * w + i + m % kx;
                rgb[3 * px] = rgb[3 * px + 1] = rgb[3 * px + 2] = b;
            }
        }
    }
    return bad;
}

/* morton_lut (src/tracer.cpp:18-23): k with bits 1 and 2 exchanged */
static inline uint32_t bundle_lut(uint32_t k) { return (k & ~6u) | ((k & 2u) << 1) | ((k & 4u) >> 1); }

/* intersect_bundle_aabb (src/tracer.h:37-80): slabs of the box against the
 * bundle's direction bounds (min, max and their midpoint) from its origin */
static inline void bundle_box(const sqo_node1* nd, const float* pos, const float* imin, const float* imax,
                              const float* imid, int* any_hit, int* mid_hit)
{
    float tmin_mid[3], tmin_any[3], tmax_mid[3], tmax_any[3];
    for (int a = 0; a < 3; ++a) {
        float lo = nd->min[a] - pos[a], hi = nd->max[a] - pos[a];
        float t1a = lo * imin[a], t1b = lo * imax[a], t2a = hi * imin[a], t2b = hi * imax[a];
        float t1 = lo * imid[a], t2 = hi * imid[a];
        float t1min = rmin(t1a, t1b), t1max = smax(t1a, t1b);
        float t2min = rmin(t2a, t2b), t2max = smax(t2a, t2b);
        tmin_mid[a] = rmin(t1, t2);
        tmin_any[a] = rmin(t1min, t2min);
        tmax_mid[a] = smax(t1, t2);
        tmax_any[a] = smax(t1max, t2max);
    }
    float front_mid = rmax(rmax(tmin_mid[0], tmin_mid[1]), tmin_mid[2]);
    float front_any = rmax(rmax(tmin_any[0], tmin_any[1]), tmin_any[2]);
    float back_mid = rmin(rmin(tmax_mid[0], tmax_mid[1]), tmax_mid[2]);
    float back_any = rmin(rmin(tmax_any[0], tmax_any[1]), tmax_any[2]);
    *mid_hit = back_mid >= front_mid;
    *any_hit = back_any >= front_any;
}

/* trace_bundle<k> with packets of 8 (src/tracer.cpp:292-362, traverse_bundle
 * 126-156): tiles of tw x th pixels (tw = floor(sqrt(k))), ray m*8 + n at
 * tile position morton_lut[m*8 + n].  The bundle descends while its
 * midpoint direction hits; where only some directions can hit, each packet
 * of 8 continues alone from that node.  Pixel of packet m:
 * bundle_tests / k + packet_tests[m] / 8. */
static int trace_bundle_img(const sqo_node1* nodes, uint32_t root, uint32_t w, uint32_t h, const float o[3],
                            uint32_t k, uint8_t* rgb)
{
    uint32_t tw = (uint32_t)floor(sqrt((double)k)), th = k / tw, np = k / 8;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 2) num_threads(sqo_get_threads())
    for (long long jj = 0; jj < (long long)h; jj += th) {
        uint32_t j = (uint32_t)jj;
        float inv[64][3];
        uint32_t px[64];
        for (uint32_t i = 0; i < w; i += tw) {
            float dmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, dmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            for (uint32_t r = 0; r < k; ++r) {
                uint32_t v = bundle_lut(r), x = i + v % tw, y = j + v / tw;
                float d[3];
                camera_dir(x, y, w, h, d);
                for (int a = 0; a < 3; ++a) {
                    inv[r][a] = 1.0f / d[a];
                    dmin[a] = rmin(dmin[a], d[a]);
                    dmax[a] = rmax(dmax[a], d[a]);
                }
                px[r] = y * w + x;
            }
            float imin[3], imax[3], imid[3];
            for (int a = 0; a < 3; ++a) {
                imin[a] = 1.0f / dmin[a];
                imax[a] = 1.0f / dmax[a];
                imid[a] = 1.0f / ((dmin[a] + dmax[a]) * 0.5f);
            }
            uint32_t btests = 0, ptests[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            uint32_t st_i[SQO_PACKET_STACK], st_c[SQO_PACKET_STACK], sp = 1;
            st_i[0] = root;
            st_c[0] = 1;
            while (sp > 0) {
                --sp;
                uint32_t bi = st_i[sp], bc = st_c[sp];
                for (uint32_t c = 0; c < bc; ++c) {
                    const sqo_node1* nd = &nodes[bi + c];
                    int any_hit, mid_hit;
                    bundle_box(nd, o, imin, imax, imid, &any_hit, &mid_hit);
                    btests++;
                    if (mid_hit) {
                        if (!(nd->flags & 1u)) {
                            if (sp >= SQO_PACKET_STACK) { bad = 1; break; }
                            st_i[sp] = nd->child;
                            st_c[sp] = nd->count;
                            sp++;
                        }
                    } else if (any_hit) {
                        for (uint32_t m = 0; m < np; ++m) {
                            uint32_t t = packet_tests(nodes, bi + c, 1, o, (const float (*)[3])(inv + 8 * m), 8);
                            if (t == UINT32_MAX) bad = 1;
                            else ptests[m] += t;
                        }
                    }
                }
            }
            for (uint32_t r = 0; r < k; ++r) {
                float t = (float)btests / (float)k + (float)ptests[r / 8] / 8.0f;
                uint8_t b = heat_byte(t);
                rgb[3 * (size_t)px[r]] = rgb[3 * (size_t)px[r] + 1] = rgb[3 * (size_t)px[r] + 2] = b;
            }
        }
    }
    return bad;
}

int sqo_trace_coherent(const sqo_node1* nodes, uint32_t root, uint32_t w, uint32_t h, const float origin[3],
                       int bundle, uint32_t k, uint8_t* rgb)
{
    if (bundle) {
        if (k != 16 && k != 64) return -1;
        uint32_t tw = (uint32_t)floor(sqrt((double)k));
        if (w % tw || h % (k / tw)) return -1;
        return trace_bundle_img(nodes, root, w, h, origin, k, rgb);
    }
    if (k != 1 && k != 2 && k != 4 && k != 8) return -1;
    uint32_t kx = (uint32_t)floor(sqrt((double)k));
    if (w % kx || h % (k / kx)) return -1;
    return trace_packet_img(nodes, root, w, h, origin, k, rgb);
}

void sqo_brute_closest(const float* tris, uint32_t n, const float* rays,
                       uint32_t nrays, uint32_t* ids, float* ts)
{
#pragma omp parallel for schedule(dynamic, 64) num_threads(sqo_get_threads())
    for (long long i = 0; i < (long long)nrays; ++i) {
        ray_pre rp;
        ray_prepare(rays + 8 * (size_t)i, &rp);
        float best_t = rp.tmax;
        uint32_t best = SQO_NO_HIT;
        for (uint32_t k = 0; k < n; ++k) {
            float t;
            if (tri_watertight(tris + 9 * (size_t)k, &rp, best_t, &t)) {
                if (t < best_t || (t == best_t && k < best)) { best_t = t; best = k; }
            }
        }
        ids[i] = best;
        ts[i] = (best == SQO_NO_HIT) ? 0.0f : best_t;
    }
}

void sqo_heatmap(const uint32_t* tests, uint32_t n, uint8_t* rgb)
{
    for (uint32_t i = 0; i < n; ++i) {
        float x = (float)tests[i] / 200.0f;
        float m = (x < 1.0f) ? x : 1.0f;
        float c = m * 255.0f;
        uint8_t b = (uint8_t)f2u(c);
        rgb[3 * (size_t)i] = b;
        rgb[3 * (size_t)i + 1] = b;
        rgb[3 * (size_t)i + 2] = b;
    }
}

/* get_heatmap_colour (src/tracer.cpp:25-45): six stops black, blue, cyan,
 * green, yellow, red; out-of-range values clamp to the end stops; between
 * stops s = x * 5, i0 = floor(s), i2 = ceil(s), fract = i2 - s and the
 * colour is col[i0] * fract + col[i2] * (1 - fract), each operation rounded
 * once (vec3f1's component-wise * and +, src/vec3.h). */
void sqo_heatmap_colour(float x, float rgb[3])
{
    static const float col[6][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}};
    if (x <= 0.0f) { rgb[0] = col[0][0]; rgb[1] = col[0][1]; rgb[2] = col[0][2]; return; }
    if (x >= 1.0f) { rgb[0] = col[5][0]; rgb[1] = col[5][1]; rgb[2] = col[5][2]; return; }
    const float s = x * 5.0f;
    const int i0 = (int)floorf(s);
    const int i2 = (int)ceilf(s);
    const float fract = (float)i2 - s;
    const float rest = 1.0f - fract;
    for (int k = 0; k < 3; ++k) {
        const float a = col[i0][k] * fract;
        const float b = col[i2][k] * rest;
        rgb[k] = a + b;
    }
}

/* The colour-ramp heatmap of box-test values v (counts, or a packet's
 * tests / k): get_heatmap_colour(v / 200) per pixel, each channel
 * (uint8)(c * 255) as the grey heatmap converts (src/tracer.cpp:222-225).  A
 * non-positive or NaN normalised value is black. */
void sqo_heatmap_ramp(const float* values, uint32_t n, uint8_t* rgb)
{
    for (uint32_t i = 0; i < n; ++i) {
        const float x = values[i] / 200.0f;
        float c[3] = {0.0f, 0.0f, 0.0f};
        if (x > 0.0f) sqo_heatmap_colour(x, c);
        for (int k = 0; k < 3; ++k) rgb[3 * (size_t)i + k] = (uint8_t)f2u(c[k] * 255.0f);
    }
}

void sqo_reintersect_f64(const float* tris, const float* rays, uint32_t nrays,
                         const uint32_t* ids, double* t64)
{
    for (uint32_t i = 0; i < nrays; ++i) {
        if (ids[i] == SQO_NO_HIT) { t64[i] = NAN; continue; }
        const float* tv = tris + 9 * (size_t)ids[i];
        const float* r = rays + 8 * (size_t)i;
        double e1[3], e2[3], nrm[3], w[3];
        for (int k = 0; k < 3; ++k) {
            e1[k] = (double)tv[3 + k] - (double)tv[k];
            e2[k] = (double)tv[6 + k] - (double)tv[k];
            w[k] = (double)tv[k] - (double)r[k];
        }
        nrm[0] = e1[1] * e2[2] - e1[2] * e2[1];
        nrm[1] = e1[2] * e2[0] - e1[0] * e2[2];
        nrm[2] = e1[0] * e2[1] - e1[1] * e2[0];
        double num = nrm[0] * w[0] + nrm[1] * w[1] + nrm[2] * w[2];
        double den = nrm[0] * r[4] + nrm[1] * r[5] + nrm[2] * r[6];
        t64[i] = num / den;
    }
}

/* ------------------------------------------------------------------------- */
/* tree inspection                                                           */

uint32_t sqo_canonical_bfs(const sqo_node1* nodes, uint32_t node_count,
                           uint32_t root, sqo_node1* out, uint32_t cap)
{
    if (root >= node_count || cap == 0) return 0xFFFFFFFFu;
    uint32_t* q = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)cap);
    uint32_t head = 0, tail = 0;
    q[tail++] = root;
    while (head < tail) {
        uint32_t idx = q[head];
        sqo_node1 rec = nodes[idx];
        if (!(rec.flags & SQO_LEAF)) {
            uint32_t first = tail;
            if ((uint64_t)rec.child + rec.count > node_count || (uint64_t)tail + rec.count > cap) {
                free(q);
                return 0xFFFFFFFFu;
            }
            for (uint32_t k = 0; k < rec.count; ++k) q[tail++] = rec.child + k;
            rec.child = first;
        }
        out[head] = rec;
        head++;
    }
    free(q);
    return head;
}

uint32_t sqo_leaf_reach(const sqo_node1* nodes, uint32_t node_count, uint32_t root,
                        uint32_t n, uint32_t* counts)
{
    memset(counts, 0, sizeof(uint32_t) * (size_t)n);
    if (root >= node_count) return 0xFFFFFFFFu;
    size_t cap = 1024;
    uint32_t* st = (uint32_t*)malloc(sizeof(uint32_t) * cap);
    size_t sp = 0;
    uint32_t visited = 0;
    st[sp++] = root;
    while (sp > 0) {
        const sqo_node1* nd = &nodes[st[--sp]];
        visited++;
        if (visited > 4u * node_count + 8u) { free(st); return 0xFFFFFFFFu; }
        if (nd->flags & SQO_LEAF) {
            for (uint32_t k = 0; k < nd->count; ++k) {
                uint32_t t = nd->child + k;
                if (t >= n) { free(st); return 0xFFFFFFFFu; }
                counts[t]++;
            }
            continue;
        }
        if ((uint64_t)nd->child + nd->count > node_count) { free(st); return 0xFFFFFFFFu; }
        for (uint32_t k = 0; k < nd->count; ++k) {
            if (sp == cap) { cap *= 2; st = (uint32_t*)realloc(st, sizeof(uint32_t) * cap); }
            st[sp++] = nd->child + k;
        }
    }
    free(st);
    return visited;
}
