/*
 * immintrin.h -- portable stand-in for the x86 intrinsics the Sequoia
 * reference uses, so that its unmodified sources compile on hosts without
 * x86 (the arm64 Grace host of a GB300).  TEST AND BASELINE INFRASTRUCTURE
 * ONLY: oracle/build_ref.sh puts this directory first on the include path
 * and force-includes this file; nothing in the library uses it.
 *
 * Each function follows the operation's published definition in Intel's
 * Intrinsics Guide (the "Operation" pseudo-code: lane widths, NaN and
 * out-of-range behaviour, masking), written here as plain C++ over GCC
 * vector types.  Only the operations the reference calls are provided:
 *   SSE/SSE2/SSE4.2: _mm_set_ps1 _mm_loadu_ps _mm_storeu_ps _mm_add_ps
 *     _mm_sub_ps _mm_mul_ps _mm_div_ps _mm_min_ps _mm_max_ps
 *     _mm_movemask_ps _mm_castps_si128 _mm_castsi128_ps _mm_cvttps_epi32
 *     _mm_slli_epi32 _mm_cmpgt_epi32 _mm_popcnt_u32
 *   AVX/AVX2: _mm_broadcast_ss _mm_permutevar_ps _mm_maskload_epi32
 *     _mm_i32gather_ps _mm_mask_i32gather_ps
 *   BMI2/LZCNT: _pdep_u32 _pdep_u64 _lzcnt_u32 _lzcnt_u64
 *   GCC's x86 move-mask builtins (__builtin_ia32_movmsk*, pmovmskb*), which
 *     the reference's simd<K, T>::movemask names directly.
 * Arithmetic lanes are separate IEEE operations, as the SSE instructions
 * are; build with -ffp-contract=off so the compiler does not fuse them.
 */
#ifndef SQ_X86COMPAT_IMMINTRIN_H
#define SQ_X86COMPAT_IMMINTRIN_H

#include <stdint.h>
#include <string.h>

#ifdef __cplusplus
#include <type_traits>
#endif

/* Same shapes as GCC's own x86 definitions: 4 floats, 2 x 64-bit integer
 * lanes (32-bit lanes are reached through the helpers below).             */
typedef float __m128 __attribute__((__vector_size__(16), __may_alias__));
typedef long long __m128i __attribute__((__vector_size__(16), __may_alias__));

#define SQX_INLINE static inline __attribute__((__always_inline__))

/* 32-bit integer lanes of an __m128i */
SQX_INLINE void sqx_get_i32(__m128i v, int32_t out[4]) { memcpy(out, &v, 16); }
SQX_INLINE __m128i sqx_from_i32(const int32_t in[4])
{
    __m128i v;
    memcpy(&v, in, 16);
    return v;
}
SQX_INLINE uint32_t sqx_float_bits(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

/* ---- SSE: set, load, store, arithmetic --------------------------------- */
SQX_INLINE __m128 _mm_set_ps1(float a) { return (__m128){a, a, a, a}; }
SQX_INLINE __m128 _mm_broadcast_ss(const float* p) { return _mm_set_ps1(*p); }
SQX_INLINE __m128 _mm_loadu_ps(const float* p)
{
    __m128 v;
    memcpy(&v, p, 16);
    return v;
}
SQX_INLINE void _mm_storeu_ps(float* p, __m128 a) { memcpy(p, &a, 16); }

SQX_INLINE __m128 _mm_add_ps(__m128 a, __m128 b)
{
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] + b[i];
    return r;
}
SQX_INLINE __m128 _mm_sub_ps(__m128 a, __m128 b)
{
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] - b[i];
    return r;
}
SQX_INLINE __m128 _mm_mul_ps(__m128 a, __m128 b)
{
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] * b[i];
    return r;
}
SQX_INLINE __m128 _mm_div_ps(__m128 a, __m128 b)
{
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] / b[i];
    return r;
}
/* MINPS / MAXPS: the second operand is returned when the comparison is
 * false, which covers a NaN in either operand and equal zeros.            */
SQX_INLINE __m128 _mm_min_ps(__m128 a, __m128 b)
{
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] < b[i] ? a[i] : b[i];
    return r;
}
SQX_INLINE __m128 _mm_max_ps(__m128 a, __m128 b)
{
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] > b[i] ? a[i] : b[i];
    return r;
}

/* ---- SSE: masks, casts, conversions, integer lanes ---------------------- */
SQX_INLINE int _mm_movemask_ps(__m128 a)
{
    int m = 0;
    for (int i = 0; i < 4; ++i) m |= (int)(sqx_float_bits(a[i]) >> 31) << i;
    return m;
}
SQX_INLINE __m128i _mm_castps_si128(__m128 a)
{
    __m128i r;
    memcpy(&r, &a, 16);
    return r;
}
SQX_INLINE __m128 _mm_castsi128_ps(__m128i a)
{
    __m128 r;
    memcpy(&r, &a, 16);
    return r;
}
/* CVTTPS2DQ: truncation toward zero; NaN and values outside the int32
 * range give the "integer indefinite" value 0x80000000.                   */
SQX_INLINE __m128i _mm_cvttps_epi32(__m128 a)
{
    int32_t r[4];
    for (int i = 0; i < 4; ++i) {
        const float f = a[i];
        r[i] = (f >= -2147483648.0f && f < 2147483648.0f) ? (int32_t)f : (int32_t)0x80000000u;
    }
    return sqx_from_i32(r);
}
/* PSLLD with an immediate: a count above 31 clears the lane.              */
SQX_INLINE __m128i _mm_slli_epi32(__m128i a, int imm)
{
    int32_t v[4];
    sqx_get_i32(a, v);
    for (int i = 0; i < 4; ++i) v[i] = ((unsigned)imm > 31u) ? 0 : (int32_t)((uint32_t)v[i] << imm);
    return sqx_from_i32(v);
}
/* PCMPGTD: signed compare, all ones where a > b.                          */
SQX_INLINE __m128i _mm_cmpgt_epi32(__m128i a, __m128i b)
{
    int32_t x[4], y[4], r[4];
    sqx_get_i32(a, x);
    sqx_get_i32(b, y);
    for (int i = 0; i < 4; ++i) r[i] = x[i] > y[i] ? -1 : 0;
    return sqx_from_i32(r);
}
SQX_INLINE int _mm_popcnt_u32(unsigned int a) { return __builtin_popcount(a); }

/* ---- AVX / AVX2 --------------------------------------------------------- */
/* VPERMILPS (variable): lane i takes a[control.i32[i] & 3].               */
SQX_INLINE __m128 _mm_permutevar_ps(__m128 a, __m128i control)
{
    int32_t c[4];
    sqx_get_i32(control, c);
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[c[i] & 3];
    return r;
}
/* VPMASKMOVD load: lane i is loaded when bit 31 of mask lane i is set,
 * else 0; masked-off lanes are not read.                                  */
SQX_INLINE __m128i _mm_maskload_epi32(const int* mem, __m128i mask)
{
    int32_t m[4], r[4];
    sqx_get_i32(mask, m);
    for (int i = 0; i < 4; ++i) r[i] = (m[i] < 0) ? mem[i] : 0;
    return sqx_from_i32(r);
}
/* VGATHERDPS: lane i reads the float at byte offset vindex.i32[i] * scale
 * from base (scale 1, 2, 4 or 8; the offset is a signed 32-bit index).    */
SQX_INLINE float sqx_gather_one(const float* base, int32_t index, int scale)
{
    float f;
    memcpy(&f, (const char*)base + (int64_t)index * scale, 4);
    return f;
}
SQX_INLINE __m128 _mm_i32gather_ps(const float* base, __m128i vindex, const int scale)
{
    int32_t ix[4];
    sqx_get_i32(vindex, ix);
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = sqx_gather_one(base, ix[i], scale);
    return r;
}
/* Masked gather: lane i is gathered when the sign bit of mask lane i is
 * set, else it keeps src's lane.                                          */
SQX_INLINE __m128 _mm_mask_i32gather_ps(__m128 src, const float* base, __m128i vindex, __m128 mask,
                                        const int scale)
{
    int32_t ix[4];
    sqx_get_i32(vindex, ix);
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = (sqx_float_bits(mask[i]) >> 31) ? sqx_gather_one(base, ix[i], scale) : src[i];
    return r;
}

/* ---- BMI2 / LZCNT ------------------------------------------------------- */
/* PDEP: the low bits of a are deposited, in order, at the set bits of mask. */
SQX_INLINE unsigned int _pdep_u32(unsigned int a, unsigned int mask)
{
    unsigned int r = 0, bit = 1;
    for (unsigned int m = mask; m; m &= m - 1) {
        if (a & bit) r |= m & (~m + 1u);
        bit <<= 1;
    }
    return r;
}
SQX_INLINE unsigned long long _pdep_u64(unsigned long long a, unsigned long long mask)
{
    unsigned long long r = 0, bit = 1;
    for (unsigned long long m = mask; m; m &= m - 1) {
        if (a & bit) r |= m & (~m + 1ull);
        bit <<= 1;
    }
    return r;
}
/* LZCNT: the operand width for a zero operand.                            */
SQX_INLINE unsigned int _lzcnt_u32(unsigned int a) { return a ? (unsigned)__builtin_clz(a) : 32u; }
SQX_INLINE unsigned long long _lzcnt_u64(unsigned long long a) { return a ? (unsigned long long)__builtin_clzll(a) : 64ull; }

/* ---- GCC's x86 move-mask builtins -------------------------------------- */
#ifdef __cplusplus
/* The sign (top) bit of every element of a vector or vector-like object
 * with operator[], element 0 in bit 0: MOVMSKPS/PD and PMOVMSKB.           */
template <class V>
SQX_INLINE int sqx_movemask(const V& v)
{
    typedef typename std::remove_cv<typename std::remove_reference<decltype(v[0])>::type>::type E;
    constexpr int n = (int)(sizeof(V) / sizeof(E));
    int m = 0;
    for (int i = 0; i < n; ++i) {
        E e = v[i];
        unsigned long long bits = 0;
        memcpy(&bits, &e, sizeof(E));
        m |= (int)((bits >> (8 * sizeof(E) - 1)) & 1ull) << i;
    }
    return m;
}
/* variadic: the argument may hold template commas, as in simd<K, char>(a) */
#define __builtin_ia32_pmovmskb(...) sqx_movemask(__VA_ARGS__)
#define __builtin_ia32_pmovmskb128(...) sqx_movemask(__VA_ARGS__)
#define __builtin_ia32_pmovmskb256(...) sqx_movemask(__VA_ARGS__)
#define __builtin_ia32_movmskps(...) sqx_movemask(__VA_ARGS__)
#define __builtin_ia32_movmskps256(...) sqx_movemask(__VA_ARGS__)
#define __builtin_ia32_movmskpd(...) sqx_movemask(__VA_ARGS__)
#define __builtin_ia32_movmskpd256(...) sqx_movemask(__VA_ARGS__)
#endif

#endif /* SQ_X86COMPAT_IMMINTRIN_H */
