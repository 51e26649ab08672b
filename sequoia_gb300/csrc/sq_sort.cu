// sq_sort.cu -- stable LSD radix sort of (key, value) pairs, onesweep style
// (Adinets & Merrill, "Onesweep: A Faster Least Significant Digit Radix Sort
// for GPUs", 2022).
//
// Replaces radix_sort / parallel_counting_sort (src/algorithms.h:41-113):
// both are stable, so the sorted permutation is unique and must match bit for
// bit.  One histogram pass counts every digit of every pass (fused into the
// Morton kernel for builds); then one kernel per digit:
//   - a block takes the next tile from an atomic counter, so tiles are
//     processed in order and a tile's predecessors are always running;
//   - a tile is 16 keys per thread of the block, whose size is chosen per
//     sort: the look-back below is a chain over the tiles, so the fewest
//     tiles that still fill the GPU are the fastest.  Up to 16384 keys per
//     SM the sort is one tile per SM (blocks of 256 to 1024 threads, sized
//     so the tiles cover every SM); beyond that 512-thread blocks, two per
//     SM.  10-bit digits: per-warp counts of 1024 digits leave room for at
//     most 26 warps beside the tile, so one tile per SM up to 13,312 keys
//     per SM and 256-thread blocks beyond;
//   - the pass's digit histogram and the tile's values are copied into
//     shared memory with cp.async while the keys are ranked;
//   - warps rank their keys by digit (stable: items are ranked in index
//     order within the warp, warps in index order within the tile); the lanes
//     sharing a digit come from one ballot per digit bit, which costs the
//     same for any number of distinct digits (a match does not);
//   - the tile publishes its per-digit counts and walks back over earlier
//     tiles' published counts (decoupled look-back) for its global offsets;
//     every wait is bounded and raises SQ_DEVERR_LOOKBACK_TIMEOUT instead of
//     spinning forever;
//   - keys and values are scattered into shared memory in digit order and
//     written out so that consecutive threads write consecutive addresses.
#include "sq_common.cuh"

#include <algorithm>

namespace {

using namespace sq;

constexpr int kItems = 16;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kWindow = 8;  // look-back words loaded per round

// Exclusive scans of two RADIX-value arrays at once (one set of barriers);
// in place is allowed (every input is read before any output is written).
template <int RADIX, int MINBLOCK>
__device__ __forceinline__ void block_exclusive_scan2(const uint32_t* in1, uint32_t* out1, const uint32_t* in2,
                                                      uint32_t* out2, uint32_t* s_tmp)
{
    const int kWarps = (int)(blockDim.x >> 5);
    constexpr int PER = (RADIX + MINBLOCK - 1) / MINBLOCK;
    uint32_t v1[PER], v2[PER];
    uint32_t sum1 = 0, sum2 = 0;
    const int t = threadIdx.x;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int d = t * PER + j;
        v1[j] = (d < RADIX) ? in1[d] : 0u;
        v2[j] = (d < RADIX) ? in2[d] : 0u;
        sum1 += v1[j];
        sum2 += v2[j];
    }
    const int lane = t & 31, warp = t >> 5;
    uint32_t x1 = sum1, x2 = sum2;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y1 = __shfl_up_sync(0xFFFFFFFFu, x1, o);
        const uint32_t y2 = __shfl_up_sync(0xFFFFFFFFu, x2, o);
        if (lane >= o) { x1 += y1; x2 += y2; }
    }
    if (lane == 31) { s_tmp[warp] = x1; s_tmp[32 + warp] = x2; }
    __syncthreads();
    if (warp == 0) {
        uint32_t w1 = (lane < kWarps) ? s_tmp[lane] : 0u, w2 = (lane < kWarps) ? s_tmp[32 + lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y1 = __shfl_up_sync(0xFFFFFFFFu, w1, o);
            const uint32_t y2 = __shfl_up_sync(0xFFFFFFFFu, w2, o);
            if (lane >= o) { w1 += y1; w2 += y2; }
        }
        if (lane < kWarps) { s_tmp[lane] = w1; s_tmp[32 + lane] = w2; }
    }
    __syncthreads();
    uint32_t run1 = x1 - sum1 + (warp > 0 ? s_tmp[warp - 1] : 0u);
    uint32_t run2 = x2 - sum2 + (warp > 0 ? s_tmp[32 + warp - 1] : 0u);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int d = t * PER + j;
        if (d < RADIX) { out1[d] = run1; out2[d] = run2; }
        run1 += v1[j];
        run2 += v2[j];
    }
    __syncthreads();
}

// 4-byte asynchronous copy global -> shared (cp.async, completed by
// cp.async.wait_all in the issuing thread)
__device__ __forceinline__ void cp_async4(uint32_t* dst, const uint32_t* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}

// 16-byte asynchronous copy global -> shared of which the first `bytes`
// (<= 16) are read and the rest zero-filled; both addresses 16-byte aligned
__device__ __forceinline__ void cp_async16(uint32_t* dst, const uint32_t* src, uint32_t bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(bytes)
                 : "memory");
}

// dynamic shared memory of a k_onesweep block of `block` threads
constexpr size_t smem_bytes(int db, int block)
{
    return sizeof(uint32_t) * (2 * (size_t)block * kItems + (size_t)(block / 32) * (1u << db) + 3 * (1u << db) + 64);
}

// MAXB: the largest block the kernel is launched with (any multiple of 32
// from 256 up to MAXB); 64 registers a thread either way.
// iota: each key's value is its index (vin is not read), as in the first
// pass of a build, whose values are the triangle numbers.
template <int DB, int MAXB>
__global__ void __launch_bounds__(MAXB, 1024 / MAXB) k_onesweep(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                     uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                                                     uint32_t shift, const uint32_t* __restrict__ hist,
                                                     uint32_t* __restrict__ lookback, uint32_t* __restrict__ counter,
                                                     uint32_t* err, uint32_t spin_limit, uint32_t tile_base, bool iota)
{
    chain_wait();  // a chained launch (passes follow one another)
    chain_release();
    constexpr int RADIX = 1 << DB;
    constexpr uint32_t MASK = RADIX - 1;
    const int kBlock = (int)blockDim.x, kWarps = kBlock >> 5, kTile = kBlock * kItems;
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* s_keys = smem;
    uint32_t* s_vals = s_keys + kTile;
    uint32_t* s_whist = s_vals + kTile;          // [kWarps][RADIX]
    uint32_t* s_gbase = s_whist + kWarps * RADIX;  // [RADIX]
    uint32_t* s_lexcl = s_gbase + RADIX;           // [RADIX]
    uint32_t* s_bcount = s_lexcl + RADIX;          // [RADIX]
    uint32_t* s_tmp = s_bcount + RADIX;            // [64]
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u) + tile_base;
    for (int j = tid; j < kWarps * RADIX; j += kBlock) s_whist[j] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)kTile;

    // The pass's digit histogram and the tile's values are copied into
    // shared memory asynchronously (cp.async), so that neither load's latency
    // falls after the look-back: the histogram into s_gbase (scanned in
    // place), the values in tile order into s_vals (each thread copies, and
    // later reads back, its own items).  Keys stay in registers through the
    // ranking.
    for (int d = tid; d < RADIX; d += kBlock) cp_async4(s_gbase + d, hist + d);
    uint32_t k[kItems], rk[kItems];
    const uint32_t wbase = base + (uint32_t)warp * (kItems * 32);
    uint32_t* wvals = s_vals + warp * (kItems * 32);
    if (!iota) {
        if ((reinterpret_cast<uintptr_t>(vin) & 15u) == 0) {
            // the warp's kItems * 32 values as 16-byte chunks, four per lane
            // (a chunk past n is not copied; one that straddles it copies
            // only the values before n)
#pragma unroll
            for (int c = 0; c < kItems / 4; ++c) {
                const uint32_t e = (uint32_t)(c * 32 + lane) * 4u;
                if (wbase + e < n) cp_async16(wvals + e, vin + wbase + e, min(4u, n - wbase - e) * 4u);
            }
        } else {
#pragma unroll
            for (int it = 0; it < kItems; ++it) {
                const uint32_t idx = wbase + it * 32 + lane;
                if (idx < n) cp_async4(wvals + it * 32 + lane, vin + idx);
            }
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const uint32_t idx = wbase + it * 32 + lane;
        k[it] = idx < n ? kin[idx] : 0xFFFFFFFFu;
    }
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t* wh = s_whist + warp * RADIX;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const uint32_t idx = wbase + it * 32 + lane;
        const bool valid = idx < n;
        const uint32_t d = valid ? ((k[it] >> shift) & MASK) : (uint32_t)RADIX;
        // lanes with the same digit, from one ballot per digit bit (constant
        // cost; a match over up to 32 distinct digits costs more)
        uint32_t peers = __ballot_sync(0xFFFFFFFFu, valid);
        if (!valid) peers = ~peers;
#pragma unroll
        for (int b = 0; b < DB; ++b) {
            const bool bit = (d >> b) & 1u;
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, bit);
            peers &= bit ? bal : ~bal;
        }
        const int leader = __ffs(peers) - 1;
        uint32_t old = 0;
        // a shared-memory atomic (not a load and a store) so that the
        // iterations do not wait on one another through wh[]
        if (lane == leader && valid) old = atomicAdd(wh + d, __popc(peers));
        old = __shfl_sync(0xFFFFFFFFu, old, leader);
        rk[it] = old + __popc(peers & lt);
    }
    __syncthreads();
    // exclusive offsets across warps per digit; block counts
    for (int d = tid; d < RADIX; d += kBlock) {
        uint32_t run = 0;
        for (int w0 = 0; w0 < kWarps; w0 += 4) {
            uint32_t c[4];  // four independent loads, then the running sum
#pragma unroll
            for (int q = 0; q < 4; ++q) c[q] = w0 + q < kWarps ? s_whist[(w0 + q) * RADIX + d] : 0u;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (w0 + q < kWarps) s_whist[(w0 + q) * RADIX + d] = run;
                run += c[q];
            }
        }
        s_bcount[d] = run;
        st_relaxed_u32(lookback + (size_t)tile * RADIX + d, (tile == 0 ? kFlagInc : kFlagAgg) | run);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    block_exclusive_scan2<RADIX, 256>(s_gbase, s_gbase, s_bcount, s_lexcl, s_tmp);
    // decoupled look-back, one digit per thread (or several).  The words of
    // kWindow predecessors are loaded at once (independent relaxed loads, one
    // memory latency: each word carries its flag and count together, so no
    // ordering with other data is needed) and consumed in order until an
    // inclusive prefix is found; an unpublished word ends the window and is
    // read again.
    for (int d = tid; d < RADIX; d += kBlock) {
        uint32_t excl = 0;
        if (tile > 0) {
            int32_t j = (int32_t)tile - 1;
            uint32_t spins = 0;
            bool done = false;
            while (!done) {
                uint32_t w[kWindow];
#pragma unroll
                for (int q = 0; q < kWindow; ++q)
                    w[q] = (j - q >= 0) ? ld_relaxed_u32(lookback + (size_t)(j - q) * RADIX + d) : kFlagInc;
                int used = 0;
#pragma unroll
                for (int q = 0; q < kWindow; ++q) {
                    if (done || used != q) continue;
                    const uint32_t f = w[q] & ~kCountMask;
                    if (f == 0) continue;  // not yet published: stop this window here
                    excl += w[q] & kCountMask;
                    used = q + 1;
                    if (f == kFlagInc || j - q == 0) done = true;
                }
                j -= used;
                if (!done && used == 0 && ++spins > spin_limit) {
                    raise_error(err, SQ_DEVERR_LOOKBACK_TIMEOUT);
                    break;
                }
            }
            st_relaxed_u32(lookback + (size_t)tile * RADIX + d, kFlagInc | ((excl + s_bcount[d]) & kCountMask));
        }
        s_gbase[d] += excl;
    }
    __syncthreads();
    // local scatter in digit order: keys first (rk becomes the position),
    // then the values, read back from s_vals before any is overwritten
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const uint32_t idx = wbase + it * 32 + lane;
        if (idx < n) {
            const uint32_t d = (k[it] >> shift) & MASK;
            rk[it] += s_lexcl[d] + wh[d];
            s_keys[rk[it]] = k[it];
        }
    }
    if (!iota) {
#pragma unroll
        for (int it = 0; it < kItems; ++it) k[it] = wvals[it * 32 + lane];
        __syncthreads();
    }
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const uint32_t idx = wbase + it * 32 + lane;
        if (idx < n) s_vals[rk[it]] = iota ? idx : k[it];
    }
    __syncthreads();
    // kItems rounds (a tile holds kItems * kBlock keys).  A block that is
    // alone on its SM unrolls them by four so that the rounds' shared-memory
    // loads overlap; with two blocks per SM the plain loop is faster.
    const uint32_t valid_count = min((uint32_t)kTile, n - base);
    auto write_out = [&](uint32_t j) {
        const uint32_t key = s_keys[j];
        const uint32_t d = (key >> shift) & MASK;
        const uint32_t gp = s_gbase[d] + (j - s_lexcl[d]);
        kout[gp] = key;
        vout[gp] = s_vals[j];
    };
    if (kBlock > 512) {
#pragma unroll 4
        for (int it = 0; it < kItems; ++it) {
            const uint32_t j = (uint32_t)(tid + it * kBlock);
            if (j < valid_count) write_out(j);
        }
    } else {
        for (uint32_t j = tid; j < valid_count; j += kBlock) write_out(j);
    }
}

template <int DB>
__global__ void __launch_bounds__(256) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n, uint32_t passes,
                                                   uint32_t* __restrict__ hist)
{
    constexpr int RADIX = 1 << DB;
    extern __shared__ uint32_t s_hist[];
    const int total = (int)passes * RADIX;
    for (int j = threadIdx.x; j < total; j += blockDim.x) s_hist[j] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        for (uint32_t p = 0; p < passes; ++p) atomicAdd(&s_hist[p * RADIX + ((key >> (p * DB)) & (RADIX - 1))], 1u);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < total; j += blockDim.x) {
        const uint32_t c = s_hist[j];
        if (c) atomicAdd(hist + j, c);
    }
}

template <int DB, int MAXB>
void launch_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n, uint32_t shift,
                 const uint32_t* hist, uint32_t* lookback, uint32_t* counter, uint32_t* err, uint32_t spin_limit,
                 uint32_t tile_base, bool iota, uint32_t block, cudaStream_t s)
{
    constexpr size_t max_bytes = smem_bytes(DB, MAXB);
    static_assert(max_bytes <= 227 * 1024, "onesweep tile does not fit in shared memory");
    // the opt-in above 48 KB of dynamic shared memory is a per-device
    // attribute of the function: set it on each device's first use
    static PerDevice<bool> configured;
    configured.get([] {
        cudaFuncSetAttribute(k_onesweep<DB, MAXB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_bytes);
        return true;
    });
    const uint32_t tile = block * kItems;
    const uint32_t tiles = (n + tile - 1) / tile;
    if (tiles <= tile_base) return;
    launch_chained(k_onesweep<DB, MAXB>, dim3(tiles - tile_base), dim3(block), smem_bytes(DB, (int)block), s, kin, vin,
                   kout, vout, n, shift, hist, lookback, counter, err, spin_limit, tile_base, iota);
}

int sms() { return sm_count(); }

// Threads per block of a pass over n keys (see the file comment).
uint32_t sort_block(uint32_t n, uint32_t digit_bits)
{
    // 10-bit digits: the per-warp counts of 1024 digits leave room for at
    // most 26 warps beside the tile in shared memory
    const uint64_t max_warps = digit_bits == 10 ? 26u : 32u;
    const uint64_t per_sm = (uint64_t)sms() * 32u * max_warps * kItems;
    if ((uint64_t)n > per_sm) return digit_bits == 10 ? 256u : 512u;
    // the fewest warps whose tiles (512 keys per warp) cover n in one tile per SM
    const uint64_t warps = ((uint64_t)n + (uint64_t)sms() * 32u * kItems - 1) / ((uint64_t)sms() * 32u * kItems);
    return 32u * (uint32_t)std::min<uint64_t>(max_warps, std::max<uint64_t>(8, warps));
}

}  // namespace

namespace sqk {

uint32_t sort_tile_keys(uint32_t n, uint32_t digit_bits)
{
    return sort_block(n, digit_bits) * (uint32_t)kItems;
}

size_t sort_lookback_words(uint32_t n, uint32_t digit_bits, uint32_t passes)
{
    const uint32_t tile = sort_tile_keys(n, digit_bits);
    const size_t tiles = (n + (size_t)tile - 1) / tile;
    return tiles * ((size_t)1 << digit_bits) * passes;
}

void sort_histogram(const uint32_t* keys, uint32_t n, uint32_t* hist, uint32_t digit_bits, uint32_t passes,
                    cudaStream_t s)
{
    if (n == 0) return;
    const uint32_t grid = min((n + 255) / 256, (uint32_t)sms() * 4u);
    const size_t bytes = sizeof(uint32_t) * passes * ((size_t)1 << digit_bits);
    if (digit_bits == 8) k_sort_hist<8><<<grid, 256, bytes, s>>>(keys, n, passes, hist);
    else if (digit_bits == 10) k_sort_hist<10><<<grid, 256, bytes, s>>>(keys, n, passes, hist);
    else k_sort_hist<6><<<grid, 256, bytes, s>>>(keys, n, passes, hist);
}

int sort_passes(uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b, uint32_t* vals_b, uint32_t n, const uint32_t* hist,
                uint32_t* lookback, uint32_t* counters, uint32_t digit_bits, uint32_t passes, uint32_t* err,
                cudaStream_t s, const SortStall* stall, bool iota_values)
{
    if (n == 0) return 0;
    const size_t radix = (size_t)1 << digit_bits;
    const size_t lb_words = sort_lookback_words(n, digit_bits, 1);
    const uint32_t block = sort_block(n, digit_bits);
    int cur = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        const uint32_t* kin = cur ? keys_b : keys_a;
        const uint32_t* vin = cur ? vals_b : vals_a;
        uint32_t* kout = cur ? keys_a : keys_b;
        uint32_t* vout = cur ? vals_a : vals_b;
        const uint32_t shift = p * digit_bits;
        const uint32_t* h = hist + p * radix;
        uint32_t* lb = lookback + p * lb_words;
        const uint32_t spin = stall ? stall->spin_limit : kSpinLimit;
        const uint32_t tb = (stall && p == 0) ? 1u : 0u;
        const bool iota = iota_values && p == 0;
        if (digit_bits == 10)
            launch_pass<10, 832>(kin, vin, kout, vout, n, shift, h, lb, counters + p, err, spin, tb, iota, block, s);
        else if (digit_bits == 8)
            launch_pass<8, 1024>(kin, vin, kout, vout, n, shift, h, lb, counters + p, err, spin, tb, iota, block, s);
        else
            launch_pass<6, 1024>(kin, vin, kout, vout, n, shift, h, lb, counters + p, err, spin, tb, iota, block, s);
        cur ^= 1;
    }
    return cur;
}

}  // namespace sqk
