// sq_api.cu -- the C ABI of libsequoia_gpu (include/sequoia_gpu.h).
//
// Host side of the library: contexts (one CUDA stream each), a caching device
// allocator so repeated builds and traces do not call cudaMalloc, host/device
// pointer detection, and the build / trace dispatch.
#include "sq_internal.cuh"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

namespace sqi {

sq_status fail(sq_ctx* c, sq_status st, const char* fmt, ...)
{
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return st;
}

static size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Caching allocator: freed blocks are kept by size and reused.
void* dalloc(sq_ctx* c, size_t bytes)
{
    if (c->fail_alloc_in >= 0 && c->fail_alloc_in-- == 0) return nullptr;  // injected failure
    if (bytes == 0) bytes = 256;
    const size_t sz = bytes < (1u << 20) ? round_up(bytes, 256) : round_up(bytes, 2u << 20);
    auto it = c->free_blocks.lower_bound(sz);
    if (it != c->free_blocks.end() && it->first <= sz * 2) {
        void* p = it->second;
        c->live_blocks[p] = it->first;
        c->free_blocks.erase(it);
        return p;
    }
    void* p = nullptr;
    if (cudaMalloc(&p, sz) != cudaSuccess) {
        cudaGetLastError();
        // release the cache and retry once
        cudaStreamSynchronize(c->stream);
        for (auto& kv : c->free_blocks) cudaFree(kv.second);
        c->free_blocks.clear();
        if (cudaMalloc(&p, sz) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    c->live_blocks[p] = sz;
    return p;
}

void dfree(sq_ctx* c, void* p)
{
    if (!p) return;
    auto it = c->live_blocks.find(p);
    if (it == c->live_blocks.end()) return;
    c->free_blocks.emplace(it->second, p);
    c->live_blocks.erase(it);
}

bool is_device_ptr(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The device address of page-locked host memory (cudaHostAlloc /
// cudaHostRegister), or null for any other pointer.  Kernels write results
// there directly: the transfer to the host overlaps the kernel instead of
// following it as a copy.
void* pinned_device_alias(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void camera_params(const sq_ray_source& rs, float* cam)
{
    if (rs.kind == SQ_RAYS_REFERENCE_CAMERA) {
        for (int k = 0; k < 3; ++k) cam[k] = rs.origin[k];
        return;
    }
    // pinhole basis in double, rounded to float: eye, forward, right, up,
    // then the half extents of the image plane at distance 1
    double f[3], r[3], u[3], up[3];
    for (int k = 0; k < 3; ++k) { f[k] = (double)rs.target[k] - (double)rs.origin[k]; up[k] = rs.up[k]; }
    const double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& x : f) x /= fl;
    r[0] = f[1] * up[2] - f[2] * up[1];
    r[1] = f[2] * up[0] - f[0] * up[2];
    r[2] = f[0] * up[1] - f[1] * up[0];
    const double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (double& x : r) x /= rl;
    u[0] = r[1] * f[2] - r[2] * f[1];
    u[1] = r[2] * f[0] - r[0] * f[2];
    u[2] = r[0] * f[1] - r[1] * f[0];
    const double th = tan((double)rs.vfov_deg * 3.14159265358979323846 / 360.0);
    for (int k = 0; k < 3; ++k) {
        cam[k] = rs.origin[k];
        cam[3 + k] = (float)f[k];
        cam[6 + k] = (float)r[k];
        cam[9 + k] = (float)u[k];
    }
    cam[12] = (float)(th * (double)rs.width / (double)rs.height);
    cam[13] = (float)th;
}

// Streams and events of banded traces, created on the first banded call.
bool band_resources(sq_ctx* c)
{
    if (c->copy_stream) return true;
    bool ok = cudaStreamCreateWithFlags(&c->band_stream[0], cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&c->band_stream[1], cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&c->band_fork, cudaEventDisableTiming) == cudaSuccess;
    for (auto& e : c->band_done) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    for (auto& e : c->band_join) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) cudaGetLastError();
    return ok;
}

sq_status check_device_error(sq_ctx* c, uint32_t* bits_out)
{
    uint32_t bits = 0;
    SQ_CUDA(c, cudaMemcpyAsync(&bits, c->ctrl, sizeof bits, cudaMemcpyDeviceToHost, c->stream));
    SQ_CUDA(c, cudaStreamSynchronize(c->stream));
    if (bits_out) *bits_out = bits;
    if (bits) {
        SQ_CUDA(c, cudaMemsetAsync(c->ctrl, 0, sizeof(uint32_t), c->stream));
        SQ_CUDA(c, cudaStreamSynchronize(c->stream));
        return fail(c, SQ_ERR_DEVICE, "device error word 0x%x (1 stack overflow, 2 look-back timeout, 4 topology, 8 SAH queue, 16 node count)", bits);
    }
    return SQ_OK;
}

}  // namespace sqi

namespace {

using namespace sqi;

uint32_t sort_passes_for(uint32_t key_bits, uint32_t digit_bits) { return (key_bits + digit_bits - 1) / digit_bits; }

sq_status new_bvh(sq_ctx* c, uint32_t n, uint32_t cap, sq_bvh** out)
{
    sq_bvh* b = new (std::nothrow) sq_bvh;
    if (!b) return fail(c, SQ_ERR_OOM, "host allocation failed");
    b->ctx = c;
    b->n = n;
    b->cap = cap;
    b->nodes = static_cast<Node*>(dalloc(c, sizeof(Node) * (size_t)cap));
    if (!b->nodes) {
        delete b;
        return fail(c, SQ_ERR_OOM, "device allocation of %u nodes failed", cap);
    }
    *out = b;
    return SQ_OK;
}

// tris argument -> device pointer (copy if host)
sq_status device_tris(sq_ctx* c, const sq_triangle* tris, uint32_t n, const float** dev, float** owned)
{
    *owned = nullptr;
    if (n == 0) { *dev = nullptr; return SQ_OK; }
    if (is_device_ptr(tris)) {
        *dev = reinterpret_cast<const float*>(tris);
        return SQ_OK;
    }
    float* d = static_cast<float*>(dalloc(c, sizeof(float) * 9ull * n));
    if (!d) return fail(c, SQ_ERR_OOM, "device allocation for %u triangles failed", n);
    SQ_CUDA(c, cudaMemcpyAsync(d, tris, sizeof(float) * 9ull * n, cudaMemcpyHostToDevice, c->stream));
    *dev = d;
    *owned = d;
    return SQ_OK;
}

// Morton / LBVH build into b (nodes allocated, tris set).
sq_status build_morton(sq_ctx* c, sq_bvh* b, const sq_build_params& p)
{
    const uint32_t n = b->n;
    uint32_t db = p.sort_digit_bits ? p.sort_digit_bits : 8u;
    if (db != 6 && db != 8 && db != 10) return fail(c, SQ_ERR_INVALID, "sort_digit_bits must be 6, 8 or 10");
    const uint32_t passes = sort_passes_for(30, db);
    const size_t radix = (size_t)1 << db;
    const size_t lb_words = sqk::sort_lookback_words(n, db, passes);
    // zeroed region: box_ord[8] | hist[passes*radix] | counters[8] | lookback | flags[n]
    const size_t z_box = 0, z_hist = 8, z_ctr = z_hist + passes * radix, z_lb = z_ctr + 8, z_flags = z_lb + lb_words;
    const size_t z_words = z_flags + n;
    uint32_t* zero = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * z_words));
    uint32_t* alt = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * 2ull * n));
    float4* info = static_cast<float4*>(dalloc(c, sizeof(float4) * 6ull * n));  // 2 x 48 B per boundary
    b->codes = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * (size_t)n));
    b->perm = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * (size_t)n));
    if (!zero || !alt || !info || !b->codes || !b->perm) {
        dfree(c, zero); dfree(c, alt); dfree(c, info);
        return fail(c, SQ_ERR_OOM, "device workspace allocation failed (n=%u)", n);
    }
    uint32_t* err = c->ctrl;
    cudaStream_t s = c->stream;
    SQ_CUDA(c, cudaEventRecord(c->ev[0], s));
    SQ_CUDA(c, cudaMemsetAsync(zero, 0, sizeof(uint32_t) * z_words, s));
    // sorted result lands in buffer A when the pass count is even
    uint32_t *ka, *va, *kb, *vb;
    if (passes % 2 == 0) { ka = b->codes; va = b->perm; kb = alt; vb = alt + n; }
    else { ka = alt; va = alt + n; kb = b->codes; vb = b->perm; }
    sqk::scene_bounds(b->tris, n, p.morton_bounds, zero + z_box, err, s);
    // the values are the triangle numbers: the sort's first pass generates
    // them instead of reading them
    sqk::morton_codes(b->tris, n, p.morton_bounds, zero + z_box, ka, nullptr, zero + z_hist, db, passes, err, s);
    SQ_CUDA(c, cudaEventRecord(c->ev[1], s));
    sqk::sort_passes(ka, va, kb, vb, n, zero + z_hist, zero + z_lb, zero + z_ctr, db, passes, err, s, nullptr, true);
    SQ_CUDA(c, cudaEventRecord(c->ev[2], s));
    // the sort's second buffer is free now: it lists the climb's open nodes;
    // box_ord leaves words 6 and 7 of the zeroed region for their count
    sqk::lbvh_climb(b->codes, b->perm, b->tris, n, b->nodes, zero + z_flags, info, alt, zero + z_box + 6, err, s);
    SQ_CUDA(c, cudaEventRecord(c->ev[3], s));
    SQ_CUDA(c, cudaGetLastError());
    c->build_timed = true;
    dfree(c, zero);
    dfree(c, alt);
    dfree(c, info);
    b->root = 0;
    return SQ_OK;
}

// Morton build over 60-bit codes (Builder::build_hierarchy_morton2,
// src/builder.cpp:2510-2544).  The 64-bit keys are sorted by two stable
// 32-bit sorts, the low words first (with the triangle index) and then the
// high words in that order (with the position): LSD order, so the result
// is the reference's stable 64-bit sort.  The climb then runs on the
// combined 64-bit codes.
sq_status build_morton64(sq_ctx* c, sq_bvh* b, const sq_build_params& p)
{
    const uint32_t n = b->n;
    if (p.sort_digit_bits && p.sort_digit_bits != 8)
        return fail(c, SQ_ERR_UNSUPPORTED, "60-bit Morton builds sort with 8-bit digits");
    const uint32_t db = 8, passes = 4;
    const size_t radix = 256;
    const size_t lb_words = sqk::sort_lookback_words(n, db, passes);
    // zeroed: box_ord[8] | hist[8 * 256] | counters[16] | look-back (2 stages) | flags[n]
    const size_t z_box = 0, z_hist = 8, z_ctr = z_hist + 8 * radix, z_lb = z_ctr + 16, z_flags = z_lb + 2 * lb_words;
    const size_t z_words = z_flags + n;
    uint32_t* zero = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * z_words));
    uint32_t* work = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * 9ull * n));
    float4* info = static_cast<float4*>(dalloc(c, sizeof(float4) * 6ull * n));
    b->codes64 = static_cast<uint64_t*>(dalloc(c, sizeof(uint64_t) * (size_t)n));
    b->perm = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * (size_t)n));
    if (!zero || !work || !info || !b->codes64 || !b->perm) {
        dfree(c, zero); dfree(c, work); dfree(c, info);
        return fail(c, SQ_ERR_OOM, "device workspace allocation failed (n=%u)", n);
    }
    uint32_t *lo = work, *hi = work + n, *vals = work + 2ull * n, *alt = work + 3ull * n;  // alt: 2n
    uint32_t *hi1 = work + 5ull * n, *pos = work + 6ull * n, *alt2 = work + 7ull * n;     // alt2: 2n
    uint32_t* err = c->ctrl;
    cudaStream_t s = c->stream;
    SQ_CUDA(c, cudaEventRecord(c->ev[0], s));
    SQ_CUDA(c, cudaMemsetAsync(zero, 0, sizeof(uint32_t) * z_words, s));
    sqk::scene_bounds(b->tris, n, p.morton_bounds, zero + z_box, err, s);
    sqk::morton_codes64(b->tris, n, zero + z_box, lo, hi, vals, zero + z_hist, s);
    SQ_CUDA(c, cudaEventRecord(c->ev[1], s));
    // an even number of passes leaves each stage's result in its input buffers
    sqk::sort_passes(lo, vals, alt, alt + n, n, zero + z_hist, zero + z_lb, zero + z_ctr, db, passes, err, s);
    sqk::gather_high(hi, vals, n, hi1, pos, s);
    sqk::sort_passes(hi1, pos, alt2, alt2 + n, n, zero + z_hist + 4 * radix, zero + z_lb + lb_words, zero + z_ctr + 8,
                     db, passes, err, s);
    sqk::combine64(hi1, pos, lo, vals, n, b->codes64, b->perm, s);
    SQ_CUDA(c, cudaEventRecord(c->ev[2], s));
    sqk::lbvh_climb64(b->codes64, b->perm, b->tris, n, b->nodes, zero + z_flags, info, alt, zero + z_box + 6, err, s);
    SQ_CUDA(c, cudaEventRecord(c->ev[3], s));
    SQ_CUDA(c, cudaGetLastError());
    c->build_timed = true;
    dfree(c, zero);
    dfree(c, work);
    dfree(c, info);
    b->root = 0;
    return SQ_OK;
}

// Binned SAH or grid build into b.
sq_status build_sah(sq_ctx* c, sq_bvh* b, const sq_build_params& p, int grid)
{
    const uint32_t n = b->n;
    const uint32_t nb = p.sah_bins ? p.sah_bins : 8u;
    const uint32_t leaf = p.leaf_size ? p.leaf_size : 8u;
    if (nb < 2 || nb > 32) return fail(c, SQ_ERR_INVALID, "sah_bins must be 2..32");
    void* ws = dalloc(c, sqk::sah_workspace_bytes(n));
    uint32_t* sortb = nullptr;
    uint32_t* zero = nullptr;
    size_t z_words = 0;
    if (grid) {
        sortb = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * 4ull * n));
        z_words = 8 + sqk::sort_lookback_words(n, 6, 1);
        zero = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * z_words));
    }
    float* scene = static_cast<float*>(dalloc(c, 64));
    if (!ws || (grid && (!sortb || !zero)) || !scene) {
        dfree(c, ws); dfree(c, sortb); dfree(c, zero); dfree(c, scene);
        return fail(c, SQ_ERR_OOM, "SAH workspace allocation failed (n=%u)", n);
    }
    cudaStream_t s = c->stream;
    SQ_CUDA(c, cudaEventRecord(c->ev[0], s));
    if (grid) SQ_CUDA(c, cudaMemsetAsync(zero, 0, sizeof(uint32_t) * z_words, s));
    SQ_CUDA(c, cudaEventRecord(c->ev[1], s));
    const int rc = sqk::build_sah(b->tris, n, nb, leaf, grid, p.flags & SQ_BUILD_GRID_SCENE_BOUNDS, b->nodes, scene, ws,
                                  sortb, grid ? sortb + n : nullptr, grid ? sortb + 2ull * n : nullptr,
                                  grid ? sortb + 3ull * n : nullptr, grid ? zero + 8 : nullptr, zero, c->ctrl,
                                  c->host_ctl, s);
    if (rc != 0) {
        dfree(c, ws); dfree(c, sortb); dfree(c, zero); dfree(c, scene);
        return fail(c, SQ_ERR_CUDA, "SAH build: %s", cudaGetErrorString((cudaError_t)rc));
    }
    SQ_CUDA(c, cudaEventRecord(c->ev[2], s));
    SQ_CUDA(c, cudaEventRecord(c->ev[3], s));
    SQ_CUDA(c, cudaMemcpyAsync(c->host_ctl + 8, scene, 6 * sizeof(float), cudaMemcpyDeviceToHost, s));
    SQ_CUDA(c, cudaStreamSynchronize(s));
    memcpy(b->scene, c->host_ctl + 8, 6 * sizeof(float));
    c->build_timed = true;
    dfree(c, ws); dfree(c, sortb); dfree(c, zero); dfree(c, scene);
    b->root = 0;
    return SQ_OK;
}

sq_status build_wide(sq_ctx* c, sq_bvh* b)
{
    const uint32_t n = b->n;
    b->nodes8 = dalloc(c, sqk::bvh8_node_bytes(n));
    b->tris8 = dalloc(c, sqk::bvh8_tri_bytes(n));
    b->ws8 = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * sqk::bvh8_ws_words(n)));
    if (!b->nodes8 || !b->tris8 || !b->ws8) return fail(c, SQ_ERR_OOM, "8-wide BVH allocation failed (n=%u)", n);
    b->meta8 = static_cast<uint32_t*>(dalloc(c, 2 * sizeof(uint32_t)));
    if (!b->meta8) return fail(c, SQ_ERR_OOM, "8-wide BVH allocation failed (n=%u)", n);
    sqk::BarrierStall stall{c->stall_barrier ? c->stall_barrier - 1u : 0u};
    const bool stalled = c->stall_barrier != 0;
    c->stall_barrier = 0;
    const int rc = sqk::build_bvh8(b->nodes, b->root, b->leaf0, b->tris, n, b->nodes8, b->tris8, b->ws8, c->host_ctl,
                                   c->ctrl, c->stream, b->meta8, stalled ? &stall : nullptr);
    if (rc != 0) return fail(c, SQ_ERR_CUDA, "8-wide collapse: %s", cudaGetErrorString((cudaError_t)rc));
    b->launches8 = c->host_ctl[4];
    if (!c->host_ctl[5]) {
        // the per-level path read both counts back already
        b->n8 = c->host_ctl[0];
        b->levels8 = c->host_ctl[3];
        dfree(c, b->meta8);
        b->meta8 = nullptr;
    }
    dfree(c, b->ws8);
    b->ws8 = nullptr;
    return SQ_OK;
}

}  // namespace

using namespace sqi;

extern "C" {

uint32_t sq_abi_version(void) { return SQ_ABI_VERSION; }

sq_status sq_create(sq_ctx** out, const sq_options* options)
{
    if (!out) return SQ_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return SQ_ERR_NO_DEVICE;
    }
    sq_ctx* c = new (std::nothrow) sq_ctx;
    if (!c) return SQ_ERR_OOM;
    c->device = options ? options->device : 0;
    if (c->device < 0 || c->device >= count) {
        delete c;
        return SQ_ERR_INVALID;
    }
    Guard g(c->device);
    if (options && (options->stream || (options->flags & SQ_OPT_EXTERNAL_STREAM))) {
        c->stream = static_cast<cudaStream_t>(options->stream);
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            return SQ_ERR_CUDA;
        }
        c->own_stream = true;
    }
    if (cudaMalloc(&c->ctrl, 64) != cudaSuccess || cudaMemset(c->ctrl, 0, 64) != cudaSuccess) {
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
        return SQ_ERR_OOM;
    }
    for (auto& e : c->ev) cudaEventCreate(&e);
    if (cudaHostAlloc(reinterpret_cast<void**>(&c->host_ctl), 64, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        sq_destroy(c);
        return SQ_ERR_OOM;
    }
    *out = c;
    return SQ_OK;
}

sq_status sq_destroy(sq_ctx* c)
{
    if (!c) return SQ_ERR_INVALID;
    Guard g(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& kv : c->free_blocks) cudaFree(kv.second);
    for (auto& kv : c->live_blocks) cudaFree(kv.first);
    for (auto& e : c->ev) cudaEventDestroy(e);
    for (auto& st : c->band_stream)
        if (st) cudaStreamDestroy(st);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->band_fork) cudaEventDestroy(c->band_fork);
    for (auto& e : c->band_done)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->band_join)
        if (e) cudaEventDestroy(e);
    cudaFree(c->ctrl);
    if (c->host_ctl) cudaFreeHost(c->host_ctl);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return SQ_OK;
}

const char* sq_last_error(const sq_ctx* c) { return c ? c->err.c_str() : "null context"; }

sq_status sq_sync(sq_ctx* c, uint32_t* device_error)
{
    if (!c) return SQ_ERR_INVALID;
    Guard g(c->device);
    return check_device_error(c, device_error);
}

sq_status sq_build(sq_ctx* c, const sq_triangle* tris, uint32_t n, const sq_build_params* params, sq_bvh** out)
{
    if (!c || !out || !params) return fail(c, SQ_ERR_INVALID, "sq_build: null argument");
    *out = nullptr;
    // size limits come before the triangle pointer is looked at, so an
    // oversize request is refused whatever buffer comes with it
    if (n > (1u << 29)) return fail(c, SQ_ERR_INVALID, "sq_build: n=%u exceeds 2^29", n);
    // the 8-wide traversal's leaf entries hold a 27-bit first-triangle index
    if ((params->flags & SQ_BUILD_WIDE8) && n > sqk::kWide8MaxTris)
        return fail(c, SQ_ERR_UNSUPPORTED, "sq_build: the 8-wide BVH takes at most 2^27 triangles (n=%u)", n);
    if (n > 0 && !tris) return fail(c, SQ_ERR_INVALID, "sq_build: null triangles");
    Guard g(c->device);
    sq_build_params p = *params;
    if (p.kind != SQ_BUILDER_MORTON && p.kind != SQ_BUILDER_SAH && p.kind != SQ_BUILDER_GRID)
        return fail(c, SQ_ERR_INVALID, "sq_build: unknown builder kind %u", p.kind);
    const uint32_t cap = (p.kind == SQ_BUILDER_GRID ? 128u : 0u) + 3u * n + 2u;
    sq_bvh* b = nullptr;
    sq_status st = new_bvh(c, n, cap, &b);
    if (st != SQ_OK) return st;
    b->kind = p.kind;
    st = device_tris(c, tris, n, &b->tris, &b->tris_own);
    if (st != SQ_OK) { sq_bvh_free(b); return st; }
    if (n == 0) {
        Node root;
        root.mnx = root.mny = root.mnz = FLT_MAX;
        root.mxx = root.mxy = root.mxz = -FLT_MAX;
        root.count_flags = sq::pack_cf(0, 0);
        root.child = 2;
        SQ_CUDA(c, cudaMemcpyAsync(b->nodes, &root, sizeof root, cudaMemcpyHostToDevice, c->stream));
        SQ_CUDA(c, cudaStreamSynchronize(c->stream));
        b->leaf0 = 2u;
        if (p.flags & SQ_BUILD_WIDE8) {
            st = build_wide(c, b);  // one wide root without children
            if (st != SQ_OK) { sq_bvh_free(b); return st; }
        }
        *out = b;
        return SQ_OK;
    }
    b->leaf0 = (p.kind == SQ_BUILDER_GRID ? 128u : 0u) + 2u * n + 2u;
    if (p.kind == SQ_BUILDER_MORTON) st = (p.flags & SQ_BUILD_MORTON64) ? build_morton64(c, b, p) : build_morton(c, b, p);
    else st = build_sah(c, b, p, p.kind == SQ_BUILDER_GRID);
    if (st != SQ_OK) { sq_bvh_free(b); return st; }
    if (p.flags & SQ_BUILD_WIDE8) {
        st = build_wide(c, b);
        if (st != SQ_OK) { sq_bvh_free(b); return st; }
    }
    SQ_CUDA(c, cudaEventRecord(c->ev[6], c->stream));
    *out = b;
    return SQ_OK;
}

sq_status sq_bvh_free(sq_bvh* b)
{
    if (!b) return SQ_ERR_INVALID;
    sq_ctx* c = b->ctx;
    Guard g(c->device);
    dfree(c, b->nodes);
    dfree(c, b->tris_own);
    dfree(c, b->codes);
    dfree(c, b->codes64);
    dfree(c, b->perm);
    dfree(c, b->nodes8);
    dfree(c, b->tris8);
    dfree(c, b->ws8);
    dfree(c, b->meta8);
    delete b;
    return SQ_OK;
}

sq_status sq_bvh_get_info(const sq_bvh* b_const, sq_bvh_info* info)
{
    if (!b_const || !info) return SQ_ERR_INVALID;
    sq_bvh* b = const_cast<sq_bvh*>(b_const);
    if (b->meta8) {
        // the collapse left its node and level counts on the device
        uint32_t m[2] = {0, 0};
        Guard g(b->ctx->device);
        if (cudaMemcpyAsync(m, b->meta8, sizeof m, cudaMemcpyDeviceToHost, b->ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(b->ctx->stream) != cudaSuccess)
            return fail(b->ctx, SQ_ERR_CUDA, "sq_bvh_get_info: %s", cudaGetErrorString(cudaGetLastError()));
        b->n8 = m[0];
        b->levels8 = m[1];
        dfree(b->ctx, b->meta8);
        b->meta8 = nullptr;
    }
    info->node_capacity = b->cap;
    info->root = b->root;
    info->tri_count = b->n;
    info->kind = b->kind;
    for (int k = 0; k < 3; ++k) { info->scene_min[k] = b->scene[k]; info->scene_max[k] = b->scene[3 + k]; }
    info->wide_nodes = b->n8;
    info->wide_levels = b->levels8;
    info->wide_launches = b->launches8;
    return SQ_OK;
}

sq_status sq_bvh_export_node1(sq_bvh* b, sq_node1* nodes, uint32_t cap, uint32_t* node_count, uint32_t* root)
{
    if (!b) return SQ_ERR_INVALID;
    sq_ctx* c = b->ctx;
    Guard g(c->device);
    if (node_count) *node_count = b->cap;
    if (root) *root = b->root;
    if (nodes) {
        if (cap < b->cap) return fail(c, SQ_ERR_INVALID, "export: capacity %u < %u nodes", cap, b->cap);
        SQ_CUDA(c, cudaMemcpyAsync(nodes, b->nodes, sizeof(Node) * (size_t)b->cap, cudaMemcpyDefault, c->stream));
    }
    return check_device_error(c, nullptr);
}

sq_status sq_bvh_export_sorted(sq_bvh* b, uint32_t* codes, uint32_t* perm)
{
    if (!b) return SQ_ERR_INVALID;
    sq_ctx* c = b->ctx;
    Guard g(c->device);
    if (!b->codes) return fail(c, SQ_ERR_INVALID, "export_sorted: not a 30-bit Morton build");
    if (codes) SQ_CUDA(c, cudaMemcpyAsync(codes, b->codes, sizeof(uint32_t) * (size_t)b->n, cudaMemcpyDefault, c->stream));
    if (perm) SQ_CUDA(c, cudaMemcpyAsync(perm, b->perm, sizeof(uint32_t) * (size_t)b->n, cudaMemcpyDefault, c->stream));
    return check_device_error(c, nullptr);
}

sq_status sq_bvh_export_sorted64(sq_bvh* b, uint64_t* codes, uint32_t* perm)
{
    if (!b) return SQ_ERR_INVALID;
    sq_ctx* c = b->ctx;
    Guard g(c->device);
    if (!b->codes64) return fail(c, SQ_ERR_INVALID, "export_sorted64: not a 60-bit Morton build");
    if (codes) SQ_CUDA(c, cudaMemcpyAsync(codes, b->codes64, sizeof(uint64_t) * (size_t)b->n, cudaMemcpyDefault,
                                          c->stream));
    if (perm) SQ_CUDA(c, cudaMemcpyAsync(perm, b->perm, sizeof(uint32_t) * (size_t)b->n, cudaMemcpyDefault, c->stream));
    return check_device_error(c, nullptr);
}

sq_status sq_bvh_import_node1(sq_ctx* c, const sq_node1* nodes, uint32_t node_count, uint32_t root,
                              const sq_triangle* tris, uint32_t n, sq_bvh** out)
{
    if (!c || !nodes || !out || (n > 0 && !tris) || root >= node_count)
        return fail(c, SQ_ERR_INVALID, "sq_bvh_import_node1: bad argument");
    *out = nullptr;
    Guard g(c->device);
    sq_bvh* b = nullptr;
    sq_status st = new_bvh(c, n, node_count, &b);
    if (st != SQ_OK) return st;
    b->root = root;
    b->kind = 0xFFFFFFFFu;
    SQ_CUDA(c, cudaMemcpyAsync(b->nodes, nodes, sizeof(Node) * (size_t)node_count, cudaMemcpyDefault, c->stream));
    if (n) {
        float* d = static_cast<float*>(dalloc(c, sizeof(float) * 9ull * n));
        if (!d) { sq_bvh_free(b); return fail(c, SQ_ERR_OOM, "import: triangle allocation failed"); }
        SQ_CUDA(c, cudaMemcpyAsync(d, tris, sizeof(float) * 9ull * n, cudaMemcpyDefault, c->stream));
        b->tris = d;
        b->tris_own = d;
    }
    SQ_CUDA(c, cudaStreamSynchronize(c->stream));
    *out = b;
    return SQ_OK;
}

sq_status sq_morton_codes(sq_ctx* c, const sq_triangle* tris, uint32_t n, uint32_t bounds_mode, uint32_t* codes,
                          float* scene_box)
{
    if (!c || (n > 0 && (!tris || !codes))) return fail(c, SQ_ERR_INVALID, "sq_morton_codes: null argument");
    Guard g(c->device);
    if (n == 0) return SQ_OK;
    const float* dt = nullptr;
    float* owned = nullptr;
    sq_status st = device_tris(c, tris, n, &dt, &owned);
    if (st != SQ_OK) return st;
    const uint32_t passes = 4, db = 8;
    const size_t z_words = 8 + passes * 256;
    uint32_t* zero = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * z_words));
    uint32_t* keys = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * 2ull * n));
    if (!zero || !keys) { dfree(c, zero); dfree(c, keys); dfree(c, owned); return fail(c, SQ_ERR_OOM, "allocation failed"); }
    cudaStream_t s = c->stream;
    SQ_CUDA(c, cudaMemsetAsync(zero, 0, sizeof(uint32_t) * z_words, s));
    sqk::scene_bounds(dt, n, bounds_mode, zero, c->ctrl, s);
    sqk::morton_codes(dt, n, bounds_mode, zero, keys, keys + n, zero + 8, db, passes, c->ctrl, s);
    SQ_CUDA(c, cudaMemcpyAsync(codes, keys, sizeof(uint32_t) * (size_t)n, cudaMemcpyDefault, s));
    uint32_t ord[6];
    SQ_CUDA(c, cudaMemcpyAsync(ord, zero, sizeof ord, cudaMemcpyDeviceToHost, s));
    st = check_device_error(c, nullptr);
    if (scene_box && st == SQ_OK) {
        float box[6];
        for (int k = 0; k < 3; ++k) {
            box[k] = -sq::ordered_to_float(ord[k]);
            box[3 + k] = sq::ordered_to_float(ord[3 + k]);
        }
        if (is_device_ptr(scene_box)) cudaMemcpy(scene_box, box, sizeof box, cudaMemcpyHostToDevice);
        else memcpy(scene_box, box, sizeof box);
    }
    dfree(c, zero);
    dfree(c, keys);
    dfree(c, owned);
    return st;
}

sq_status sq_radix_sort_pairs(sq_ctx* c, const uint32_t* keys_in, const uint32_t* values_in, uint32_t n,
                              uint32_t key_bits, uint32_t digit_bits, uint32_t* keys_out, uint32_t* values_out)
{
    if (!c || (n > 0 && (!keys_in || !values_in || !keys_out || !values_out)))
        return fail(c, SQ_ERR_INVALID, "sq_radix_sort_pairs: null argument");
    if (key_bits < 1 || key_bits > 32) return fail(c, SQ_ERR_INVALID, "key_bits must be 1..32");
    if (digit_bits == 0) digit_bits = 8;
    if (digit_bits != 6 && digit_bits != 8 && digit_bits != 10) return fail(c, SQ_ERR_INVALID, "digit_bits must be 6, 8 or 10");
    if (n >= (1u << 30)) return fail(c, SQ_ERR_INVALID, "n too large");
    Guard g(c->device);
    if (n == 0) return SQ_OK;
    const uint32_t passes = sort_passes_for(key_bits, digit_bits);
    const size_t radix = (size_t)1 << digit_bits;
    const size_t lb_words = sqk::sort_lookback_words(n, digit_bits, passes);
    const size_t z_hist = 0, z_ctr = passes * radix, z_lb = z_ctr + 8;
    const size_t z_words = z_lb + lb_words;
    // an armed look-back stall applies to a one-pass sort of two tiles or
    // more, where every scatter stays inside the output (see SortStall)
    sqk::SortStall stall{c->stall_lookback ? c->stall_lookback - 1u : 0u};
    const bool stalled = c->stall_lookback != 0;
    c->stall_lookback = 0;
    if (stalled && (passes != 1 || n <= sqk::sort_tile_keys(n, digit_bits)))
        return fail(c, SQ_ERR_INVALID, "look-back stall injection needs a one-pass sort of two tiles or more");
    uint32_t* zero = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * z_words));
    uint32_t* buf = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * 4ull * n));
    if (!zero || !buf) { dfree(c, zero); dfree(c, buf); return fail(c, SQ_ERR_OOM, "allocation failed"); }
    cudaStream_t s = c->stream;
    uint32_t *ka = buf, *va = buf + n, *kb = buf + 2ull * n, *vb = buf + 3ull * n;
    SQ_CUDA(c, cudaMemcpyAsync(ka, keys_in, sizeof(uint32_t) * (size_t)n, cudaMemcpyDefault, s));
    SQ_CUDA(c, cudaMemcpyAsync(va, values_in, sizeof(uint32_t) * (size_t)n, cudaMemcpyDefault, s));
    SQ_CUDA(c, cudaMemsetAsync(zero, 0, sizeof(uint32_t) * z_words, s));
    SQ_CUDA(c, cudaEventRecord(c->ev[1], s));
    sqk::sort_histogram(ka, n, zero + z_hist, digit_bits, passes, s);
    const int which = sqk::sort_passes(ka, va, kb, vb, n, zero + z_hist, zero + z_lb, zero + z_ctr, digit_bits, passes,
                                       c->ctrl, s, stalled ? &stall : nullptr);
    SQ_CUDA(c, cudaEventRecord(c->ev[2], s));
    const uint32_t* rk = which ? kb : ka;
    const uint32_t* rv = which ? vb : va;
    SQ_CUDA(c, cudaMemcpyAsync(keys_out, rk, sizeof(uint32_t) * (size_t)n, cudaMemcpyDefault, s));
    SQ_CUDA(c, cudaMemcpyAsync(values_out, rv, sizeof(uint32_t) * (size_t)n, cudaMemcpyDefault, s));
    SQ_CUDA(c, cudaGetLastError());
    const bool host_out = !is_device_ptr(keys_out) || !is_device_ptr(values_out);
    sq_status st = SQ_OK;
    if (host_out) st = check_device_error(c, nullptr);
    dfree(c, zero);
    dfree(c, buf);
    return st;
}

// Camera images of at least this many rays with page-locked host outputs
// are traced in bands (see sq_trace).
constexpr uint64_t kBandMinRays = 1u << 21;

// An 8-wide camera trace in up to sq_ctx::kMaxBands row bands of 8x4 tiles:
// band k traces on band_stream[k % 2] into the device buffers (hits_dev,
// heat_dev, or the caller's device outputs), and copy_stream copies its rows
// to the host outputs as soon as it is done.  The bands shrink towards the
// end (tile-row shares 8:7:6:5:4:3:2:1 of 36), so the copy left when the
// last band finishes is small and each earlier copy has the later bands'
// trace time to hide in.  The context stream waits for everything at the
// end.  Returns false on a CUDA error.
bool trace8_bands(sq_ctx* c, sqk::Trace8Args w, sq_hit* hits, uint8_t* heat, const sq_hit* hits_dev,
                  const uint8_t* heat_dev)
{
    cudaStream_t s = c->stream;
    const uint32_t tiles_x = (w.width + 7u) / 8u, tiles_y = (w.height + 3u) / 4u;
    const uint32_t nb = std::min<uint32_t>(sq_ctx::kMaxBands, tiles_y);
    uint32_t* counters = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * sq_ctx::kMaxBands));
    if (!counters) return false;
    bool ok = cudaMemsetAsync(counters, 0, sizeof(uint32_t) * sq_ctx::kMaxBands, s) == cudaSuccess &&
              cudaEventRecord(c->band_fork, s) == cudaSuccess &&
              cudaStreamWaitEvent(c->band_stream[0], c->band_fork, 0) == cudaSuccess &&
              cudaStreamWaitEvent(c->band_stream[1], c->band_fork, 0) == cudaSuccess &&
              cudaStreamWaitEvent(c->copy_stream, c->band_fork, 0) == cudaSuccess;
    // cumulative shares of band k's end: sum of (nb - j) for j <= k, over nb (nb + 1) / 2
    const uint64_t total = (uint64_t)nb * (nb + 1) / 2;
    uint64_t cum = 0;
    for (uint32_t k = 0; ok && k < nb; ++k) {
        const uint32_t ty0 = (uint32_t)((uint64_t)tiles_y * cum / total);
        cum += nb - k;
        const uint32_t ty1 = (uint32_t)((uint64_t)tiles_y * cum / total);
        if (ty1 == ty0) continue;
        cudaStream_t bs = c->band_stream[k & 1u];
        w.tile0 = ty0 * tiles_x;
        w.tile_end = ty1 * tiles_x;
        w.work = counters + k;
        sqk::trace8(w, bs);
        ok = cudaGetLastError() == cudaSuccess && cudaEventRecord(c->band_done[k], bs) == cudaSuccess &&
             cudaStreamWaitEvent(c->copy_stream, c->band_done[k], 0) == cudaSuccess;
        // rows [4 ty0, 4 ty1) of the image are one contiguous range of rays
        const size_t r0 = (size_t)std::min(4u * ty0, w.height) * w.width;
        const size_t r1 = (size_t)std::min(4u * ty1, w.height) * w.width;
        if (ok && hits_dev && hits)
            ok = cudaMemcpyAsync(hits + r0, hits_dev + r0, sizeof(sq_hit) * (r1 - r0), cudaMemcpyDeviceToHost,
                                 c->copy_stream) == cudaSuccess;
        if (ok && heat_dev && heat)
            ok = cudaMemcpyAsync(heat + 3 * r0, heat_dev + 3 * r0, 3 * (r1 - r0), cudaMemcpyDeviceToHost,
                                 c->copy_stream) == cudaSuccess;
    }
    // join all three streams back into the context stream, even after an
    // error, so nothing is left running against freed buffers
    cudaStream_t side[3] = {c->band_stream[0], c->band_stream[1], c->copy_stream};
    for (int q = 0; q < 3; ++q) {
        const bool j = cudaEventRecord(c->band_join[q], side[q]) == cudaSuccess &&
                       cudaStreamWaitEvent(s, c->band_join[q], 0) == cudaSuccess;
        ok = ok && j;
    }
    dfree(c, counters);  // reused only by later work on the context stream, which waits for the bands
    return ok;
}

sq_status sq_trace(sq_ctx* c, const sq_bvh* b, const sq_ray_source* rays, uint32_t mode, sq_hit* hits,
                   uint8_t* heatmap_rgb)
{
    if (!c || !b || !rays) return fail(c, SQ_ERR_INVALID, "sq_trace: null argument");
    const bool force_binary = (mode & SQ_TRACE_FORCE_BINARY) != 0;
    const bool sched_refill = (mode & SQ_TRACE_SCHED_REFILL) != 0;
    const bool sched_tiles = (mode & SQ_TRACE_SCHED_TILES) != 0;
    const bool heat_ramp = (mode & SQ_TRACE_HEAT_RAMP) != 0;
    const uint32_t width_k = (mode >> 16) & 0xFFu;
    if (sched_refill && sched_tiles) return fail(c, SQ_ERR_INVALID, "sq_trace: choose one ray schedule");
    mode &= 0xFFu;
    if (mode > SQ_TRACE_BUNDLE) return fail(c, SQ_ERR_INVALID, "sq_trace: unknown mode %u", mode);
    const bool coherent = mode == SQ_TRACE_PACKET || mode == SQ_TRACE_BUNDLE;
    if (coherent) {
        // trace_packet<k> / trace_bundle<k>: the reference camera, heatmap only
        if (rays->kind != SQ_RAYS_REFERENCE_CAMERA)
            return fail(c, SQ_ERR_INVALID, "sq_trace: packet and bundle modes trace the reference camera");
        if (hits) return fail(c, SQ_ERR_UNSUPPORTED, "sq_trace: packet and bundle modes produce the heatmap only");
        if (!heatmap_rgb) return fail(c, SQ_ERR_INVALID, "sq_trace: packet and bundle modes need a heatmap");
        if (!sqk::coherent_shape_ok(mode == SQ_TRACE_BUNDLE, width_k, rays->width, rays->height))
            return fail(c, SQ_ERR_INVALID,
                        "sq_trace: %s width %u needs an image made of whole packet blocks (got %ux%u)",
                        mode == SQ_TRACE_BUNDLE ? "bundle" : "packet", width_k, rays->width, rays->height);
    } else if (width_k) {
        return fail(c, SQ_ERR_INVALID, "sq_trace: a width applies to packet and bundle modes only");
    }
    Guard g(c->device);
    sqk::TraceArgs a;
    memset(&a, 0, sizeof a);
    a.nodes = b->nodes;
    a.node_count = b->cap;
    a.tri_count = b->n;
    a.root = b->root;
    a.tris = b->tris;
    a.mode = mode;
    a.ray_kind = rays->kind;
    a.refill = sched_refill ? 1u : 0u;  // the binary tree: 32-ray batches per warp unless asked
    a.heat_ramp = heat_ramp ? 1u : 0u;
    a.root_group = 1u;
    uint64_t count = 0;
    float* rays_own = nullptr;
    if (rays->kind == SQ_RAYS_REFERENCE_CAMERA || rays->kind == SQ_RAYS_PINHOLE) {
        if (rays->width == 0 || rays->height == 0) return fail(c, SQ_ERR_INVALID, "sq_trace: empty image");
        a.width = rays->width;
        a.height = rays->height;
        count = (uint64_t)rays->width * rays->height;
        camera_params(*rays, a.cam);
    } else if (rays->kind == SQ_RAYS_EXPLICIT) {
        count = rays->ray_count;
        a.ray_count = rays->ray_count;
        if (count && !rays->rays) return fail(c, SQ_ERR_INVALID, "sq_trace: null ray array");
        if (count && is_device_ptr(rays->rays) && (reinterpret_cast<uintptr_t>(rays->rays) & 15u) == 0) {
            a.rays = reinterpret_cast<const float*>(rays->rays);
        } else if (count) {
            rays_own = static_cast<float*>(dalloc(c, sizeof(sq_ray) * count));
            if (!rays_own) return fail(c, SQ_ERR_OOM, "ray allocation failed");
            SQ_CUDA(c, cudaMemcpyAsync(rays_own, rays->rays, sizeof(sq_ray) * count, cudaMemcpyDefault, c->stream));
            a.rays = rays_own;
        }
    } else {
        return fail(c, SQ_ERR_INVALID, "sq_trace: unknown ray kind %u", rays->kind);
    }
    if (count > 0xFFFFFFFFull / 3) return fail(c, SQ_ERR_INVALID, "sq_trace: too many rays");
    const bool hits_dev = hits && is_device_ptr(hits);
    const bool heat_dev = heatmap_rgb && is_device_ptr(heatmap_rgb);
    // page-locked host outputs are written by the kernel in place
    sq_hit* hits_map = (hits && !hits_dev) ? static_cast<sq_hit*>(pinned_device_alias(hits)) : nullptr;
    uint8_t* heat_map = (heatmap_rgb && !heat_dev) ? static_cast<uint8_t*>(pinned_device_alias(heatmap_rgb)) : nullptr;
    // ... except for a large camera image on the 8-wide tree: the image is
    // traced in row bands into device memory, and the copy engine moves each
    // finished band to the host while the next bands trace.  A kernel's
    // stores into host memory slow it down more than that copy costs.
    const bool wide_path = !coherent && b->nodes8 && mode != SQ_TRACE_REF && !force_binary;
    const bool pinned_out = (hits_map || heat_map) && (!hits || hits_dev || hits_map) &&
                            (!heatmap_rgb || heat_dev || heat_map);
    const bool banded = wide_path && rays->kind != SQ_RAYS_EXPLICIT && !sched_refill && pinned_out &&
                        count >= kBandMinRays && band_resources(c);
    if (banded) hits_map = nullptr, heat_map = nullptr;
    sq_hit* hits_tmp = nullptr;
    uint8_t* heat_tmp = nullptr;
    if (hits && !hits_dev && !hits_map) {
        hits_tmp = static_cast<sq_hit*>(dalloc(c, sizeof(sq_hit) * count));
        if (!hits_tmp) { dfree(c, rays_own); return fail(c, SQ_ERR_OOM, "hit buffer allocation failed"); }
    }
    if (heatmap_rgb && !heat_dev && !heat_map) {
        heat_tmp = static_cast<uint8_t*>(dalloc(c, 3ull * count));
        if (!heat_tmp) { dfree(c, rays_own); dfree(c, hits_tmp); return fail(c, SQ_ERR_OOM, "heatmap allocation failed"); }
    }
    a.hits = hits_dev ? hits : (hits_map ? hits_map : hits_tmp);
    a.heat = heat_dev ? heatmap_rgb : (heat_map ? heat_map : heat_tmp);
    a.work = c->ctrl + 1;
    a.err = c->ctrl;
    a.stats = reinterpret_cast<unsigned long long*>(c->ctrl + 4);
    cudaStream_t s = c->stream;
    SQ_CUDA(c, cudaMemsetAsync(c->ctrl + 1, 0, 11 * sizeof(uint32_t), s));
    SQ_CUDA(c, cudaEventRecord(c->ev[4], s));
    if (count > 0) {
        if (coherent) {
            sqk::trace_coherent(a, mode == SQ_TRACE_BUNDLE, width_k, s);
        } else if (b->nodes8 && mode != SQ_TRACE_REF && !force_binary) {
            sqk::Trace8Args w;
            memset(&w, 0, sizeof w);
            w.nodes = b->nodes8;
            w.tris8 = static_cast<const float4*>(b->tris8);
            w.mode = mode;
            w.ray_kind = a.ray_kind;
            w.width = a.width;
            w.height = a.height;
            memcpy(w.cam, a.cam, sizeof w.cam);
            w.rays = a.rays;
            w.ray_count = a.ray_count;
            w.hits = a.hits;
            w.heat = a.heat;
            w.work = a.work;
            w.err = a.err;
            w.stats = a.stats;
            w.heat_ramp = a.heat_ramp;
            // default: explicit rays refill lanes; camera rays keep coherent
            // 8x4 tiles per warp
            w.refill = sched_refill ? 1u : (sched_tiles ? 0u : (a.ray_kind == SQ_RAYS_EXPLICIT ? 1u : 0u));
            if (banded) {
                if (!trace8_bands(c, w, hits, heatmap_rgb, hits_tmp, heat_tmp)) {
                    dfree(c, rays_own); dfree(c, hits_tmp); dfree(c, heat_tmp);
                    return fail(c, SQ_ERR_CUDA, "sq_trace: banded trace: %s", cudaGetErrorString(cudaGetLastError()));
                }
            } else {
                sqk::trace8(w, s);
            }
        } else {
            sqk::trace(a, s);
        }
    }
    SQ_CUDA(c, cudaEventRecord(c->ev[5], s));
    SQ_CUDA(c, cudaGetLastError());
    c->trace_timed = true;
    if (hits_tmp && !banded) SQ_CUDA(c, cudaMemcpyAsync(hits, hits_tmp, sizeof(sq_hit) * count, cudaMemcpyDeviceToHost, s));
    if (heat_tmp && !banded) SQ_CUDA(c, cudaMemcpyAsync(heatmap_rgb, heat_tmp, 3ull * count, cudaMemcpyDeviceToHost, s));
    sq_status st = SQ_OK;
    if (hits_tmp || heat_tmp || hits_map || heat_map) st = check_device_error(c, nullptr);
    dfree(c, rays_own);
    dfree(c, hits_tmp);
    dfree(c, heat_tmp);
    return st;
}

sq_status sq_traverse(sq_ctx* c, const sq_bvh* b, uint32_t index, uint32_t count, const sq_ray* rays, uint32_t n,
                      sq_hit* hits)
{
    if (!c || !b || (n && (!rays || !hits))) return fail(c, SQ_ERR_INVALID, "sq_traverse: null argument");
    if (count == 0 || (uint64_t)index + count > b->cap)
        return fail(c, SQ_ERR_INVALID, "sq_traverse: node group [%u, %u + %u) outside the %u nodes", index, index,
                    count, b->cap);
    if (n == 0) return SQ_OK;
    Guard g(c->device);
    sqk::TraceArgs a;
    memset(&a, 0, sizeof a);
    a.nodes = b->nodes;
    a.node_count = b->cap;
    a.tri_count = b->n;
    a.root = index;
    a.root_group = count;
    a.tris = b->tris;
    a.mode = SQ_TRACE_REF;
    a.ray_kind = SQ_RAYS_EXPLICIT;
    a.ray_count = n;
    float* rays_own = nullptr;
    if (is_device_ptr(rays) && (reinterpret_cast<uintptr_t>(rays) & 15u) == 0) {
        a.rays = reinterpret_cast<const float*>(rays);
    } else {
        rays_own = static_cast<float*>(dalloc(c, sizeof(sq_ray) * (size_t)n));
        if (!rays_own) return fail(c, SQ_ERR_OOM, "sq_traverse: ray allocation failed");
        a.rays = rays_own;
    }
    const bool hits_dev = is_device_ptr(hits);
    sq_hit* hits_map = hits_dev ? nullptr : static_cast<sq_hit*>(pinned_device_alias(hits));
    sq_hit* hits_tmp = nullptr;
    if (!hits_dev && !hits_map) {
        hits_tmp = static_cast<sq_hit*>(dalloc(c, sizeof(sq_hit) * (size_t)n));
        if (!hits_tmp) {
            dfree(c, rays_own);
            return fail(c, SQ_ERR_OOM, "sq_traverse: hit buffer allocation failed");
        }
    }
    a.hits = hits_dev ? hits : (hits_map ? hits_map : hits_tmp);
    a.work = c->ctrl + 1;
    a.err = c->ctrl;
    a.stats = reinterpret_cast<unsigned long long*>(c->ctrl + 4);
    cudaStream_t s = c->stream;
    cudaError_t e = cudaSuccess;
    if (rays_own) e = cudaMemcpyAsync(rays_own, rays, sizeof(sq_ray) * (size_t)n, cudaMemcpyDefault, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->ctrl + 1, 0, 11 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev[4], s);
    if (e == cudaSuccess) {
        sqk::trace(a, s);
        e = cudaEventRecord(c->ev[5], s);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess && hits_tmp)
        e = cudaMemcpyAsync(hits, hits_tmp, sizeof(sq_hit) * (size_t)n, cudaMemcpyDeviceToHost, s);
    sq_status st = e == cudaSuccess ? SQ_OK : fail(c, SQ_ERR_CUDA, "sq_traverse: %s", cudaGetErrorString(e));
    if (st == SQ_OK) {
        c->trace_timed = true;
        if (!hits_dev) st = check_device_error(c, nullptr);
    }
    dfree(c, rays_own);
    dfree(c, hits_tmp);
    return st;
}

sq_status sq_trace_batches(sq_ctx* c, const sq_bvh* b, const sq_ray_source* batches, uint32_t count, uint32_t mode,
                           sq_hit* hits, uint8_t* heatmap_rgb)
{
    if (!c || !b || (count && !batches)) return fail(c, SQ_ERR_INVALID, "sq_trace_batches: null argument");
    const bool force_binary = (mode & SQ_TRACE_FORCE_BINARY) != 0;
    const bool sched_refill = (mode & SQ_TRACE_SCHED_REFILL) != 0;
    const bool sched_tiles = (mode & SQ_TRACE_SCHED_TILES) != 0;
    if (sched_refill && sched_tiles) return fail(c, SQ_ERR_INVALID, "sq_trace_batches: choose one ray schedule");
    if (mode >> 16) return fail(c, SQ_ERR_INVALID, "sq_trace_batches: packet and bundle modes are single-image");
    const uint32_t heat_ramp = (mode & SQ_TRACE_HEAT_RAMP) ? 1u : 0u;
    mode &= 0xFFu;
    if (mode > SQ_TRACE_ANYHIT) return fail(c, SQ_ERR_INVALID, "sq_trace_batches: unknown mode %u", mode);
    const bool wide = b->nodes8 && mode != SQ_TRACE_REF && !force_binary;
    Guard g(c->device);
    // the job table: one job per batch, outputs batch after batch
    std::vector<sqk::BatchJob> jobs(count);
    uint64_t rays = 0, batches32 = 0, xrays = 0, staged = 0;
    for (uint32_t k = 0; k < count; ++k) {
        const sq_ray_source& rs = batches[k];
        sqk::BatchJob& j = jobs[k];
        memset(&j, 0, sizeof j);
        j.ray_kind = rs.kind;
        j.root = wide ? 0u : b->root;
        j.out_offset = (uint32_t)rays;
        j.batch_begin = (uint32_t)batches32;
        uint64_t cnt;
        if (rs.kind == SQ_RAYS_EXPLICIT) {
            cnt = rs.ray_count;
            if (cnt && !rs.rays) return fail(c, SQ_ERR_INVALID, "sq_trace_batches: batch %u has no ray array", k);
            if (cnt && !(is_device_ptr(rs.rays) && (reinterpret_cast<uintptr_t>(rs.rays) & 15u) == 0)) {
                j.ray_offset = (uint32_t)staged;  // copied to the staging array below
                staged += cnt;
            } else {
                j.rays = reinterpret_cast<const float*>(rs.rays);
            }
            xrays += cnt;
            batches32 += (cnt + 31) / 32;
        } else if (rs.kind == SQ_RAYS_PINHOLE || rs.kind == SQ_RAYS_REFERENCE_CAMERA) {
            if (rs.width == 0 || rs.height == 0) return fail(c, SQ_ERR_INVALID, "sq_trace_batches: batch %u: empty image", k);
            j.width = rs.width;
            j.height = rs.height;
            cnt = (uint64_t)rs.width * rs.height;
            batches32 += (uint64_t)((rs.width + 7) / 8) * ((rs.height + 3) / 4);
            camera_params(rs, j.cam);
        } else {
            return fail(c, SQ_ERR_INVALID, "sq_trace_batches: batch %u: unknown ray kind %u", k, rs.kind);
        }
        j.ray_count = (uint32_t)cnt;
        rays += cnt;
        if (rays > 0xFFFFFFFFull / 3 || batches32 > 0xFFFFFFFFull)
            return fail(c, SQ_ERR_INVALID, "sq_trace_batches: too many rays");
    }
    sqk::BatchJob* d_jobs = count ? static_cast<sqk::BatchJob*>(dalloc(c, sizeof(sqk::BatchJob) * count)) : nullptr;
    float* d_staged = staged ? static_cast<float*>(dalloc(c, sizeof(sq_ray) * staged)) : nullptr;
    const bool hits_dev = hits && is_device_ptr(hits);
    const bool heat_dev = heatmap_rgb && is_device_ptr(heatmap_rgb);
    sq_hit* hits_map = (hits && !hits_dev) ? static_cast<sq_hit*>(pinned_device_alias(hits)) : nullptr;
    uint8_t* heat_map = (heatmap_rgb && !heat_dev) ? static_cast<uint8_t*>(pinned_device_alias(heatmap_rgb)) : nullptr;
    sq_hit* hits_tmp = (hits && !hits_dev && !hits_map && rays) ? static_cast<sq_hit*>(dalloc(c, sizeof(sq_hit) * rays))
                                                                 : nullptr;
    uint8_t* heat_tmp = (heatmap_rgb && !heat_dev && !heat_map && rays) ? static_cast<uint8_t*>(dalloc(c, 3ull * rays))
                                                                        : nullptr;
    auto release = [&]() {
        dfree(c, d_jobs);
        dfree(c, d_staged);
        dfree(c, hits_tmp);
        dfree(c, heat_tmp);
    };
    if ((count && !d_jobs) || (staged && !d_staged) || (hits && !hits_dev && !hits_map && rays && !hits_tmp) ||
        (heatmap_rgb && !heat_dev && !heat_map && rays && !heat_tmp)) {
        release();
        return fail(c, SQ_ERR_OOM, "sq_trace_batches: allocation failed");
    }
    cudaStream_t s = c->stream;
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        release();
        return fail(c, e == cudaErrorMemoryAllocation ? SQ_ERR_OOM : SQ_ERR_CUDA, "sq_trace_batches: %s: %s", what,
                    cudaGetErrorString(e));
    };
    cudaError_t e;
    for (uint32_t k = 0; k < count; ++k)
        if (batches[k].kind == SQ_RAYS_EXPLICIT && batches[k].ray_count && !jobs[k].rays &&
            (e = cudaMemcpyAsync(d_staged + 8ull * jobs[k].ray_offset, batches[k].rays,
                                 sizeof(sq_ray) * batches[k].ray_count, cudaMemcpyDefault, s)) != cudaSuccess)
            return cuda_fail(e, "ray copy");
    for (auto& j : jobs)
        if (j.ray_kind == SQ_RAYS_EXPLICIT && !j.rays) j.rays = d_staged;
    if (count && (e = cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(sqk::BatchJob) * count, cudaMemcpyHostToDevice, s)) !=
                     cudaSuccess)
        return cuda_fail(e, "job table copy");
    sqk::BatchTraceArgs a;
    memset(&a, 0, sizeof a);
    a.nodes = b->nodes;
    a.node_count = b->cap;
    a.tri_count = b->n;
    a.nodes8 = b->nodes8;
    a.tris8 = static_cast<const float4*>(b->tris8);
    a.tris = b->tris;
    a.rays = d_staged;
    a.jobs = d_jobs;
    a.njobs = count;
    a.total_batches = (uint32_t)batches32;
    a.mode = mode;
    a.hits = hits_dev ? hits : (hits_map ? hits_map : hits_tmp);
    a.heat = heat_dev ? heatmap_rgb : (heat_map ? heat_map : heat_tmp);
    a.work = c->ctrl + 1;
    a.err = c->ctrl;
    a.stats = reinterpret_cast<unsigned long long*>(c->ctrl + 4);
    // per-lane refill by default when most rays are explicit (incoherent)
    a.refill = sched_refill ? 1u : (sched_tiles ? 0u : (2ull * xrays > rays ? 1u : 0u));
    a.heat_ramp = heat_ramp;
    if ((e = cudaMemsetAsync(c->ctrl + 1, 0, 11 * sizeof(uint32_t), s)) != cudaSuccess) return cuda_fail(e, "reset");
    if ((e = cudaEventRecord(c->ev[4], s)) != cudaSuccess) return cuda_fail(e, "event");
    if (rays) {
        if (wide) sqk::trace8_batch(a, 128, s);
        else sqk::trace_batch(a, 128, s);
    }
    if ((e = cudaEventRecord(c->ev[5], s)) != cudaSuccess) return cuda_fail(e, "event");
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "launch");
    c->trace_timed = true;
    if (hits_tmp && (e = cudaMemcpyAsync(hits, hits_tmp, sizeof(sq_hit) * rays, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_fail(e, "hit copy");
    if (heat_tmp && (e = cudaMemcpyAsync(heatmap_rgb, heat_tmp, 3ull * rays, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_fail(e, "heatmap copy");
    sq_status st = SQ_OK;
    if (hits_tmp || heat_tmp || hits_map || heat_map) st = check_device_error(c, nullptr);
    release();
    return st;
}

sq_status sq_debug_inject(sq_ctx* c, uint32_t what, uint32_t limit)
{
    if (!c) return SQ_ERR_INVALID;
    switch (what) {
    case SQ_DEBUG_OFF:
        c->stall_lookback = c->stall_barrier = 0;
        c->fail_alloc_in = -1;
        return SQ_OK;
    case SQ_DEBUG_STALL_LOOKBACK:
    case SQ_DEBUG_STALL_BARRIER:
        if (limit == 0 || limit > (1u << 20))
            return fail(c, SQ_ERR_INVALID, "sq_debug_inject: a poll limit of 1..2^20 is needed");
        (what == SQ_DEBUG_STALL_LOOKBACK ? c->stall_lookback : c->stall_barrier) = limit + 1u;
        return SQ_OK;
    case SQ_DEBUG_FAIL_ALLOC:
        c->fail_alloc_in = limit;
        return SQ_OK;
    default:
        return fail(c, SQ_ERR_INVALID, "sq_debug_inject: unknown injection %u", what);
    }
}

sq_status sq_debug_memory(const sq_ctx* c, uint64_t out[4])
{
    if (!c || !out) return SQ_ERR_INVALID;
    out[0] = c->live_blocks.size();
    out[1] = 0;
    for (const auto& kv : c->live_blocks) out[1] += kv.second;
    out[2] = c->free_blocks.size();
    out[3] = 0;
    for (const auto& kv : c->free_blocks) out[3] += kv.first;
    return SQ_OK;
}

sq_status sq_last_trace_stats(sq_ctx* c, uint64_t stats[4])
{
    if (!c || !stats) return SQ_ERR_INVALID;
    Guard g(c->device);
    SQ_CUDA(c, cudaStreamSynchronize(c->stream));
    unsigned long long st[4] = {0, 0, 0, 0};
    SQ_CUDA(c, cudaMemcpy(st, c->ctrl + 4, sizeof st, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 4; ++k) stats[k] = st[k];
    return SQ_OK;
}

sq_status sq_last_timings(sq_ctx* c, float stage_ms[8])
{
    if (!c || !stage_ms) return SQ_ERR_INVALID;
    Guard g(c->device);
    for (int k = 0; k < 8; ++k) stage_ms[k] = -1.0f;
    SQ_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->build_timed) {
        cudaEventElapsedTime(&stage_ms[0], c->ev[0], c->ev[6]);
        cudaEventElapsedTime(&stage_ms[7], c->ev[3], c->ev[6]);
        cudaEventElapsedTime(&stage_ms[1], c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&stage_ms[2], c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&stage_ms[3], c->ev[2], c->ev[3]);
    }
    if (c->trace_timed) {
        cudaEventElapsedTime(&stage_ms[4], c->ev[4], c->ev[5]);
        unsigned long long st[2] = {0, 0};
        SQ_CUDA(c, cudaMemcpy(st, c->ctrl + 4, sizeof st, cudaMemcpyDeviceToHost));
        stage_ms[5] = (float)st[0];
        stage_ms[6] = (float)st[1];
    }
    cudaGetLastError();
    return SQ_OK;
}

}  // extern "C"
