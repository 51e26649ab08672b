// sq_batch.cu -- many meshes and ray tiles, built and traced by one launch
// sequence that is captured once in a CUDA graph and replayed.
//
// Build (all meshes together, no host synchronisation), Morton builder:
//   k_seg_bounds     every mesh's box (warp-aggregated atomics per mesh)
//   k_seg_morton     30-bit Morton codes in each mesh's own box (as if the
//                    reference's setup_morton, src/builder.cpp:2204-2237, ran
//                    per mesh) + the code digit histograms
//   onesweep         stable sort by code, then stable sort by mesh id: the
//                    result is (mesh, code) order, each mesh contiguous
//   climb            the LBVH climb of sq_lbvh.cu (k_lbvh_climb and
//                    k_lbvh_global over mesh segments): nothing merges across
//                    a mesh boundary; mesh m's root record is slot 3N + 2 + m
//   8-wide collapse  (optional) seeded with all mesh roots, a fixed number
//                    of level kernels with device-side task counts: 8-wide
//                    node m is mesh m's root
// SAH builder: sqk::build_sah_batch (sq_sah.cu) -- per-mesh root boxes and
// root tasks, then the binned SAH's level kernels over all meshes' tasks at
// once, a fixed number of levels with device-side task counts, the small
// phase and the leaves; the same records a single build of each mesh writes.
// Trace: one persistent kernel over a job table (mesh, camera or rays,
// output offset); warps take 32-ray batches of any job.
//
// Autotuner: sq_batch_autotune times every combination of sort digit width
// (6/8/10; Morton) or SAH bin count (8/16/32; SAH), BVH width (2 or 8-wide
// quantised) and trace block shape (64/128/256 threads) on the caller's
// batch and keeps the fastest; results are cached in a JSON-lines file keyed
// by the batch's size class and builder.
#include "sq_internal.cuh"
#include "sq_lbvh_dev.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace sqi;

struct sq_batch {
    sq_ctx* ctx = nullptr;
    uint32_t meshes = 0, tris = 0, rays = 0, explicit_rays = 0;
    sq_batch_params params{};
    // device data
    float* d_tris = nullptr;          // concatenated triangles
    uint32_t* d_off = nullptr;        // mesh m: triangles [off[m], off[m + 1])
    float* d_rays = nullptr;          // concatenated explicit rays
    sqk::BatchJob* d_jobs = nullptr;
    uint32_t* d_roots = nullptr;      // binary root record of each mesh
    Node* d_nodes = nullptr;          // 3N + 2 + M records
    void* d_nodes8 = nullptr;
    void* d_tris8 = nullptr;
    uint32_t* d_ws8 = nullptr;
    uint32_t* d_zero = nullptr;       // zeroed each run: boxes, histograms, counters, look-back, flags
    size_t zero_words = 0;
    uint32_t* d_keys = nullptr;       // 4 x N sort buffers + codes by triangle + sorted codes
    float4* d_info = nullptr;         // 4N climb sibling records
    void* d_sah_ws = nullptr;         // SAH batches: the builder's workspace
    sq_hit* d_hits = nullptr;
    uint8_t* d_heat = nullptr;
    std::vector<sqk::BatchJob> jobs;  // host copy (roots patched per width)
    uint32_t total_batches = 0;
    cudaGraphExec_t graph = nullptr;
    bool captured = false;
};

namespace {

using namespace sq;

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

// box_ord[8m + k] = ordered(-min_k), [8m + 3 + k] = ordered(max_k)
__global__ void __launch_bounds__(256) k_seg_bounds(const float* __restrict__ tris, uint32_t n,
                                                    const uint32_t* __restrict__ off, uint32_t M,
                                                    uint32_t* __restrict__ box_ord)
{
    chain_wait();  // a chained launch (the batch build's kernels follow one another)
    chain_release();
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t m = 0xFFFFFFFFu;
        uint32_t e[6] = {0, 0, 0, 0, 0, 0};
        if (valid) {
            m = mesh_of(off, M, i);
            float t[9];
            load_tri(tris, i, t);
            const Box b = tri_box(t);
            for (int k = 0; k < 3; ++k) { e[k] = float_to_ordered(-b.mn[k]); e[3 + k] = float_to_ordered(b.mx[k]); }
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, m);
#pragma unroll
        for (int k = 0; k < 6; ++k) e[k] = __reduce_max_sync(peers, e[k]);
        if (valid && (threadIdx.x & 31) == (uint32_t)(__ffs(peers) - 1))
            for (int k = 0; k < 6; ++k) atomicMax(box_ord + 8ull * m + k, e[k]);
    }
}

__global__ void __launch_bounds__(256) k_seg_morton(const float* __restrict__ tris, uint32_t n,
                                                    const uint32_t* __restrict__ off, uint32_t M,
                                                    const uint32_t* __restrict__ box_ord, uint32_t* __restrict__ keys,
                                                    uint32_t* __restrict__ vals, uint32_t* __restrict__ code_by_tri,
                                                    uint32_t* __restrict__ hist, uint32_t db, uint32_t passes)
{
    chain_wait();  // a chained launch (the batch build's kernels follow one another)
    chain_release();
    extern __shared__ uint32_t s_hist[];
    const uint32_t radix = 1u << db;
    for (uint32_t j = threadIdx.x; j < passes * radix; j += blockDim.x) s_hist[j] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t m = mesh_of(off, M, i);
        const uint32_t* bo = box_ord + 8ull * m;
        float t[9];
        load_tri(tris, i, t);
        const Box b = tri_box(t);
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            const float smin = -ordered_to_float(bo[k]);
            const float smax = ordered_to_float(bo[3 + k]);
            const float ext = smax - smin;
            const float c = (b.mn[k] + b.mx[k]) * 0.5f;
            const float u = (c - smin) / ext;
            q[k] = f2u(u * 1023.0f);
        }
        const uint32_t code = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
        keys[i] = code;
        vals[i] = i;
        code_by_tri[i] = code;
        for (uint32_t p = 0; p < passes; ++p) atomicAdd(&s_hist[p * radix + ((code >> (p * db)) & (radix - 1))], 1u);
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < passes * radix; j += blockDim.x) {
        const uint32_t c = s_hist[j];
        if (c) atomicAdd(hist + j, c);
    }
}

// mesh id of each sorted element, as the key of the second sort
__global__ void k_mesh_keys(const uint32_t* __restrict__ vals, uint32_t n, const uint32_t* __restrict__ off, uint32_t M,
                            uint32_t* __restrict__ mkeys)
{
    chain_wait();  // a chained launch (the batch build's kernels follow one another)
    chain_release();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mkeys[i] = mesh_of(off, M, vals[i]);
}

__global__ void k_gather_codes(const uint32_t* __restrict__ perm, uint32_t n, const uint32_t* __restrict__ code_by_tri,
                               uint32_t* __restrict__ codes)
{
    chain_wait();  // a chained launch (the batch build's kernels follow one another)
    chain_release();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        codes[i] = code_by_tri[perm[i]];
}

// root records of meshes without triangles
__global__ void k_empty_roots(const uint32_t* __restrict__ off, uint32_t M, Node* __restrict__ nodes, uint32_t root0,
                              uint32_t leaf0)
{
    chain_wait();  // a chained launch (the batch build's kernels follow one another)
    chain_release();
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        if (off[m + 1] != off[m]) continue;
        Box b;
        box_reset(b);
        store_node(nodes + root0 + m, b, leaf0 + off[m], 0u, 0);
    }
}

int sms() { return sm_count(); }

uint32_t mesh_passes(uint32_t M) { return M <= 256 ? 1u : (M <= 65536 ? 2u : 3u); }

// Enqueue one whole run (build + trace) on the context stream.
sq_status enqueue_run(sq_batch* b)
{
    sq_ctx* c = b->ctx;
    cudaStream_t s = c->stream;
    const uint32_t N = b->tris, M = b->meshes;
    const uint32_t db = b->params.sort_digit_bits ? b->params.sort_digit_bits : 8u;
    const uint32_t passes = (30 + db - 1) / db;
    const uint32_t mp = mesh_passes(M);
    const size_t radix = (size_t)1 << db;
    const size_t lb_words = sqk::sort_lookback_words(N, db, passes);
    const size_t lb_words_m = sqk::sort_lookback_words(N, 8, mp);
    // zero region layout (words)
    uint32_t* z = b->d_zero;
    uint32_t* box_ord = z;                               // 8M
    uint32_t* hist = box_ord + 8ull * M;                 // passes * radix
    uint32_t* hist_m = hist + passes * radix;            // mp * 256
    uint32_t* ctr = hist_m + mp * 256;                   // 16
    uint32_t* lb = ctr + 16;                             // lb_words
    uint32_t* lb_m = lb + lb_words;                      // lb_words_m
    uint32_t* flags = lb_m + lb_words_m;                 // N
    const size_t words = (size_t)(flags - z) + N;
    if (words > b->zero_words) return fail(c, SQ_ERR_INVALID, "batch: workspace too small");
    uint32_t* ka = b->d_keys;
    uint32_t* va = ka + N;
    uint32_t* kb = va + N;
    uint32_t* vb = kb + N;
    uint32_t* code_by_tri = vb + N;
    uint32_t* codes = code_by_tri + N;
    if (b->params.builder != SQ_BUILDER_SAH) SQ_CUDA(c, cudaMemsetAsync(z, 0, sizeof(uint32_t) * words, s));
    if (b->params.builder == SQ_BUILDER_SAH) {
        const uint32_t nb = b->params.sah_bins ? b->params.sah_bins : 8u;
        const uint32_t leaf = b->params.leaf_size ? b->params.leaf_size : 8u;
        const int rc = sqk::build_sah_batch(b->d_tris, N, b->d_off, M, nb, leaf, 3u * N + 2u, b->d_nodes, b->d_sah_ws,
                                            c->ctrl, s);
        if (rc) return fail(c, SQ_ERR_CUDA, "batch SAH build: %s", cudaGetErrorString((cudaError_t)rc));
    } else if (N > 0) {
        const uint32_t g = min((N + 255) / 256, (uint32_t)sms() * 8u);
        launch_chained(k_seg_bounds, dim3(g), dim3(256), 0, s, (const float*)b->d_tris, N, (const uint32_t*)b->d_off, M,
                       box_ord);
        launch_chained(k_seg_morton, dim3(g), dim3(256), sizeof(uint32_t) * passes * radix, s, (const float*)b->d_tris, N,
                       (const uint32_t*)b->d_off, M, (const uint32_t*)box_ord, ka, va, code_by_tri, hist, db, passes);
        int w = sqk::sort_passes(ka, va, kb, vb, N, hist, lb, ctr, db, passes, c->ctrl, s);
        uint32_t* sv = w ? vb : va;   // values sorted by code
        uint32_t* mk = w ? ka : kb;   // free key buffer for the mesh keys
        uint32_t* ok = w ? kb : ka;
        uint32_t* ov = w ? va : vb;
        launch_chained(k_mesh_keys, dim3(g), dim3(256), 0, s, (const uint32_t*)sv, N, (const uint32_t*)b->d_off, M, mk);
        sqk::sort_histogram(mk, N, hist_m, 8, mp, s);
        const int w2 = sqk::sort_passes(mk, sv, ok, ov, N, hist_m, lb_m, ctr + 8, 8, mp, c->ctrl, s);
        uint32_t* perm = w2 ? ov : sv;
        launch_chained(k_gather_codes, dim3(g), dim3(256), 0, s, (const uint32_t*)perm, N, (const uint32_t*)code_by_tri,
                       codes);
        // the climb of a single build, per mesh segment; the open-node list
        // after the codes, its count in mesh 0's two spare box words
        sqk::lbvh_climb_seg(codes, perm, b->d_tris, N, b->d_off, M, 3u * N + 2u, b->d_nodes, flags, b->d_info,
                            codes + N, box_ord + 6, c->ctrl, s);
    }
    launch_chained(k_empty_roots, dim3((M + 255) / 256), dim3(256), 0, s, (const uint32_t*)b->d_off, M, b->d_nodes,
                   3u * N + 2u, 2u * N + 2u);
    const bool wide = b->params.wide != 0;
    if (wide) {
        const int rc = sqk::build_bvh8_queue(b->d_nodes, b->d_roots, M, 2u * N + 2u, b->d_tris, N, b->d_nodes8,
                                             b->d_tris8, b->d_ws8, c->ctrl, s);
        if (rc) return fail(c, SQ_ERR_CUDA, "batch collapse: %s", cudaGetErrorString((cudaError_t)rc));
    }
    // trace
    SQ_CUDA(c, cudaMemsetAsync(c->ctrl + 1, 0, 11 * sizeof(uint32_t), s));
    sqk::BatchTraceArgs a;
    memset(&a, 0, sizeof a);
    a.nodes = b->d_nodes;
    a.node_count = 3u * N + 2u + M;
    a.tri_count = N;
    a.nodes8 = b->d_nodes8;
    a.tris8 = static_cast<const float4*>(b->d_tris8);
    a.tris = b->d_tris;
    a.rays = b->d_rays;
    a.jobs = b->d_jobs;
    a.njobs = M;
    a.total_batches = b->total_batches;
    a.mode = b->params.mode;
    a.hits = b->d_hits;
    a.heat = b->d_heat;
    a.work = c->ctrl + 1;
    a.err = c->ctrl;
    a.stats = reinterpret_cast<unsigned long long*>(c->ctrl + 4);
    // per-lane ray refill when most rays are explicit (incoherent); camera
    // tiles keep whole 32-ray batches per warp
    a.refill = 2ull * b->explicit_rays > (uint64_t)b->rays ? 1u : 0u;
    const int block = b->params.block_threads ? (int)b->params.block_threads : 128;
    if (wide && a.mode != SQ_TRACE_REF) sqk::trace8_batch(a, block, s);
    else sqk::trace_batch(a, block, s);
    SQ_CUDA(c, cudaGetLastError());
    return SQ_OK;
}

// (Re)build the job table for the current width and (re)capture the graph.
sq_status prepare(sq_batch* b)
{
    sq_ctx* c = b->ctx;
    const bool wide = b->params.wide != 0 && b->params.mode != SQ_TRACE_REF;
    if (wide && b->tris > sqk::kWide8MaxTris)
        return fail(c, SQ_ERR_UNSUPPORTED, "batch: the 8-wide BVH takes at most 2^27 triangles (%u)", b->tris);
    for (uint32_t m = 0; m < b->meshes; ++m) b->jobs[m].root = wide ? m : 3u * b->tris + 2u + m;
    SQ_CUDA(c, cudaMemcpyAsync(b->d_jobs, b->jobs.data(), sizeof(sqk::BatchJob) * b->meshes, cudaMemcpyHostToDevice,
                               c->stream));
    // one eager run initialises every kernel's launch configuration, then capture
    sq_status st = enqueue_run(b);
    if (st != SQ_OK) return st;
    SQ_CUDA(c, cudaStreamSynchronize(c->stream));
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->captured = false;
    if (b->params.flags & SQ_BATCH_GRAPH) {
        cudaGraph_t g = nullptr;
        SQ_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        st = enqueue_run(b);
        cudaGraph_t captured = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &captured);
        if (st != SQ_OK) { if (captured) cudaGraphDestroy(captured); return st; }
        if (e != cudaSuccess) return fail(c, SQ_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        g = captured;
        const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) return fail(c, SQ_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
        b->captured = true;
    }
    return check_device_error(c, nullptr);
}

std::string size_class(const sq_batch* b)
{
    char buf[128];
    auto bucket = [](double v) { return v > 0 ? (int)std::floor(std::log2(v) * 2.0) : -1; };
    snprintf(buf, sizeof buf, "meshes%d_tris%d_rays%d_mode%u_builder%u", bucket(b->meshes), bucket(b->tris),
             bucket(b->rays), b->params.mode, b->params.builder);
    return buf;
}

}  // namespace

extern "C" {

sq_status sq_batch_create(sq_ctx* c, const sq_batch_mesh* meshes, uint32_t mesh_count, const sq_batch_params* params,
                          sq_batch** out)
{
    if (!c || !meshes || !params || !out || mesh_count == 0) return fail(c, SQ_ERR_INVALID, "sq_batch_create: bad argument");
    if (params->mode > SQ_TRACE_ANYHIT) return fail(c, SQ_ERR_INVALID, "sq_batch_create: unknown mode");
    if (params->builder != SQ_BUILDER_MORTON && params->builder != SQ_BUILDER_SAH)
        return fail(c, SQ_ERR_UNSUPPORTED, "sq_batch_create: batches build with the Morton or the SAH builder");
    if (params->builder == SQ_BUILDER_SAH &&
        ((params->sah_bins && params->sah_bins != 8 && params->sah_bins != 16 && params->sah_bins != 32) ||
         params->leaf_size > 65535u))
        return fail(c, SQ_ERR_INVALID, "sq_batch_create: SAH bins must be 8, 16 or 32 and leaf_size at most 65535");
    *out = nullptr;
    Guard g(c->device);
    sq_batch* b = new (std::nothrow) sq_batch;
    if (!b) return fail(c, SQ_ERR_OOM, "host allocation failed");
    b->ctx = c;
    b->params = *params;
    b->meshes = mesh_count;
    std::vector<uint32_t> off(mesh_count + 1, 0);
    uint64_t total = 0, rays = 0, xrays = 0, batches = 0;
    b->jobs.resize(mesh_count);
    for (uint32_t m = 0; m < mesh_count; ++m) {
        off[m] = (uint32_t)total;
        total += meshes[m].tri_count;
        const sq_ray_source& rs = meshes[m].rays;
        sqk::BatchJob& j = b->jobs[m];
        memset(&j, 0, sizeof j);
        j.ray_kind = rs.kind;
        j.tri_offset = off[m];
        j.out_offset = (uint32_t)rays;
        j.batch_begin = (uint32_t)batches;
        uint64_t cnt;
        if (rs.kind == SQ_RAYS_EXPLICIT) {
            cnt = rs.ray_count;
            j.ray_offset = (uint32_t)xrays;
            xrays += cnt;
            batches += (cnt + 31) / 32;
        } else if (rs.kind == SQ_RAYS_PINHOLE || rs.kind == SQ_RAYS_REFERENCE_CAMERA) {
            j.width = rs.width;
            j.height = rs.height;
            cnt = (uint64_t)rs.width * rs.height;
            batches += (uint64_t)((rs.width + 7) / 8) * ((rs.height + 3) / 4);
            camera_params(rs, j.cam);
        } else {
            delete b;
            return fail(c, SQ_ERR_INVALID, "sq_batch_create: unknown ray kind for mesh %u", m);
        }
        j.ray_count = (uint32_t)cnt;
        rays += cnt;
    }
    off[mesh_count] = (uint32_t)total;
    if (total >= (1u << 28) || rays >= (1u << 31)) { delete b; return fail(c, SQ_ERR_INVALID, "batch too large"); }
    const uint32_t N = (uint32_t)total, M = mesh_count;
    b->tris = N;
    b->rays = (uint32_t)rays;
    b->explicit_rays = (uint32_t)xrays;
    b->total_batches = (uint32_t)batches;
    // device buffers
    const size_t mp = mesh_passes(M);
    size_t zero = 8ull * M + 4 * 1024 + mp * 256 + 16 + sqk::sort_lookback_words(N, 10, 3) +
                  sqk::sort_lookback_words(N, 6, 5) + sqk::sort_lookback_words(N, 8, 4) +
                  sqk::sort_lookback_words(N, 8, mp) + N + 64;
    b->zero_words = zero;
    b->d_tris = static_cast<float*>(dalloc(c, sizeof(float) * 9ull * (N ? N : 1)));
    b->d_off = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * (M + 1)));
    b->d_rays = static_cast<float*>(dalloc(c, sizeof(sq_ray) * (xrays ? xrays : 1)));
    b->d_jobs = static_cast<sqk::BatchJob*>(dalloc(c, sizeof(sqk::BatchJob) * M));
    b->d_roots = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * M));
    b->d_nodes = static_cast<Node*>(dalloc(c, sizeof(Node) * (3ull * N + 2 + M)));
    b->d_nodes8 = dalloc(c, 80ull * (sqk::bvh8_capacity(N) + M));
    b->d_tris8 = dalloc(c, sqk::bvh8_tri_bytes(N));
    b->d_ws8 = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * (sqk::bvh8_ws_words(N) + 4ull * M)));
    b->d_zero = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * zero));
    b->d_keys = static_cast<uint32_t*>(dalloc(c, sizeof(uint32_t) * 7ull * (N ? N : 1)));
    b->d_info = static_cast<float4*>(dalloc(c, sizeof(float4) * 6ull * (N ? N : 1)));
    b->d_hits = static_cast<sq_hit*>(dalloc(c, sizeof(sq_hit) * (rays ? rays : 1)));
    b->d_heat = static_cast<uint8_t*>(dalloc(c, 3ull * (rays ? rays : 1)));
    if (params->builder == SQ_BUILDER_SAH) {
        b->d_sah_ws = dalloc(c, sqk::sah_batch_workspace_bytes(N, M));
        if (!b->d_sah_ws) {
            sq_batch_free(b);
            return fail(c, SQ_ERR_OOM, "batch allocation failed");
        }
    }
    if (!b->d_tris || !b->d_off || !b->d_rays || !b->d_jobs || !b->d_roots || !b->d_nodes || !b->d_nodes8 ||
        !b->d_tris8 || !b->d_ws8 || !b->d_zero || !b->d_keys || !b->d_info || !b->d_hits || !b->d_heat) {
        sq_batch_free(b);
        return fail(c, SQ_ERR_OOM, "batch allocation failed");
    }
    cudaStream_t s = c->stream;
    for (uint32_t m = 0; m < M; ++m) {
        if (meshes[m].tri_count)
            SQ_CUDA(c, cudaMemcpyAsync(b->d_tris + 9ull * off[m], meshes[m].tris, sizeof(float) * 9ull * meshes[m].tri_count,
                                       cudaMemcpyDefault, s));
        if (meshes[m].rays.kind == SQ_RAYS_EXPLICIT && meshes[m].rays.ray_count)
            SQ_CUDA(c, cudaMemcpyAsync(b->d_rays + 8ull * b->jobs[m].ray_offset, meshes[m].rays.rays,
                                       sizeof(sq_ray) * meshes[m].rays.ray_count, cudaMemcpyDefault, s));
    }
    SQ_CUDA(c, cudaMemcpyAsync(b->d_off, off.data(), sizeof(uint32_t) * (M + 1), cudaMemcpyHostToDevice, s));
    std::vector<uint32_t> roots(M);
    for (uint32_t m = 0; m < M; ++m) roots[m] = 3u * N + 2u + m;
    SQ_CUDA(c, cudaMemcpyAsync(b->d_roots, roots.data(), sizeof(uint32_t) * M, cudaMemcpyHostToDevice, s));
    SQ_CUDA(c, cudaStreamSynchronize(s));
    const sq_status st = prepare(b);
    if (st != SQ_OK) {
        sq_batch_free(b);
        return st;
    }
    *out = b;
    return SQ_OK;
}

sq_status sq_batch_run(sq_batch* b, sq_hit* hits, uint8_t* heatmap_rgb)
{
    if (!b) return SQ_ERR_INVALID;
    sq_ctx* c = b->ctx;
    Guard g(c->device);
    cudaStream_t s = c->stream;
    SQ_CUDA(c, cudaEventRecord(c->ev[0], s));
    if (b->captured) {
        SQ_CUDA(c, cudaGraphLaunch(b->graph, s));
    } else {
        const sq_status st = enqueue_run(b);
        if (st != SQ_OK) return st;
    }
    SQ_CUDA(c, cudaEventRecord(c->ev[6], s));
    SQ_CUDA(c, cudaEventRecord(c->ev[3], s));
    SQ_CUDA(c, cudaEventRecord(c->ev[4], s));
    SQ_CUDA(c, cudaEventRecord(c->ev[5], s));
    c->build_timed = true;
    c->trace_timed = false;
    bool host = false;
    if (hits) {
        host |= !is_device_ptr(hits);
        SQ_CUDA(c, cudaMemcpyAsync(hits, b->d_hits, sizeof(sq_hit) * (size_t)b->rays, cudaMemcpyDefault, s));
    }
    if (heatmap_rgb) {
        host |= !is_device_ptr(heatmap_rgb);
        SQ_CUDA(c, cudaMemcpyAsync(heatmap_rgb, b->d_heat, 3ull * b->rays, cudaMemcpyDefault, s));
    }
    if (host) return check_device_error(c, nullptr);
    return SQ_OK;
}

sq_status sq_batch_info_get(const sq_batch* b, sq_batch_info* info)
{
    if (!b || !info) return SQ_ERR_INVALID;
    info->meshes = b->meshes;
    info->tris = b->tris;
    info->rays = b->rays;
    info->graph = b->captured ? 1u : 0u;
    info->params = b->params;
    return SQ_OK;
}

sq_status sq_batch_free(sq_batch* b)
{
    if (!b) return SQ_ERR_INVALID;
    sq_ctx* c = b->ctx;
    Guard g(c->device);
    cudaStreamSynchronize(c->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    void* bufs[] = {b->d_tris, b->d_off, b->d_rays, b->d_jobs, b->d_roots, b->d_nodes, b->d_nodes8, b->d_tris8,
                    b->d_ws8, b->d_zero, b->d_keys, b->d_info, b->d_hits, b->d_heat, b->d_sah_ws};
    for (void* p : bufs) dfree(c, p);
    delete b;
    return SQ_OK;
}

sq_status sq_batch_autotune(sq_batch* b, const char* cache_path, sq_batch_params* best, float* best_ms)
{
    if (!b || !best) return SQ_ERR_INVALID;
    sq_ctx* c = b->ctx;
    Guard g(c->device);
    const std::string key = size_class(b);
    sq_batch_params base = b->params;
    const bool sah = base.builder == SQ_BUILDER_SAH;
    // cache lookup
    if (cache_path) {
        if (FILE* fh = fopen(cache_path, "r")) {
            char line[512];
            while (fgets(line, sizeof line, fh)) {
                char k[160];
                unsigned db = 0, bins = 0, wide = 0, block = 0;
                float ms = 0;
                if (sscanf(line, "{\"key\": \"%159[^\"]\", \"sort_digit_bits\": %u, \"sah_bins\": %u, \"wide\": %u, "
                                 "\"block_threads\": %u, \"ms\": %f}",
                           k, &db, &bins, &wide, &block, &ms) == 6 && key == k) {
                    b->params.sort_digit_bits = db;
                    b->params.sah_bins = bins;
                    b->params.wide = wide;
                    b->params.block_threads = block;
                    fclose(fh);
                    const sq_status st = prepare(b);
                    if (st != SQ_OK) return st;
                    *best = b->params;
                    if (best_ms) *best_ms = ms;
                    return SQ_OK;
                }
            }
            fclose(fh);
        }
    }
    // the builder's own knob: sort digit width (Morton) or bin count (SAH)
    const uint32_t digits[3] = {6, 8, 10}, bin_counts[3] = {8, 16, 32}, widths[2] = {0, 1}, blocks[3] = {64, 128, 256};
    const uint32_t* knob = sah ? bin_counts : digits;
    float best_t = 3.4e38f;
    sq_batch_params best_p = base;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int ki = 0; ki < 3; ++ki)
        for (uint32_t w : widths)
            for (uint32_t bl : blocks) {
                if (w && b->tris > sqk::kWide8MaxTris) continue;  // beyond the 8-wide form's reach
                b->params = base;
                if (sah) b->params.sah_bins = knob[ki];
                else b->params.sort_digit_bits = knob[ki];
                b->params.wide = w;
                b->params.block_threads = bl;
                sq_status st = prepare(b);
                if (st != SQ_OK) { cudaEventDestroy(e0); cudaEventDestroy(e1); return st; }
                float t = 3.4e38f;
                for (int rep = 0; rep < 3; ++rep) {
                    cudaEventRecord(e0, c->stream);
                    if (b->captured) cudaGraphLaunch(b->graph, c->stream);
                    else enqueue_run(b);
                    cudaEventRecord(e1, c->stream);
                    cudaEventSynchronize(e1);
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < t) t = ms;
                }
                if (t < best_t) { best_t = t; best_p = b->params; }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->params = best_p;
    const sq_status st = prepare(b);
    if (st != SQ_OK) return st;
    *best = best_p;
    if (best_ms) *best_ms = best_t;
    if (cache_path) {
        if (FILE* fh = fopen(cache_path, "a")) {
            fprintf(fh, "{\"key\": \"%s\", \"sort_digit_bits\": %u, \"sah_bins\": %u, \"wide\": %u, \"block_threads\": %u, "
                        "\"ms\": %.4f}\n",
                    key.c_str(), best_p.sort_digit_bits, best_p.sah_bins, best_p.wide, best_p.block_threads, best_t);
            fclose(fh);
        }
    }
    return SQ_OK;
}

}  // extern "C"
