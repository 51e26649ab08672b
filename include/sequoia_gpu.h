/*
 * sequoia_gpu.h -- C ABI of the GB300 BVH build and ray-trace library
 * (libsequoia_gpu.so).
 *
 * This header is the drop-in boundary for Sequoia's build/trace path.  Every
 * entry point names the reference interface it replaces (paths are relative
 * to the Sequoia source tree).  Plain pointers and sizes only: no C++, no
 * torch, no CUDA types in the signatures (a CUDA stream is passed as void*).
 *
 * Memory: every pointer argument may be host memory (pageable or pinned) or
 * device memory of the context's GPU; the library detects which and copies
 * as needed.  Calls whose outputs are all device pointers are asynchronous on
 * the context stream; calls with a host output synchronise before returning.
 *
 * Errors: every call returns sq_status; sq_last_error() gives the message of
 * the last failing call on that context.  Kernels never spin without a bound:
 * a bounded wait that expires, or a traversal stack that would overflow,
 * raises a device error word that the next synchronising call reports as
 * SQ_ERR_DEVICE.
 *
 * Threading: one context is single-threaded; different contexts are
 * independent and may be used from different host threads.
 */
#ifndef SEQUOIA_GPU_H
#define SEQUOIA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SQ_ABI_VERSION 2u

typedef enum sq_status {
    SQ_OK = 0,
    SQ_ERR_INVALID = 1,     /* bad argument (null pointer, size, mode)        */
    SQ_ERR_CUDA = 2,        /* a CUDA runtime call failed                     */
    SQ_ERR_OOM = 3,         /* device or pinned allocation failed             */
    SQ_ERR_DEVICE = 4,      /* a kernel raised the device error word          */
    SQ_ERR_UNSUPPORTED = 5, /* valid request this build does not implement    */
    SQ_ERR_NO_DEVICE = 6,   /* no CUDA device / extension unusable            */
    SQ_ERR_TOO_LARGE = 7    /* request exceeds a fixed capacity (see below)   */
} sq_status;

/* Device error word bits (sq_device_error) */
#define SQ_DEVERR_STACK_OVERFLOW   0x1u  /* traversal stack limit reached          */
#define SQ_DEVERR_LOOKBACK_TIMEOUT 0x2u  /* radix-sort look-back wait ran out       */
#define SQ_DEVERR_TOPOLOGY         0x4u  /* LBVH climb found an inconsistent state  */
#define SQ_DEVERR_SAH_QUEUE        0x8u  /* SAH task queue overflow / wait ran out  */
#define SQ_DEVERR_NODE_COUNT       0x10u /* a node would hold more than 65535 prims */
#define SQ_DEVERR_COPY_TIMEOUT     0x20u /* a bulk copy into shared memory did not complete */

typedef struct sq_ctx sq_ctx;
typedef struct sq_bvh sq_bvh;

/* Same 36-byte layout as Sequoia's Triangle (src/aabb.h:17-24). */
typedef struct sq_triangle {
    float v0[3];
    float v1[3];
    float v2[3];
} sq_triangle;

/* Same 32-byte layout as Sequoia's Node1 (src/aabb.h:34-42).  A leaf has
 * flags == SQ_NODE_LEAF, count == 1 and child == triangle index; an internal
 * node has children [child, child + count).                                  */
typedef struct sq_node1 {
    float min[3];
    uint16_t count;
    uint16_t flags;
    float max[3];
    uint32_t child;
} sq_node1;
#define SQ_NODE_LEAF 1u

/* Same 32-byte layout as Sequoia's Ray<1> (src/ray.h:8-14). */
typedef struct sq_ray {
    float origin[3];
    float tmin;
    float dir[3];
    float tmax;
} sq_ray;

/* One record per ray. id == SQ_NO_HIT when nothing was hit.  In SQ_TRACE_REF
 * mode id is 0 (hit) or SQ_NO_HIT (miss) and t is 0, because the reference
 * tracer keeps only a hit flag (src/tracer.h:112-115).                        */
typedef struct sq_hit {
    uint32_t id;
    float t;
    uint32_t tests; /* ray-box tests performed: the heatmap counter           */
} sq_hit;
#define SQ_NO_HIT 0xFFFFFFFFu

typedef struct sq_options {
    int device;      /* CUDA device ordinal                                  */
    void* stream;    /* cudaStream_t to run on; NULL = context-owned stream  */
    uint32_t flags;  /* SQ_OPT_*                                             */
} sq_options;
/* Run on options->stream exactly as given, even when it is NULL (the legacy
 * default stream), instead of creating a context-owned stream.              */
#define SQ_OPT_EXTERNAL_STREAM 0x1u

typedef enum sq_builder_kind {
    SQ_BUILDER_MORTON = 0, /* Builder::build_hierarchy_morton (src/builder.cpp:2474) */
    SQ_BUILDER_SAH = 1,    /* Builder::build_hierarchy        (src/builder.cpp:1576) */
    SQ_BUILDER_GRID = 2    /* Builder::build_hierarchy_grid   (src/builder.cpp:2133) */
} sq_builder_kind;

/* Morton quantisation domain.  PRIMITIVE follows the reference: codes are
 * normalised by the union of the triangle AABBs (src/builder.cpp:2206-2215).
 * CENTROID normalises by the bounds of the centroids.                        */
#define SQ_MORTON_BOUNDS_PRIMITIVE 0u
#define SQ_MORTON_BOUNDS_CENTROID 1u

/* build flags */
#define SQ_BUILD_GRID_SCENE_BOUNDS 0x1u /* grid: give cell nodes the scene box,
                                           as the plain reference grid builder
                                           does (src/builder.cpp:2173-2174)      */
#define SQ_BUILD_MORTON64 0x4u          /* Morton builder over 60-bit codes (20
                                           bits per axis, 8 sort passes) as
                                           Builder::build_hierarchy_morton2
                                           (src/builder.cpp:2510)               */
#define SQ_BUILD_WIDE8 0x2u             /* also collapse the binary tree into an
                                           8-wide BVH with 8-bit quantised child
                                           boxes (rounded outward); closest and
                                           any-hit traces then use it.  At most
                                           2^27 triangles (SQ_ERR_UNSUPPORTED
                                           above that)                         */

typedef struct sq_build_params {
    uint32_t kind;            /* sq_builder_kind                                  */
    uint32_t sah_bins;        /* SAH/grid bins: 8, 16 or 32 (0 = 8)               */
    uint32_t leaf_size;       /* SAH/grid: leaf when count <= leaf_size (0 = 8)   */
    uint32_t sort_digit_bits; /* Morton sort digit width 6, 8 or 10 (0 = 8)       */
    uint32_t morton_bounds;   /* SQ_MORTON_BOUNDS_*                               */
    uint32_t flags;           /* SQ_BUILD_*                                       */
} sq_build_params;

typedef struct sq_bvh_info {
    uint32_t node_capacity;   /* entries in the node array                        */
    uint32_t root;            /* root node index                                  */
    uint32_t tri_count;
    uint32_t kind;            /* sq_builder_kind, or 0xFFFFFFFF for imported trees */
    float scene_min[3];
    float scene_max[3];
    uint32_t wide_nodes;      /* 8-wide quantised nodes (0 if none)               */
    uint32_t wide_levels;     /* levels of the 8-wide tree                        */
    uint32_t wide_launches;   /* kernel launches of the 8-wide collapse           */
} sq_bvh_info;

typedef enum sq_trace_mode {
    SQ_TRACE_REF = 0,     /* the reference tracer: every box test counted, no
                             near-child order, no early exit, Moller-Trumbore
                             hit flag (src/tracer.cpp:47-65, src/tracer.h:12-116) */
    SQ_TRACE_CLOSEST = 1, /* near-child order, t shrink, watertight test         */
    SQ_TRACE_ANYHIT = 2,  /* as CLOSEST, stops at the first accepted hit         */
    SQ_TRACE_PACKET = 3,  /* trace_packet<k> (src/tracer.cpp:232-281): packets of
                             k = 1, 2, 4 or 8 rays count box tests together;
                             heatmap only (hits must be NULL), reference camera,
                             width and height multiples of the packet block     */
    SQ_TRACE_BUNDLE = 4   /* trace_bundle<k> (src/tracer.cpp:292-362): tiles of
                             k = 16 or 64 rays tested as a bundle, split into
                             packets of 8; same restrictions as PACKET          */
} sq_trace_mode;
/* The packet or bundle size k rides in bits 16..23 of the mode:
 * SQ_TRACE_PACKET | SQ_TRACE_WIDTH(8), SQ_TRACE_BUNDLE | SQ_TRACE_WIDTH(64). */
#define SQ_TRACE_WIDTH(k) ((uint32_t)(k) << 16)
/* OR into the mode: trace the binary (Node1) tree even when the BVH also has
 * an 8-wide quantised tree.                                                  */
#define SQ_TRACE_FORCE_BINARY 0x100u
/* OR into a CLOSEST or ANYHIT mode to choose how rays are assigned to GPU
 * lanes (the results are the same either way; only the speed differs):
 *   SQ_TRACE_SCHED_REFILL  a lane whose ray has finished takes the next ray
 *                          at once (best for incoherent rays);
 *   SQ_TRACE_SCHED_TILES   a warp traces 32 rays (an 8x4 pixel tile, or 32
 *                          consecutive explicit rays) to the end, then takes
 *                          the next 32 (best for coherent camera rays).
 * Without either: the binary tree uses TILES; the 8-wide tree uses REFILL
 * for explicit rays and TILES for camera rays.                               */
#define SQ_TRACE_SCHED_REFILL 0x200u
#define SQ_TRACE_SCHED_TILES 0x400u
/* OR into any mode: heatmap pixels in the reference's colour ramp
 * get_heatmap_colour (src/tracer.cpp:25-45, defined there but unused) of
 * tests / 200 -- black, blue, cyan, green, yellow, red -- each channel
 * (uint8)(c * 255), instead of the grey (uint8)(min(1, tests / 200) * 255). */
#define SQ_TRACE_HEAT_RAMP 0x800u

typedef enum sq_ray_kind {
    SQ_RAYS_REFERENCE_CAMERA = 0, /* trace()'s camera (src/tracer.cpp:202-216)   */
    SQ_RAYS_PINHOLE = 1,          /* eye / look-at / vertical FOV pinhole        */
    SQ_RAYS_EXPLICIT = 2          /* caller-supplied sq_ray array                */
} sq_ray_kind;

typedef struct sq_ray_source {
    uint32_t kind;     /* sq_ray_kind                                         */
    uint32_t width;    /* camera kinds: image size; ray i = y * width + x     */
    uint32_t height;
    float origin[3];   /* REFERENCE_CAMERA: camera position; PINHOLE: eye     */
    float target[3];   /* PINHOLE: look-at point                              */
    float up[3];       /* PINHOLE: up vector                                  */
    float vfov_deg;    /* PINHOLE: vertical field of view in degrees          */
    const sq_ray* rays;/* EXPLICIT: host or device array                      */
    uint32_t ray_count;/* EXPLICIT: number of rays                            */
} sq_ray_source;

/* ---- context ------------------------------------------------------------ */

/* No reference counterpart: the reference is a global OpenMP program.       */
sq_status sq_create(sq_ctx** out, const sq_options* options);
/* Releases all device memory the context holds, that of its BVHs and
 * batches included: free those first; none may be used or freed after.     */
sq_status sq_destroy(sq_ctx* ctx);
const char* sq_last_error(const sq_ctx* ctx);
uint32_t sq_abi_version(void);
/* Wait for all work on the context stream, then report and clear the device
 * error word (SQ_ERR_DEVICE if it was set; the bits go to *device_error).    */
sq_status sq_sync(sq_ctx* ctx, uint32_t* device_error);

/* ---- build -------------------------------------------------------------- */

/* Replaces Builder::build_hierarchy, build_hierarchy_morton and
 * build_hierarchy_grid (src/builder.h:85-94, src/builder.cpp:1576, 2474,
 * 2133).  tris: n triangles, host or device.  A device tris pointer is
 * referenced, not copied, exactly as Hierarchy::tri_base references the
 * caller's vector (src/builder.cpp:1613): it must outlive the BVH.  The BVH
 * lives on the device until sq_bvh_free.  Morton builds return without
 * waiting for the device; the next call on the context (a trace) is ordered
 * after the build on the context's stream.                                   */
sq_status sq_build(sq_ctx* ctx, const sq_triangle* tris, uint32_t n,
                   const sq_build_params* params, sq_bvh** out);
sq_status sq_bvh_free(sq_bvh* bvh);
/* Sizes of a built BVH.  The first call after an 8-wide build waits for the
 * build to finish (its node count is read back then).                        */
sq_status sq_bvh_get_info(const sq_bvh* bvh, sq_bvh_info* info);

/* Copy the node array out in Sequoia's Node1 layout so that the reference's
 * traverse() (src/tracer.cpp:47) can walk a GPU-built tree.  nodes may be host
 * or device; cap is its capacity in entries.                                 */
sq_status sq_bvh_export_node1(sq_bvh* bvh, sq_node1* nodes, uint32_t cap,
                              uint32_t* node_count, uint32_t* root);

/* Upload a Node1 tree built elsewhere (the reference's Hierarchy: node_base,
 * node_count, root_index, tri_base; src/aabb.h:197-205) so the GPU traverses
 * exactly that tree.  Triangles are copied to the device.                    */
sq_status sq_bvh_import_node1(sq_ctx* ctx, const sq_node1* nodes,
                              uint32_t node_count, uint32_t root,
                              const sq_triangle* tris, uint32_t n,
                              sq_bvh** out);

/* Build stages, exposed for parity checks and for callers that want only a
 * stage.  Replaces setup_morton + bit_interleave_32 (src/builder.cpp:2204-
 * 2237, src/algorithms.cpp:8-14): codes[i] is the 30-bit Morton code of
 * triangle i; scene_box receives {min xyz, max xyz} of the quantisation box. */
sq_status sq_morton_codes(sq_ctx* ctx, const sq_triangle* tris, uint32_t n,
                          uint32_t bounds_mode, uint32_t* codes,
                          float* scene_box);

/* Replaces radix_sort<uint32_t, RadixInput32> (src/algorithms.h:89-113):
 * stable ascending sort of (key, value) pairs by key over the low key_bits
 * bits (1..32), onesweep with decoupled look-back.  keys_out / values_out
 * may alias keys_in / values_in.                                            */
sq_status sq_radix_sort_pairs(sq_ctx* ctx, const uint32_t* keys_in,
                              const uint32_t* values_in, uint32_t n,
                              uint32_t key_bits, uint32_t digit_bits,
                              uint32_t* keys_out, uint32_t* values_out);

/* The sorted Morton codes and triangle permutation of the last Morton build
 * of this BVH (n entries each).                                              */
sq_status sq_bvh_export_sorted(sq_bvh* bvh, uint32_t* codes, uint32_t* perm);
/* The same for a SQ_BUILD_MORTON64 build: the sorted 60-bit codes of
 * setup_morton2 + radix_sort<uint64_t> (src/builder.cpp:2247-2279, 2521). */
sq_status sq_bvh_export_sorted64(sq_bvh* bvh, uint64_t* codes, uint32_t* perm);

/* Radix sort that allocates nothing.  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc / cudaFree (for example a host
 * whose memory pool has already reserved the GPU's memory, or a loop that
 * cannot afford cudaFree's implicit device synchronisation).  Same result as
 * sq_radix_sort_pairs, but every pointer must be device memory of the current
 * device, no context is used, and the sort's scratch is one fixed device
 * array inside the library (about 12.6 MB, held on each GPU where the
 * library's code is loaded until the process exits).  n above
 * SQ_NOALLOC_MAX_KEYS returns SQ_ERR_TOO_LARGE before touching anything.
 * Runs on `stream` (NULL = legacy default stream).  Every call ends by
 * reading the scratch's error word back and synchronising `stream`, so it
 * returns only when the sort has finished.  The first call on a device also
 * looks up the scratch address there; make it before any stream capture
 * begins.  Calls share the scratch, so
 * calls that overlap on the GPU race and must not be issued.  keys_out /
 * values_out may alias keys_in / values_in.                                */
#define SQ_NOALLOC_MAX_KEYS (1u << 20)
sq_status sq_radix_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* values_in, uint32_t n,
                                      uint32_t key_bits, uint32_t digit_bits, uint32_t* keys_out,
                                      uint32_t* values_out, void* stream);

/* ---- trace -------------------------------------------------------------- */

/* Replaces trace() and traverse() (src/tracer.h:118-135,
 * src/tracer.cpp:47-65, 195-230).  hits: one sq_hit per ray (may be NULL);
 * heatmap_rgb: width*height*3 bytes, byte = (uint8)(min(1, tests/200)*255)
 * in all three channels as in src/tracer.cpp:222-225 (may be NULL; for
 * explicit rays it holds ray_count*3 bytes).  Outputs host or device:
 * device outputs are written on the context's stream and the call returns
 * without waiting; host outputs are complete when the call returns.
 * Page-locked host outputs (cudaHostAlloc / cudaHostRegister) have their
 * transfer overlap the trace: a camera image of 2^21 rays or more on an
 * 8-wide tree is traced in row bands into device memory, each band copied
 * to the host on a side stream while later bands trace; other traces write
 * them in place from the kernel.  Pageable host outputs go through a device
 * buffer and one copy.                                                       */
sq_status sq_trace(sq_ctx* ctx, const sq_bvh* bvh, const sq_ray_source* rays,
                   uint32_t mode, sq_hit* hits, uint8_t* heatmap_rgb);

/* traverse() (src/tracer.h:118, src/tracer.cpp:47-65) for n explicit rays
 * (host or device): the reference's traversal -- every box of the node
 * group [index, index + count) tested, then the groups of the inner nodes
 * hit, no ordering, no early exit, Moller-Trumbore triangle tests -- started
 * from that node group rather than the root.  hits[i] (host or device) gets
 * id 0 (hit) or SQ_NO_HIT and the ray's box-test count, as SQ_TRACE_REF.
 * Host hits are complete when the call returns.                             */
sq_status sq_traverse(sq_ctx* ctx, const sq_bvh* bvh, uint32_t index, uint32_t count, const sq_ray* rays,
                      uint32_t n, sq_hit* hits);

/* Many ray batches against one BVH in one kernel launch.  No reference
 * counterpart (the reference traces one image per call, src/tracer.cpp:195).
 * Each of the `count` batches is a ray source of its own: explicit rays in
 * their own buffer (device buffers are read in place, others are copied
 * first) or a camera.  hits / heatmap_rgb (optional, host or device) receive
 * the results batch after batch, exactly as `count` sq_trace calls would
 * write them; one launch traces all batches, its warps taking 32-ray pieces
 * of any batch.  mode: SQ_TRACE_REF, CLOSEST or ANYHIT, with
 * SQ_TRACE_FORCE_BINARY and the schedule flags (default: per-lane refill
 * when most rays are explicit).                                              */
sq_status sq_trace_batches(sq_ctx* ctx, const sq_bvh* bvh, const sq_ray_source* batches, uint32_t count,
                           uint32_t mode, sq_hit* hits, uint8_t* heatmap_rgb);

/* ---- batches: many meshes and ray tiles, one launch sequence ------------ */

/* Build-and-trace of many independent meshes at once: the reference's
 * build_hierarchy_morton or build_hierarchy (binned SAH) + trace
 * (src/builder.cpp:2474, 1576, src/tracer.cpp:195) run for every mesh, as
 * one sequence of launches over all meshes, captured once in a CUDA graph
 * (SQ_BATCH_GRAPH) and replayed by sq_batch_run.  The sequence never waits
 * on the host: the SAH build runs a fixed number of level launches with
 * device-side task counts.  The reference has no batched form; each mesh's
 * result equals a separate sq_build + sq_trace of that mesh with the same
 * builder settings (same trees, same hits).                               */
typedef struct sq_batch sq_batch;

typedef struct sq_batch_mesh {
    const sq_triangle* tris;   /* host or device; copied into the batch     */
    uint32_t tri_count;
    sq_ray_source rays;        /* camera or explicit rays for this mesh     */
} sq_batch_mesh;

#define SQ_BATCH_GRAPH 0x1u    /* capture the run in a CUDA graph           */

typedef struct sq_batch_params {
    uint32_t builder;          /* SQ_BUILDER_MORTON or SQ_BUILDER_SAH       */
    uint32_t sort_digit_bits;  /* Morton: 6, 8 or 10 (0 = 8)                */
    uint32_t wide;             /* 1: trace the 8-wide quantised BVH         */
    uint32_t block_threads;    /* trace block: 64, 128 or 256 (0 = 128)     */
    uint32_t mode;             /* sq_trace_mode                             */
    uint32_t flags;            /* SQ_BATCH_*                                */
    uint32_t sah_bins;         /* SAH: 8, 16 or 32 bins (0 = 8)             */
    uint32_t leaf_size;        /* SAH: leaf when count <= leaf_size (0 = 8) */
} sq_batch_params;

typedef struct sq_batch_info {
    uint32_t meshes, tris, rays;
    uint32_t graph;            /* 1 if the run is a captured CUDA graph     */
    sq_batch_params params;
} sq_batch_info;

sq_status sq_batch_create(sq_ctx* ctx, const sq_batch_mesh* meshes, uint32_t mesh_count,
                          const sq_batch_params* params, sq_batch** out);
/* One run: build every mesh and trace every tile.  hits / heatmap_rgb (host
 * or device, optional) receive all rays' records, mesh after mesh; triangle
 * ids are per mesh.                                                          */
sq_status sq_batch_run(sq_batch* batch, sq_hit* hits, uint8_t* heatmap_rgb);
sq_status sq_batch_info_get(const sq_batch* batch, sq_batch_info* info);
sq_status sq_batch_free(sq_batch* batch);
/* Time every sort digit width (6/8/10; Morton batches) or SAH bin count
 * (8/16/32; SAH batches), BVH width (binary / 8-wide) and trace block shape
 * (64/128/256) on this batch, keep the fastest (the batch is re-prepared
 * with it) and return it.  Digit width, width and block shape never change
 * a result; the SAH bin count changes the trees, so box-test counts and
 * any-hit ids may change with it (closest-hit ids and t do not).
 * cache_path (optional): JSON-lines file; a cached choice for the batch's
 * size class is used without timing, a new choice is appended.             */
sq_status sq_batch_autotune(sq_batch* batch, const char* cache_path, sq_batch_params* best,
                            float* best_ms);

/* Device time of the stages of the last sq_build / sq_trace on this context,
 * in milliseconds, measured with CUDA events on the context stream
 * (synchronises).  stage_ms[0] = build total, [1] = bounds+codes, [2] = sort,
 * [3] = topology+refit, [4] = trace; [5] and [6] are the last trace's total
 * ray-box and ray-triangle test counts (as floats); [7] = the 8-wide
 * collapse (included in [0]).                                                */
sq_status sq_last_timings(sq_ctx* ctx, float stage_ms[8]);

/* Counters of the last sq_trace on this context (synchronises): stats[0] =
 * ray-box tests, [1] = ray-triangle tests, [2] = bytes the traversal
 * requested (ray in, hit record and heatmap out, node records, triangles),
 * [3] = nodes visited (binary: node records tested; 8-wide: nodes loaded).
 * No reference counterpart (the reference keeps only the per-ray count,
 * src/tracer.h:32).                                                          */
sq_status sq_last_trace_stats(sq_ctx* ctx, uint64_t stats[4]);

/* ---- failure-detection test hooks ---------------------------------------- */

/* Fault injection for the failure-detection tests; no reference counterpart
 * (the reference asserts or exits on failure).  Each injection is armed for
 * one use on this context, then clears itself:
 *   SQ_DEBUG_STALL_LOOKBACK  the next sq_radix_sort_pairs, which must be a
 *                            one-pass sort (key_bits <= digit_bits) that
 *                            spans more than one tile (any sort of more than
 *                            16384 keys does), runs without its first tile: the
 *                            look-back of the tiles after it waits on words
 *                            that nothing publishes, gives up after `limit`
 *                            polls and raises SQ_DEVERR_LOOKBACK_TIMEOUT.
 *   SQ_DEBUG_STALL_BARRIER   the next 8-wide collapse's grid barrier waits
 *                            for one block more than the grid: every block
 *                            gives up after `limit` polls and raises
 *                            SQ_DEVERR_SAH_QUEUE.
 *   SQ_DEBUG_FAIL_ALLOC      device allocation number `limit` from now (0 =
 *                            the next one) fails as if the GPU were out of
 *                            memory; the call reports SQ_ERR_OOM.
 *   SQ_DEBUG_OFF             disarm all of them.
 * No injection faults or hangs the GPU: a wait that gives up returns, the
 * kernel finishes, and the context stays usable (the error word is reported
 * and cleared by the next sq_sync).  The results of the call that carried
 * the injection are not valid.                                               */
#define SQ_DEBUG_OFF 0u
#define SQ_DEBUG_STALL_LOOKBACK 1u
#define SQ_DEBUG_STALL_BARRIER 2u
#define SQ_DEBUG_FAIL_ALLOC 3u
sq_status sq_debug_inject(sq_ctx* ctx, uint32_t what, uint32_t limit);
/* Device memory the context holds in its caching allocator: out[0] / out[1]
 * = blocks / bytes held by live objects (BVHs, batches, buffers of a call in
 * flight), out[2] / out[3] = blocks / bytes cached for reuse.               */
sq_status sq_debug_memory(const sq_ctx* ctx, uint64_t out[4]);

#ifdef __cplusplus
}
#endif

#endif /* SEQUOIA_GPU_H */
