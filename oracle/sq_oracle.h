/*
 * sq_oracle.h -- CPU restatement of Sequoia's BVH build and trace path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the GPU library is
 * checked against; only tests, the smoke check and the benchmark's CPU
 * baseline load it.  It is never linked into libsequoia_gpu.so.
 *
 * Each function states the reference lines (paths relative to the Sequoia
 * source tree) whose arithmetic it restates.  All floating-point work is
 * IEEE single-op (the library is compiled with -ffp-contract=off) so the
 * results are reproducible on x86-64 and aarch64 and match the GPU kernels,
 * which use the same operation order with round-to-nearest and no FMA.
 *
 * Parity pinning: tests/golden holds outputs of the reference itself, built
 * from its own sources by oracle/Makefile (target `ref`), and the tests check
 * this restatement against them.
 */
#ifndef SQ_ORACLE_H
#define SQ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sqo_node1 {
    float min[3];
    uint16_t count;
    uint16_t flags;
    float max[3];
    uint32_t child;
} sqo_node1;

#define SQO_LEAF 1u
#define SQO_NO_HIT 0xFFFFFFFFu

/* trace modes (same numbering as the library) */
#define SQO_TRACE_REF 0
#define SQO_TRACE_CLOSEST 1
#define SQO_TRACE_ANYHIT 2

/* number of OpenMP threads the oracle may use (0 = all) */
void sqo_set_threads(int n);
int sqo_get_threads(void);

/* per-triangle AABB {min xyz, max xyz} and the scene box (union) */
void sqo_tri_aabbs(const float* tris, uint32_t n, float* aabbs, float* scene);

/* setup_morton + bit_interleave_32 (src/builder.cpp:2204-2237,
 * src/algorithms.cpp:8-14).  bounds_mode 0: primitive AABB union (reference),
 * 1: centroid bounds.  scene_box (6 floats) receives the quantisation box.  */
void sqo_morton_codes(const float* tris, uint32_t n, int bounds_mode,
                      uint32_t* codes, float* scene_box);
uint32_t sqo_bit_interleave_32(uint32_t x, uint32_t y, uint32_t z);

/* radix_sort over (key, value) pairs, stable, ascending
 * (src/algorithms.h:41-113); in place, digit_bits-wide LSD passes covering
 * key_bits bits. */
void sqo_sort_pairs(uint32_t* keys, uint32_t* values, uint32_t n,
                    uint32_t key_bits, uint32_t digit_bits);

/* find_split_morton (src/builder.cpp:2281-2314) over codes[0..count) */
uint32_t sqo_find_split_morton(const uint32_t* codes, uint32_t count);
/* 60-bit codes of build_hierarchy_morton2 (src/builder.cpp:2247-2279,
 * 2316-2349, 2413-2472, 2510-2544) */
uint64_t sqo_bit_interleave_64(uint64_t x, uint64_t y, uint64_t z);
void sqo_morton_codes64(const float* tris, uint32_t n, int bounds_mode, uint64_t* codes, float* scene_box);
void sqo_sort_pairs64(uint64_t* keys, uint32_t* values, uint32_t n);
uint32_t sqo_find_split_morton64(const uint64_t* codes, uint32_t count);
uint32_t sqo_build_morton64(const float* tris, uint32_t n, int bounds_mode, sqo_node1* nodes, uint64_t* codes_out,
                            uint32_t* perm_out);

/* Node capacity of a range-tree layout for n triangles */
uint32_t sqo_node_capacity(uint32_t n, int kind);

/* Morton LBVH: the logical tree of recurse_morton / build_hierarchy_morton
 * (src/builder.cpp:2351-2409, 2474-2508) laid out in the range-tree layout
 * (see sq_oracle.c) with refitted bounds.  codes_out / perm_out receive the
 * sorted codes and permutation (may be NULL).  Returns the root index.      */
uint32_t sqo_build_morton(const float* tris, uint32_t n, int bounds_mode,
                          sqo_node1* nodes, uint32_t* codes_out,
                          uint32_t* perm_out);

/* Binned SAH (src/builder.cpp:114-147, 334-398, 488-628, 1053-1156,
 * 1576-1618) with bins and leaf size as parameters and a stable partition;
 * range-tree layout.  perm_out receives the final triangle order.  Returns
 * the root index, or 0xFFFFFFFF if a leaf would exceed 65535 triangles.     */
uint32_t sqo_build_sah(const float* tris, uint32_t n, uint32_t bins,
                       uint32_t leaf_size, sqo_node1* nodes, uint32_t* perm_out);

/* Grid builder (src/builder.cpp:1665-1753, 2133-2194): 4x4x4 cells in Morton
 * order, one SAH build per cell, 63-node heap above them.  scene_bounds_cells
 * != 0 reproduces the plain grid builder's cell boxes (scene box, F11).     */
uint32_t sqo_build_grid(const float* tris, uint32_t n, uint32_t bins,
                        uint32_t leaf_size, int scene_bounds_cells,
                        sqo_node1* nodes, uint32_t* perm_out);

/* Ray generation.  rays: 8 floats per ray {ox,oy,oz,tmin,dx,dy,dz,tmax},
 * ray index y*w + x.  Reference camera: src/tracer.cpp:202-216.           */
void sqo_rays_reference_camera(uint32_t w, uint32_t h, const float origin[3],
                               float* rays);
/* Pinhole camera basis (double precision, rounded to float):
 * basis = {eye xyz, fwd xyz, right xyz, up xyz, sx, sy}.                   */
void sqo_pinhole_basis(const float eye[3], const float target[3],
                       const float up[3], float vfov_deg, uint32_t w,
                       uint32_t h, float basis[14]);
void sqo_rays_pinhole(uint32_t w, uint32_t h, const float basis[14],
                      float* rays);

/* Traversal.  ids / ts / tests may be NULL.  Returns 0, or 1 if a stack
 * limit was hit (the ray result is then incomplete).                       */
int sqo_trace(const sqo_node1* nodes, uint32_t root, const float* tris,
              const float* rays, uint32_t nrays, int mode, uint32_t* ids,
              float* ts, uint32_t* tests);

/* Brute-force closest hit over all triangles with the watertight test
 * (ties: smallest id).  The canonical closest-hit answer.                   */
void sqo_brute_closest(const float* tris, uint32_t n, const float* rays,
                       uint32_t nrays, uint32_t* ids, float* ts);

/* Heatmap bytes (src/tracer.cpp:222-225): 3 bytes per ray */
void sqo_heatmap(const uint32_t* tests, uint32_t n, uint8_t* rgb);
/* get_heatmap_colour (src/tracer.cpp:25-45) and the colour-ramp heatmap */
void sqo_heatmap_colour(float x, float rgb[3]);
void sqo_heatmap_ramp(const float* values, uint32_t n, uint8_t* rgb);
/* trace_packet<k> (bundle = 0; k = 1, 2, 4, 8) or trace_bundle<k> (bundle =
 * 1; k = 16, 64) heatmap of the reference camera at origin, w x h (w and h
 * multiples of the packet or tile size).  Returns 0, 1 on a stack overflow,
 * -1 on bad arguments. */
int sqo_trace_coherent(const sqo_node1* nodes, uint32_t root, uint32_t w, uint32_t h, const float origin[3],
                       int bundle, uint32_t k, uint8_t* rgb);

/* FP64 re-intersection of hit (ray, triangle) pairs: t64 of the ray with the
 * triangle's plane, in double from the FP32 inputs.  NaN for misses.       */
void sqo_reintersect_f64(const float* tris, const float* rays, uint32_t nrays,
                         const uint32_t* ids, double* t64);

/* Canonical BFS form of a tree, independent of its layout: records in BFS
 * order from the root; an internal record's child is rewritten as the BFS
 * ordinal of its first child.  Returns the number of records, or
 * 0xFFFFFFFF if the walk exceeds cap or leaves the node array.             */
uint32_t sqo_canonical_bfs(const sqo_node1* nodes, uint32_t node_count,
                           uint32_t root, sqo_node1* out, uint32_t cap);

/* Reachability: counts[t] = number of leaf records that reach triangle t.
 * Returns the number of records visited, or 0xFFFFFFFF on a bad index.     */
uint32_t sqo_leaf_reach(const sqo_node1* nodes, uint32_t node_count,
                        uint32_t root, uint32_t n, uint32_t* counts);

#ifdef __cplusplus
}
#endif

#endif
