// sq_bvh8_dev.cuh -- the 8-wide quantised node shared by the collapse
// (sq_bvh8.cu) and the traversal (sq_bvh8_trace.cu).
//
// Node (80 bytes, five 16-byte loads):
//   origin xyz (float), exponents (3 bytes, biased by 127) + inner-child mask,
//   first inner child node, first leaf triangle, 4-bit triangle count per
//   child slot, and per child slot qlo xyz / qhi xyz (8 bits each).
// Child box on axis a: [origin_a + qlo * 2^e_a, origin_a + qhi * 2^e_a].
// Leaf triangles sit in a 48-byte triangle array in leaf order, with the
// original triangle index in the fourth float of the first vertex.
#pragma once

#include "sq_common.cuh"

namespace sq {

struct __align__(16) Node8 {
    float ox, oy, oz;
    uint32_t exps_imask;  // e_x | e_y << 8 | e_z << 16 | imask << 24 (exponents biased by 127)
    uint32_t child_base;
    uint32_t tri_base;
    uint32_t counts;      // 4 bits per child slot: triangles of a leaf child (0: inner or empty)
    uint32_t valid;       // bit per child slot: slot used
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(Node8) == 80, "Node8 is 80 bytes");

__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((uint32_t)(e + 127) << 23); }

}  // namespace sq
