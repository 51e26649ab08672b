// sq_trace_dev.cuh -- device pieces of the reference tracer shared by the
// single-ray kernels (sq_trace.cu) and the packet / bundle kernels
// (sq_coherent.cu): the reference camera, Node1 loads and the reference's
// ray-box test.
#pragma once

#include "sq_common.cuh"

namespace sq {

struct Ray {
    float o[3], d[3], tmin, tmax;
};

__device__ __forceinline__ void gen_reference_camera(uint32_t x, uint32_t y, uint32_t w, uint32_t h, const float* org,
                                                     Ray& r)
{
    // src/tracer.cpp:207-216
    const float aspect = (float)w / (float)h;
    float nx = ((float)x + 0.5f) / (float)w;
    nx = nx * 2.0f;
    nx = nx - 1.0f;
    float ny = ((float)y + 0.5f) / (float)h;
    ny = ny * 2.0f;
    ny = ny - 1.0f;
    nx = nx * aspect;
    const float pz = 1.0f;
    float l2 = nx * nx + ny * ny;
    l2 = l2 + pz * pz;
    const float len = sqrtf(l2);
    r.o[0] = org[0]; r.o[1] = org[1]; r.o[2] = org[2];
    r.d[0] = nx / len; r.d[1] = ny / len; r.d[2] = pz / len;
    r.tmin = 0.0f;
    r.tmax = 10000.0f;
}

struct NodeRec {
    float mn[3], mx[3];
    uint32_t cf, child;
};

__device__ __forceinline__ NodeRec load_node(const Node* __restrict__ nodes, uint32_t i)
{
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    NodeRec r;
    r.mn[0] = a.x; r.mn[1] = a.y; r.mn[2] = a.z; r.cf = __float_as_uint(a.w);
    r.mx[0] = b.x; r.mx[1] = b.y; r.mx[2] = b.z; r.child = __float_as_uint(b.w);
    return r;
}

// intersect_ray_aabb<1> (src/tracer.h:12-35)
__device__ __forceinline__ bool box_ref(const NodeRec& nd, const float* o, const float* inv, float tmax)
{
    const float t1x = (nd.mn[0] - o[0]) * inv[0];
    const float t2x = (nd.mx[0] - o[0]) * inv[0];
    const float t1y = (nd.mn[1] - o[1]) * inv[1];
    const float t2y = (nd.mx[1] - o[1]) * inv[1];
    const float t1z = (nd.mn[2] - o[2]) * inv[2];
    const float t2z = (nd.mx[2] - o[2]) * inv[2];
    const float nx = ref_min(t1x, t2x), ny = ref_min(t1y, t2y), nz = ref_min(t1z, t2z);
    const float fx = simd_max(t1x, t2x), fy = simd_max(t1y, t2y), fz = simd_max(t1z, t2z);
    const float front = simd_max(simd_max(nx, ny), nz);
    const float back = ref_min(ref_min(fx, fy), fz);
    return (back >= front) && (back <= tmax);
}

}  // namespace sq
