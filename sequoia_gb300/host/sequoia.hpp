// sequoia.hpp -- C++ drop-in for Sequoia's build/trace entry points.
//
// The same names, argument meanings and ownership as the reference
// (src/aabb.h:17-24, 180-205, src/builder.h:78-104, src/tracer.h:129-135,
// src/main.cpp:108): Builder::build_hierarchy* return a Hierarchy whose
// node_base was allocated with new[] (the caller delete[]s it) and whose
// tri_base points into the caller's vector; trace() returns a new[]'d
// w*h*3 heatmap.  Every call runs on the GPU through the C ABI of
// sequoia_gpu.h; nothing here computes on the host except the OBJ parse.
//
// Errors: the reference has no error path (it asserts or exits); these
// functions throw sequoia::Error when the library reports one -- no GPU, a
// failed CUDA call, a device error word -- and never fall back to the CPU.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "sequoia_gpu.h"
#include "sequoia_host.h"

namespace sequoia {

struct vec3f1 {
    float x, y, z;
    vec3f1() : x(0), y(0), z(0) {}
    vec3f1(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
};

// src/aabb.h:17-24 (36 bytes)
struct Triangle {
    vec3f1 v0, v1, v2;
    Triangle() = default;
    Triangle(const vec3f1& a, const vec3f1& b, const vec3f1& c) : v0(a), v1(b), v2(c) {}
};

enum AABB_FLAGS { AABB_FLAGS_NONE = 0x00, AABB_FLAGS_LEAF = 0x01 };

// src/aabb.h:180-195 (32 bytes).  Inner node: children child .. child+count-1.
// Leaf: triangles child .. child+count-1 of tri_base.
struct Node1 {
    vec3f1 min;
    uint16_t count;
    uint16_t flags;
    vec3f1 max;
    uint32_t child;
};

struct PluckerTriangle;  // never produced (the reference leaves it null too)

// src/aabb.h:197-205
struct Hierarchy {
    Node1* node_base;
    unsigned node_count;
    Triangle* tri_base;
    PluckerTriangle* plucker_tri_base;
    unsigned tri_count;
    unsigned root_index;
};

static_assert(sizeof(Triangle) == sizeof(sq_triangle), "Triangle layout");
static_assert(sizeof(Node1) == sizeof(sq_node1), "Node1 layout");

struct Error : std::runtime_error {
    sq_status status;
    Error(sq_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

// src/builder.h:78-104.  The reference's variants build the same logical
// trees as the GPU builders they map to: build_hierarchy_horizontal bins its
// top levels by a parallel reduction (src/builder.cpp:400-426, 1479-1574)
// into the same bins as build_hierarchy, so it is the SAH tree; grid_sse and
// grid_m128 are build_hierarchy_grid with each cell node bounded by its own
// triangles (build_hierarchy_grid gives cell nodes the scene box,
// src/builder.cpp:2173-2174).  Both equivalences are checked against the
// reference's own trees.
class Builder {
public:
    static Hierarchy build_hierarchy(std::vector<Triangle>& primitives);
    static Hierarchy build_hierarchy_morton(std::vector<Triangle>& primitives);
    static Hierarchy build_hierarchy_morton2(std::vector<Triangle>& primitives);  // 60-bit codes
    static Hierarchy build_hierarchy_grid(std::vector<Triangle>& primitives);
    static Hierarchy build_hierarchy_grid_sse(std::vector<Triangle>& primitives);
    static Hierarchy build_hierarchy_grid_m128(std::vector<Triangle>& primitives);
    static Hierarchy build_hierarchy_horizontal(std::vector<Triangle>& primitives);
};

// src/ray.h:8-14 and 25-30 for one ray (K = 1): the same 32-byte ray layout
// as sq_ray, and the hit flag plus box-test count of traverse().
template <size_t K>
struct Ray;
template <>
struct Ray<1> {
    vec3f1 origin;
    float tmin;
    vec3f1 direction;
    float tmax;
};
template <size_t K>
struct HitAttributes;
template <>
struct HitAttributes<1> {
    int32_t hit = 0;        // all bits set (-1) once a triangle was hit, as the reference's SIMD mask
    int32_t num_tests = 0;  // ray-box tests, added to what the attributes held
};
static_assert(sizeof(Ray<1>) == sizeof(sq_ray), "Ray<1> layout");

// src/tracer.h:118, src/tracer.cpp:47-65: the reference's traversal of one
// ray from the node group [index, index + count) -- usually (root_index, 1)
// -- OR-ing the hit flag into attributes.hit and adding the box tests to
// attributes.num_tests.  One ray per call is one GPU launch; the overload
// below takes many rays at once.
void traverse(Hierarchy& hierarchy, uint32_t index, uint32_t count, Ray<1>& ray, HitAttributes<1>& attributes);
// The same for n rays in one launch (attributes[i] for rays[i]).
void traverse(Hierarchy& hierarchy, uint32_t index, uint32_t count, const Ray<1>* rays,
              HitAttributes<1>* attributes, size_t n);

// src/tracer.cpp:195-230: w*h rays from the reference camera at `origin`, the
// per-ray box-test count as a grey heatmap (new[]'d, w*h*3 bytes).
uint8_t* trace(Hierarchy& hierarchy, uint32_t w, uint32_t h, vec3f1 origin);

// src/tracer.h:131-135: the packet (K = 1, 2, 4, 8) and bundle (K = 16, 64)
// tracers, whose heatmaps count box tests per packet / bundle exactly as the
// reference's do (the same bytes).  w and h must be multiples of the packet
// block (the reference writes outside the image otherwise).
uint8_t* trace_coherent(Hierarchy& hierarchy, uint32_t w, uint32_t h, vec3f1 origin, bool bundle, uint32_t k);
template <size_t K>
uint8_t* trace_packet(Hierarchy& hierarchy, uint32_t w, uint32_t h, vec3f1 origin)
{
    return trace_coherent(hierarchy, w, h, origin, false, (uint32_t)K);
}
template <size_t K>
uint8_t* trace_bundle(Hierarchy& hierarchy, uint32_t w, uint32_t h, vec3f1 origin)
{
    return trace_coherent(hierarchy, w, h, origin, true, (uint32_t)K);
}

// src/main.cpp:108-179, with the same parse (sq_obj_load); prints the same
// "Geometry" summary.  A file that cannot be opened is reported on stderr and
// exits with status 1, as the reference does; a malformed file throws.
std::vector<Triangle> loadOBJFromFile(std::string filename);

// ---- GB300 additions -------------------------------------------------------

// Parameters of the next builds (bins, leaf size, sort digit width, Morton
// bounds, SQ_BUILD_WIDE8).  kind and the grid scene-bounds flag are set by
// the Builder function called.
void set_build_params(const sq_build_params& params);
sq_build_params build_params();
// Threads of the OBJ parse (0 = all hardware threads; the CLI's -threads).
void set_host_threads(uint32_t threads);
// The process-wide context (device from SEQUOIA_DEVICE, default 0).
sq_ctx* context();
// The device tree behind a Hierarchy returned by Builder (null if none).
sq_bvh* device_tree(const Hierarchy& hierarchy);
// delete[] node_base and free the device tree.
void release(Hierarchy& hierarchy);
// Timings of the last build or trace (sq_last_timings).
void last_timings(float stage_ms[8]);

}  // namespace sequoia
