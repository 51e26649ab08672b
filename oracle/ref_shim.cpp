// ref_shim.cpp -- C entry points over the Sequoia reference's own functions.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together
// with the reference's builder.cpp, tracer.cpp, algorithms.cpp and main.cpp
// (taken unmodified from the reference tree, main renamed) into
// oracle/_ref/libseqref_*.so.  It exists only where the reference tree is
// present (x86-64: the reference uses x86 intrinsics), and is used to pin
// the CPU restatement in sq_oracle.c and to produce tests/golden.
#include "aabb.h"
#include "algorithms.h"
#include "builder.h"
#include "ray.h"
#include "tracer.h"

#include <omp.h>

#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

// Same layout and name as the record type local to src/builder.cpp:2196-2202,
// so the reference's setup_morton / find_split_morton link against it.
typedef struct alignas(8) RadixInput32 {
    uint32_t code;
    unsigned index;
    __forceinline operator uint32_t() const { return code; }
    __forceinline bool operator<(const RadixInput32& m) const { return code < m.code; }
} RadixInput32;

// Same layout and name as the 64-bit record of src/builder.cpp:2239-2245.
typedef struct alignas(16) RadixInput64 {
    uint64_t code;
    unsigned index;
    __forceinline operator uint64_t() const { return code; }
    __forceinline bool operator<(const RadixInput64& m) const { return code < m.code; }
} RadixInput64;

void setup_morton(std::vector<Triangle>& primitives, std::vector<RadixInput32>& morton_codes, AABB1& scene_aabb);
unsigned find_split_morton(std::vector<RadixInput32>::iterator begin, std::vector<RadixInput32>::iterator end);
void setup_morton2(std::vector<Triangle>& primitives, std::vector<RadixInput64>& morton_codes, AABB1& scene_aabb);
unsigned find_split_morton2(std::vector<RadixInput64>::iterator begin, std::vector<RadixInput64>::iterator end);
std::vector<Triangle> loadOBJFromFile(std::string filename);
vec3f1 get_heatmap_colour(float normalised);  // src/tracer.cpp:25-45, not declared in a header
// stb_image_write v1.14 as compiled into the reference's main.cpp
extern "C" int stbi_write_bmp(char const* filename, int w, int h, int comp, const void* data);
extern "C" void stbi_flip_vertically_on_write(int flag);

static std::vector<Triangle> to_tris(const float* t, uint32_t n)
{
    std::vector<Triangle> v(n);
    for (uint32_t i = 0; i < n; ++i) {
        const float* p = t + 9 * (size_t)i;
        v[i] = Triangle(vec3f1(p[0], p[1], p[2]), vec3f1(p[3], p[4], p[5]), vec3f1(p[6], p[7], p[8]));
    }
    return v;
}

extern "C" {

void ref_set_threads(int n) { omp_set_num_threads(n > 64 ? 64 : n); }

// setup_morton (src/builder.cpp:2204): codes and the scene box
void ref_setup_morton(const float* tris, uint32_t n, uint32_t* codes, uint32_t* index, float* scene)
{
    std::vector<Triangle> v = to_tris(tris, n);
    std::vector<RadixInput32> mc(n);
    AABB1 box;
    setup_morton(v, mc, box);
    for (uint32_t i = 0; i < n; ++i) { codes[i] = mc[i].code; index[i] = mc[i].index; }
    scene[0] = box.min.x; scene[1] = box.min.y; scene[2] = box.min.z;
    scene[3] = box.max.x; scene[4] = box.max.y; scene[5] = box.max.z;
}

// radix_sort<uint32_t, RadixInput32>(..., 8) as build_hierarchy_morton calls it
void ref_radix_sort(uint32_t* codes, uint32_t* index, uint32_t n)
{
    std::vector<RadixInput32> mc(n), scratch(n);
    for (uint32_t i = 0; i < n; ++i) { mc[i].code = codes[i]; mc[i].index = index[i]; }
    radix_sort<uint32_t, RadixInput32>(mc.begin(), mc.end(), scratch.begin(), scratch.end(), 8);
    for (uint32_t i = 0; i < n; ++i) { codes[i] = mc[i].code; index[i] = mc[i].index; }
}

// find_split_morton over codes[0..count)
uint32_t ref_find_split_morton(const uint32_t* codes, uint32_t count)
{
    std::vector<RadixInput32> mc(count);
    for (uint32_t i = 0; i < count; ++i) { mc[i].code = codes[i]; mc[i].index = i; }
    return find_split_morton(mc.begin(), mc.end());
}

// setup_morton2 (src/builder.cpp:2247-2279): 60-bit codes and the scene box
void ref_setup_morton2(const float* tris, uint32_t n, uint64_t* codes, uint32_t* index, float* scene)
{
    std::vector<Triangle> v = to_tris(tris, n);
    std::vector<RadixInput64> mc(n);
    AABB1 box;
    setup_morton2(v, mc, box);
    for (uint32_t i = 0; i < n; ++i) { codes[i] = mc[i].code; index[i] = mc[i].index; }
    scene[0] = box.min.x; scene[1] = box.min.y; scene[2] = box.min.z;
    scene[3] = box.max.x; scene[4] = box.max.y; scene[5] = box.max.z;
}

// radix_sort<uint64_t, RadixInput64>(..., 8) as build_hierarchy_morton2 calls it
void ref_radix_sort64(uint64_t* codes, uint32_t* index, uint32_t n)
{
    std::vector<RadixInput64> mc(n), scratch(n);
    for (uint32_t i = 0; i < n; ++i) { mc[i].code = codes[i]; mc[i].index = index[i]; }
    radix_sort<uint64_t, RadixInput64>(mc.begin(), mc.end(), scratch.begin(), scratch.end(), 8);
    for (uint32_t i = 0; i < n; ++i) { codes[i] = mc[i].code; index[i] = mc[i].index; }
}

// find_split_morton2 over codes[0..count)
uint32_t ref_find_split_morton2(const uint64_t* codes, uint32_t count)
{
    std::vector<RadixInput64> mc(count);
    for (uint32_t i = 0; i < count; ++i) { mc[i].code = codes[i]; mc[i].index = i; }
    return find_split_morton2(mc.begin(), mc.end());
}

// Builders.  kind: 0 recursive, 1 horizontal, 2 grid, 3 grid_sse,
// 4 grid_m128 ("grid_avx"), 5 morton, 6 morton2.  Copies min(cap, node_count)
// records.
int ref_build(int kind, const float* tris, uint32_t n, Node1* out, uint32_t cap,
              uint32_t* node_count, uint32_t* root)
{
    std::vector<Triangle> v = to_tris(tris, n);
    Hierarchy h;
    uint32_t count = 2 * n;
    switch (kind) {
    case 0: h = Builder::build_hierarchy(v); break;
    case 1: h = Builder::build_hierarchy_horizontal(v); break;
    case 2: h = Builder::build_hierarchy_grid(v); count += 128; break;
    case 3: h = Builder::build_hierarchy_grid_sse(v); count += 128; break;
    case 4: h = Builder::build_hierarchy_grid_m128(v); count += 128; break;
    case 5: h = Builder::build_hierarchy_morton(v); break;
    case 6: h = Builder::build_hierarchy_morton2(v); break;
    default: return 1;
    }
    uint32_t m = count < cap ? count : cap;
    memcpy(out, h.node_base, sizeof(Node1) * m);
    *node_count = count;
    *root = h.root_index;
    delete[] h.node_base;
    return 0;
}

// Time a build only (no copy): returns 0
int ref_build_only(int kind, const float* tris, uint32_t n)
{
    static std::vector<Triangle> v;
    v = to_tris(tris, n);
    Hierarchy h;
    switch (kind) {
    case 0: h = Builder::build_hierarchy(v); break;
    case 1: h = Builder::build_hierarchy_horizontal(v); break;
    case 2: h = Builder::build_hierarchy_grid(v); break;
    case 3: h = Builder::build_hierarchy_grid_sse(v); break;
    case 4: h = Builder::build_hierarchy_grid_m128(v); break;
    case 5: h = Builder::build_hierarchy_morton(v); break;
    default: return 1;
    }
    delete[] h.node_base;
    return 0;
}

// Wall time of one build, in milliseconds (steady clock around the builder
// call only; the triangle conversion and the node array's release are
// outside).  kind as ref_build.  Returns a negative value for an unknown
// kind.
double ref_time_build(int kind, const float* tris, uint32_t n)
{
    std::vector<Triangle> v = to_tris(tris, n);
    Hierarchy h;
    const auto t0 = std::chrono::steady_clock::now();
    switch (kind) {
    case 0: h = Builder::build_hierarchy(v); break;
    case 1: h = Builder::build_hierarchy_horizontal(v); break;
    case 2: h = Builder::build_hierarchy_grid(v); break;
    case 3: h = Builder::build_hierarchy_grid_sse(v); break;
    case 4: h = Builder::build_hierarchy_grid_m128(v); break;
    case 5: h = Builder::build_hierarchy_morton(v); break;
    case 6: h = Builder::build_hierarchy_morton2(v); break;
    default: return -1.0;
    }
    const auto t1 = std::chrono::steady_clock::now();
    delete[] h.node_base;
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

static Hierarchy make_h(Node1* nodes, uint32_t node_count, uint32_t root, std::vector<Triangle>& v)
{
    Hierarchy h;
    h.node_base = nodes;
    h.node_count = node_count;
    h.tri_base = v.data();
    h.plucker_tri_base = nullptr;
    h.tri_count = (unsigned)v.size();
    h.root_index = root;
    return h;
}

// trace (src/tracer.cpp:195) / trace_packet<K> / trace_bundle<K>.
// tracer: 0 basic, 1 packet<8>, 2 bundle<64>, 100 + K packet<K> (K = 1, 2,
// 4, 8), 200 + K bundle<K> (K = 16, 64).  img: w*h*3 bytes.
int ref_trace(int tracer, const Node1* nodes, uint32_t node_count, uint32_t root,
              const float* tris, uint32_t n, uint32_t w, uint32_t h, const float* origin,
              uint8_t* img)
{
    std::vector<Triangle> v = to_tris(tris, n);
    std::vector<Node1> nd(nodes, nodes + node_count);
    Hierarchy hh = make_h(nd.data(), node_count, root, v);
    vec3f1 o(origin[0], origin[1], origin[2]);
    uint8_t* r = nullptr;
    switch (tracer) {
    case 0: r = trace(hh, w, h, o); break;
    case 1: r = trace_packet<8>(hh, w, h, o); break;
    case 2: r = trace_bundle<64>(hh, w, h, o); break;
    case 101: r = trace_packet<1>(hh, w, h, o); break;
    case 102: r = trace_packet<2>(hh, w, h, o); break;
    case 104: r = trace_packet<4>(hh, w, h, o); break;
    case 108: r = trace_packet<8>(hh, w, h, o); break;
    case 216: r = trace_bundle<16>(hh, w, h, o); break;
    case 264: r = trace_bundle<64>(hh, w, h, o); break;
    default: return 1;
    }
    memcpy(img, r, (size_t)w * h * 3);
    delete[] r;
    return 0;
}

// Wall time of one trace() / trace_packet<K> / trace_bundle<K> call in
// milliseconds (steady clock around the tracer only).  tracer as ref_trace.
double ref_time_trace(int tracer, const Node1* nodes, uint32_t node_count, uint32_t root, const float* tris,
                      uint32_t n, uint32_t w, uint32_t h, const float* origin)
{
    std::vector<Triangle> v = to_tris(tris, n);
    std::vector<Node1> nd(nodes, nodes + node_count);
    Hierarchy hh = make_h(nd.data(), node_count, root, v);
    vec3f1 o(origin[0], origin[1], origin[2]);
    uint8_t* r = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    switch (tracer) {
    case 0: r = trace(hh, w, h, o); break;
    case 1: r = trace_packet<8>(hh, w, h, o); break;
    case 2: r = trace_bundle<64>(hh, w, h, o); break;
    default: return -1.0;
    }
    const auto t1 = std::chrono::steady_clock::now();
    delete[] r;
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

// traverse (src/tracer.cpp:47) for explicit rays {ox,oy,oz,tmin,dx,dy,dz,tmax}
int ref_traverse(const Node1* nodes, uint32_t node_count, uint32_t root, const float* tris,
                 uint32_t n, const float* rays, uint32_t nrays, uint32_t* hit, uint32_t* tests)
{
    std::vector<Triangle> v = to_tris(tris, n);
    std::vector<Node1> nd(nodes, nodes + node_count);
    Hierarchy hh = make_h(nd.data(), node_count, root, v);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)nrays; ++i) {
        const float* r = rays + 8 * (size_t)i;
        Ray<1> ray;
        ray.origin[0][0] = r[0]; ray.origin[1][0] = r[1]; ray.origin[2][0] = r[2];
        ray.tmin = simdf<1>::broadcast(r[3]);
        ray.direction[0][0] = r[4]; ray.direction[1][0] = r[5]; ray.direction[2][0] = r[6];
        ray.tmax = simdf<1>::broadcast(r[7]);
        HitAttributes<1> attr;
        traverse(hh, root, 1, ray, attr);
        hit[i] = attr.hit[0] ? 1u : 0u;
        tests[i] = (uint32_t)attr.num_tests[0];
    }
    return 0;
}

// loadOBJFromFile (src/main.cpp:108-179): returns the triangle count; copies
// up to cap triangles.
uint32_t ref_load_obj(const char* path, float* out, uint32_t cap)
{
    std::vector<Triangle> v = loadOBJFromFile(std::string(path));
    uint32_t m = (uint32_t)v.size() < cap ? (uint32_t)v.size() : cap;
    for (uint32_t i = 0; i < m; ++i) {
        float* p = out + 9 * (size_t)i;
        p[0] = v[i].v0.x; p[1] = v[i].v0.y; p[2] = v[i].v0.z;
        p[3] = v[i].v1.x; p[4] = v[i].v1.y; p[5] = v[i].v1.z;
        p[6] = v[i].v2.x; p[7] = v[i].v2.y; p[8] = v[i].v2.z;
    }
    return (uint32_t)v.size();
}

// get_heatmap_colour (src/tracer.cpp:25-45) of each x: rgb[3 * i + k]
void ref_heatmap_colour(const float* x, uint32_t n, float* rgb)
{
    for (uint32_t i = 0; i < n; ++i) {
        const vec3f1 c = get_heatmap_colour(x[i]);
        rgb[3 * (size_t)i] = c.x;
        rgb[3 * (size_t)i + 1] = c.y;
        rgb[3 * (size_t)i + 2] = c.z;
    }
}

// The reference's image output (src/main.cpp:335-336): flip on, 24-bit BMP
int ref_write_bmp(const char* path, uint32_t w, uint32_t h, const uint8_t* rgb)
{
    stbi_flip_vertically_on_write(1);
    return stbi_write_bmp(path, (int)w, (int)h, 3, rgb);
}

}  // extern "C"
