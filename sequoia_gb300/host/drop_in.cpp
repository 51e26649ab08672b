// drop_in.cpp -- Builder::build_hierarchy*, trace() and loadOBJFromFile over
// the C ABI (see sequoia.hpp).
//
// A Hierarchy carries only host pointers, but the tree it describes already
// lives on the GPU when Builder made it.  A small registry maps node_base to
// that device tree so that trace() on a freshly built Hierarchy does not
// upload it again; an entry is trusted only while node_base, node_count,
// root_index, tri_base, tri_count and the root record still match what the
// build returned.  Any other Hierarchy (one the reference built, or one the
// caller changed) is uploaded with sq_bvh_import_node1.
#include "sequoia.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <mutex>

namespace sequoia {
namespace {

struct Entry {
    const Node1* node_base;
    unsigned node_count, root_index, tri_count;
    const Triangle* tri_base;
    Node1 root_record;
    sq_bvh* bvh;
};

constexpr size_t kMaxEntries = 8;

std::mutex g_mu;
sq_ctx* g_ctx = nullptr;
std::list<Entry> g_trees;  // most recent first
sq_build_params g_params = {SQ_BUILDER_MORTON, 8, 8, 8, SQ_MORTON_BOUNDS_PRIMITIVE, 0};
uint32_t g_host_threads = 0;

void check(sq_status s, const char* what)
{
    if (s == SQ_OK) return;
    const char* m = g_ctx ? sq_last_error(g_ctx) : "";
    throw Error(s, std::string(what) + ": " + (m && *m ? m : "error " + std::to_string((int)s)));
}

sq_ctx* ctx_locked()
{
    if (!g_ctx) {
        sq_options o;
        memset(&o, 0, sizeof(o));
        const char* dev = getenv("SEQUOIA_DEVICE");
        o.device = dev ? atoi(dev) : 0;
        sq_ctx* c = nullptr;
        const sq_status s = sq_create(&c, &o);
        if (s != SQ_OK) throw Error(s, "sequoia: no usable CUDA device (sq_create failed)");
        g_ctx = c;
    }
    return g_ctx;
}

bool matches(const Entry& e, const Hierarchy& h)
{
    return e.node_base == h.node_base && e.node_count == h.node_count && e.root_index == h.root_index &&
           e.tri_base == h.tri_base && e.tri_count == h.tri_count && h.root_index < h.node_count &&
           memcmp(&e.root_record, h.node_base + h.root_index, sizeof(Node1)) == 0;
}

void drop_locked(const Node1* node_base)
{
    for (auto it = g_trees.begin(); it != g_trees.end();) {
        if (it->node_base == node_base) {
            sq_bvh_free(it->bvh);
            it = g_trees.erase(it);
        } else {
            ++it;
        }
    }
}

void remember_locked(const Hierarchy& h, sq_bvh* bvh)
{
    drop_locked(h.node_base);
    Entry e;
    e.node_base = h.node_base;
    e.node_count = h.node_count;
    e.root_index = h.root_index;
    e.tri_count = h.tri_count;
    e.tri_base = h.tri_base;
    // an out-of-range root never matches (matches() checks it first)
    if (h.node_base && h.root_index < h.node_count) e.root_record = h.node_base[h.root_index];
    else memset(static_cast<void*>(&e.root_record), 0, sizeof(Node1));
    e.bvh = bvh;
    g_trees.push_front(e);
    while (g_trees.size() > kMaxEntries) {
        sq_bvh_free(g_trees.back().bvh);
        g_trees.pop_back();
    }
}

sq_bvh* lookup_locked(const Hierarchy& h)
{
    for (auto it = g_trees.begin(); it != g_trees.end(); ++it) {
        if (matches(*it, h)) {
            g_trees.splice(g_trees.begin(), g_trees, it);
            return g_trees.front().bvh;
        }
    }
    return nullptr;
}

Hierarchy build(std::vector<Triangle>& prims, uint32_t kind, uint32_t flags_set, uint32_t flags_clear)
{
    std::lock_guard<std::mutex> lock(g_mu);
    sq_ctx* c = ctx_locked();
    if (prims.size() > 0xFFFFFFFFull) throw Error(SQ_ERR_TOO_LARGE, "sequoia: more than 2^32-1 triangles");
    sq_build_params p = g_params;
    p.kind = kind;
    p.flags = (p.flags | flags_set) & ~flags_clear;
    const uint32_t n = (uint32_t)prims.size();
    sq_bvh* bvh = nullptr;
    check(sq_build(c, reinterpret_cast<const sq_triangle*>(prims.data()), n, &p, &bvh), "sq_build");
    sq_bvh_info info;
    sq_status s = sq_bvh_get_info(bvh, &info);
    Node1* nodes = nullptr;
    uint32_t count = 0, root = 0;
    if (s == SQ_OK) {
        nodes = new Node1[info.node_capacity ? info.node_capacity : 1];
        s = sq_bvh_export_node1(bvh, reinterpret_cast<sq_node1*>(nodes), info.node_capacity, &count, &root);
    }
    if (s != SQ_OK) {
        delete[] nodes;
        sq_bvh_free(bvh);
        check(s, "sq_bvh_export_node1");
    }
    Hierarchy h;
    h.node_base = nodes;
    h.node_count = count;
    h.tri_base = prims.data();
    h.plucker_tri_base = nullptr;
    h.tri_count = n;
    h.root_index = root;
    remember_locked(h, bvh);
    return h;
}

}  // namespace

Hierarchy Builder::build_hierarchy(std::vector<Triangle>& p) { return build(p, SQ_BUILDER_SAH, 0, 0); }
Hierarchy Builder::build_hierarchy_horizontal(std::vector<Triangle>& p) { return build(p, SQ_BUILDER_SAH, 0, 0); }
Hierarchy Builder::build_hierarchy_morton(std::vector<Triangle>& p) { return build(p, SQ_BUILDER_MORTON, 0, 0); }
Hierarchy Builder::build_hierarchy_grid(std::vector<Triangle>& p)
{
    return build(p, SQ_BUILDER_GRID, SQ_BUILD_GRID_SCENE_BOUNDS, 0);
}
Hierarchy Builder::build_hierarchy_grid_sse(std::vector<Triangle>& p)
{
    return build(p, SQ_BUILDER_GRID, 0, SQ_BUILD_GRID_SCENE_BOUNDS);
}
Hierarchy Builder::build_hierarchy_grid_m128(std::vector<Triangle>& p)
{
    return build(p, SQ_BUILDER_GRID, 0, SQ_BUILD_GRID_SCENE_BOUNDS);
}
Hierarchy Builder::build_hierarchy_morton2(std::vector<Triangle>& p)
{
    return build(p, SQ_BUILDER_MORTON, SQ_BUILD_MORTON64, 0);
}

namespace {

// The device tree of a Hierarchy: the one Builder made, else an upload.
sq_bvh* tree_locked(sq_ctx* c, Hierarchy& hierarchy)
{
    sq_bvh* bvh = lookup_locked(hierarchy);
    if (!bvh) {
        check(sq_bvh_import_node1(c, reinterpret_cast<const sq_node1*>(hierarchy.node_base), hierarchy.node_count,
                                  hierarchy.root_index, reinterpret_cast<const sq_triangle*>(hierarchy.tri_base),
                                  hierarchy.tri_count, &bvh),
              "sq_bvh_import_node1");
        remember_locked(hierarchy, bvh);
    }
    return bvh;
}

uint8_t* camera_trace(Hierarchy& hierarchy, uint32_t w, uint32_t h, vec3f1 origin, uint32_t mode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    sq_ctx* c = ctx_locked();
    sq_bvh* bvh = tree_locked(c, hierarchy);
    sq_ray_source rs;
    memset(&rs, 0, sizeof(rs));
    rs.kind = SQ_RAYS_REFERENCE_CAMERA;
    rs.width = w;
    rs.height = h;
    rs.origin[0] = origin.x;
    rs.origin[1] = origin.y;
    rs.origin[2] = origin.z;
    uint8_t* image = new uint8_t[3ull * w * h];
    const sq_status s = sq_trace(c, bvh, &rs, mode, nullptr, image);
    if (s != SQ_OK) {
        delete[] image;
        check(s, "sq_trace");
    }
    return image;
}

}  // namespace

uint8_t* trace(Hierarchy& hierarchy, uint32_t w, uint32_t h, vec3f1 origin)
{
    return camera_trace(hierarchy, w, h, origin, SQ_TRACE_REF);
}

void traverse(Hierarchy& hierarchy, uint32_t index, uint32_t count, const Ray<1>* rays,
              HitAttributes<1>* attributes, size_t n)
{
    if (n == 0) return;
    if (n > 0xFFFFFFFFull) throw Error(SQ_ERR_TOO_LARGE, "traverse: more than 2^32-1 rays");
    std::vector<sq_hit> hits(n);
    {
        std::lock_guard<std::mutex> lock(g_mu);
        sq_ctx* c = ctx_locked();
        sq_bvh* bvh = tree_locked(c, hierarchy);
        check(sq_traverse(c, bvh, index, count, reinterpret_cast<const sq_ray*>(rays), (uint32_t)n, hits.data()),
              "sq_traverse");
    }
    for (size_t i = 0; i < n; ++i) {
        if (hits[i].id != SQ_NO_HIT) attributes[i].hit = -1;
        attributes[i].num_tests += (int32_t)hits[i].tests;
    }
}

void traverse(Hierarchy& hierarchy, uint32_t index, uint32_t count, Ray<1>& ray, HitAttributes<1>& attributes)
{
    traverse(hierarchy, index, count, &ray, &attributes, 1);
}

uint8_t* trace_coherent(Hierarchy& hierarchy, uint32_t w, uint32_t h, vec3f1 origin, bool bundle, uint32_t k)
{
    return camera_trace(hierarchy, w, h, origin, (bundle ? SQ_TRACE_BUNDLE : SQ_TRACE_PACKET) | SQ_TRACE_WIDTH(k));
}

std::vector<Triangle> loadOBJFromFile(std::string filename)
{
    FILE* fp = fopen(filename.c_str(), "r");
    if (!fp) {
        fprintf(stderr, "Can't open OBJ file %s!\n", filename.c_str());
        exit(1);
    }
    fclose(fp);
    sq_triangle* tris = nullptr;
    uint32_t n = 0;
    sq_obj_info info;
    const sq_status s = sq_obj_load(filename.c_str(), g_host_threads, &tris, &n, &info);
    if (s != SQ_OK) throw Error(s, std::string("loadOBJFromFile: ") + sq_host_last_error());
    printf("Geometry\n");
    printf("  faces:        %d\n", (int)info.faces);
    printf("  verts:        %d\n", (int)info.vertices);
    std::vector<Triangle> out(n);
    if (n) memcpy(static_cast<void*>(out.data()), tris, sizeof(Triangle) * (size_t)n);
    sq_obj_free(tris);
    return out;
}

void set_build_params(const sq_build_params& params)
{
    std::lock_guard<std::mutex> lock(g_mu);
    g_params = params;
}

sq_build_params build_params()
{
    std::lock_guard<std::mutex> lock(g_mu);
    return g_params;
}

void set_host_threads(uint32_t threads) { g_host_threads = threads; }

sq_ctx* context()
{
    std::lock_guard<std::mutex> lock(g_mu);
    return ctx_locked();
}

sq_bvh* device_tree(const Hierarchy& hierarchy)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return lookup_locked(hierarchy);
}

void release(Hierarchy& hierarchy)
{
    {
        std::lock_guard<std::mutex> lock(g_mu);
        drop_locked(hierarchy.node_base);
    }
    delete[] hierarchy.node_base;
    hierarchy.node_base = nullptr;
    hierarchy.node_count = 0;
}

void last_timings(float stage_ms[8])
{
    std::lock_guard<std::mutex> lock(g_mu);
    check(sq_last_timings(ctx_locked(), stage_ms), "sq_last_timings");
}

}  // namespace sequoia
