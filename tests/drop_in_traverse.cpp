// Test program for the C++ drop-in's traverse() (compiled and run by
// tests/test_gpu_trace.py against libsequoia_gpu.so).
//
//   drop_in_traverse <tris.bin> <rays.bin> <out.bin>
//
// tris.bin: float32 triangles (9 floats each); rays.bin: float32 rays
// {origin, tmin, direction, tmax}.  Builds the SAH tree with
// Builder::build_hierarchy, traverses the first 64 rays one call per ray
// (attributes accumulated twice, to check that traverse adds to them) and
// all rays with the many-ray overload from (root_index, 1), and writes
// int32 {hit, num_tests} per ray for the single calls' first pass, then for
// the overload, then the accumulated second pass of the first 64.
#include <cstdio>
#include <vector>

#include "sequoia.hpp"

using namespace sequoia;

template <class T>
static std::vector<T> read_all(const char* path)
{
    std::vector<T> v;
    FILE* f = fopen(path, "rb");
    if (!f) return v;
    fseek(f, 0, SEEK_END);
    const long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    v.resize((size_t)bytes / sizeof(T));
    if (fread(v.data(), sizeof(T), v.size(), f) != v.size()) v.clear();
    fclose(f);
    return v;
}

int main(int argc, char** argv)
{
    if (argc != 4) return 2;
    std::vector<Triangle> tris = read_all<Triangle>(argv[1]);
    std::vector<Ray<1>> rays = read_all<Ray<1>>(argv[2]);
    if (tris.empty() || rays.empty()) return 3;
    Hierarchy h = Builder::build_hierarchy(tris);
    const size_t few = rays.size() < 64 ? rays.size() : 64;
    std::vector<HitAttributes<1>> one(few), twice(few), many(rays.size());
    for (size_t i = 0; i < few; ++i) {
        traverse(h, h.root_index, 1, rays[i], one[i]);
        traverse(h, h.root_index, 1, rays[i], twice[i]);
        traverse(h, h.root_index, 1, rays[i], twice[i]);
    }
    traverse(h, h.root_index, 1, rays.data(), many.data(), rays.size());
    FILE* f = fopen(argv[3], "wb");
    if (!f) return 4;
    fwrite(one.data(), sizeof(HitAttributes<1>), one.size(), f);
    fwrite(many.data(), sizeof(HitAttributes<1>), many.size(), f);
    fwrite(twice.data(), sizeof(HitAttributes<1>), twice.size(), f);
    fclose(f);
    release(h);
    return 0;
}
