// sequoia_main.cpp -- the `sequoia` command line tool on the GPU library.
//
// Same usage as the reference's tool (src/main.cpp:416-540):
//   sequoia <scene.obj> [-builder <type>] [-tracer basic | packet <n> | bundle <n>]
//                       [-threads <n>] [-res <x> <y>] [-benchmark]
// run: load the OBJ, put the camera at (cx, cy, 2*min.z - cz) of the scene
// box (src/main.cpp:312-318), build, trace, write render.bmp.  -benchmark:
// every builder and tracer at 1920x1080, benchmark{1,2,3}.bmp.
// Options of this build only:
//   -bins <n> -leaf <n>   SAH/grid bins (8, 16, 32) and leaf size
//   -wide                 also build the 8-wide quantised BVH (closest/anyhit)
//   -mode ref|closest|anyhit
//                         ref (default) is the reference's traversal; closest
//                         and anyhit are the front-to-back traversals, whose
//                         heatmap counts their own (fewer) box tests
//   -o <file>             output image instead of render.bmp
//   -device <n>           CUDA device
// Times are wall-clock milliseconds around each call (the build includes the
// device-to-host copy of the node array that Builder returns); the device
// time of each stage is printed beside them.
#include "sequoia.hpp"

#include <chrono>
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

using namespace sequoia;

namespace {

enum class BuilderType { recursive, horizontal, grid, grid_sse, grid_avx, morton };
enum class TracerType { basic, packet, bundle };

struct Arguments {
    std::string filename;
    BuilderType builder = BuilderType::recursive;
    TracerType tracer = TracerType::basic;
    uint32_t packet_width = 8, bundle_width = 64;
    uint32_t w = 1920, h = 1080;
    uint32_t threads = 0;
    bool benchmark = false;
    uint32_t bins = 8, leaf = 8;
    bool wide = false;
    uint32_t mode = SQ_TRACE_REF;
    std::string out = "render.bmp";
};

const char* kBuilderNames[] = {"recursive", "horizontal", "grid", "grid_sse", "grid_avx", "morton"};

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

void usage()
{
    printf("Usage:\n");
    printf("    sequoia <scene.obj> [<args>]\n");
    printf("        args:\n");
    printf("            -builder <type> : recursive | horizontal | grid | grid_sse | grid_avx | morton\n");
    printf("                recursive, horizontal : binned SAH (GPU breadth-first)\n");
    printf("                grid, grid_sse, grid_avx : 4x4x4 grid of per-cell SAH builds\n");
    printf("                morton         : 30-bit Morton codes, radix sort, LBVH\n");
    printf("            -tracer  <type> : basic | packet <n> (1, 2, 4, 8) | bundle <n> (16, 64)\n");
    printf("            -threads <n>    : threads of the OBJ parse\n");
    printf("            -res <x> <y>    : output resolution\n");
    printf("            -benchmark      : time every builder and tracer\n");
    printf("            -bins <n> -leaf <n> -wide -mode ref|closest|anyhit -o <file> -device <n>\n");
}

[[noreturn]] void bad(const char* msg)
{
    printf("Error: %s\n", msg);
    usage();
    exit(2);
}

const char* need(int& i, int argc, char** argv)
{
    if (++i >= argc) bad("missing value");
    return argv[i];
}

Arguments parse_arguments(int argc, char** argv)
{
    Arguments a;
    if (argc < 2) {
        printf("Error: not enough arguments\n");
        usage();
        exit(0);
    }
    a.filename = argv[1];
    for (int i = 2; i < argc; ++i) {
        const std::string k = argv[i];
        if (k == "-builder") {
            const std::string v = need(i, argc, argv);
            bool found = false;
            for (int b = 0; b < 6; ++b) {
                if (v == kBuilderNames[b]) {
                    a.builder = (BuilderType)b;
                    found = true;
                }
            }
            if (!found) {
                printf("Error: invalid builder type\n");
                exit(0);
            }
        } else if (k == "-tracer") {
            const std::string v = need(i, argc, argv);
            if (v == "basic") {
                a.tracer = TracerType::basic;
            } else if (v == "packet") {
                a.tracer = TracerType::packet;
                a.packet_width = (uint32_t)atoi(need(i, argc, argv));
                if (a.packet_width != 1 && a.packet_width != 2 && a.packet_width != 4 && a.packet_width != 8)
                    bad("packet width must be 1, 2, 4 or 8");
            } else if (v == "bundle") {
                a.tracer = TracerType::bundle;
                a.bundle_width = (uint32_t)atoi(need(i, argc, argv));
                if (a.bundle_width != 16 && a.bundle_width != 64) bad("bundle width must be 16 or 64");
            } else {
                printf("Error: invalid tracer type\n");
                exit(0);
            }
        } else if (k == "-threads") {
            a.threads = (uint32_t)atoi(need(i, argc, argv));
        } else if (k == "-res") {
            a.w = (uint32_t)atoi(need(i, argc, argv));
            a.h = (uint32_t)atoi(need(i, argc, argv));
        } else if (k == "-benchmark") {
            a.benchmark = true;
        } else if (k == "-bins") {
            a.bins = (uint32_t)atoi(need(i, argc, argv));
        } else if (k == "-leaf") {
            a.leaf = (uint32_t)atoi(need(i, argc, argv));
        } else if (k == "-wide") {
            a.wide = true;
        } else if (k == "-mode") {
            const std::string v = need(i, argc, argv);
            if (v == "ref") a.mode = SQ_TRACE_REF;
            else if (v == "closest") a.mode = SQ_TRACE_CLOSEST;
            else if (v == "anyhit") a.mode = SQ_TRACE_ANYHIT;
            else bad("mode must be ref, closest or anyhit");
        } else if (k == "-o") {
            a.out = need(i, argc, argv);
        } else if (k == "-device") {
            setenv("SEQUOIA_DEVICE", need(i, argc, argv), 1);
        }
        // unknown arguments are skipped, as the reference's parser does
    }
    if (a.w == 0 || a.h == 0) bad("resolution must be positive");
    return a;
}

Hierarchy run_builder(BuilderType b, std::vector<Triangle>& prims)
{
    switch (b) {
    case BuilderType::recursive: return Builder::build_hierarchy(prims);
    case BuilderType::horizontal: return Builder::build_hierarchy_horizontal(prims);
    case BuilderType::grid: return Builder::build_hierarchy_grid(prims);
    case BuilderType::grid_sse: return Builder::build_hierarchy_grid_sse(prims);
    case BuilderType::grid_avx: return Builder::build_hierarchy_grid_m128(prims);
    case BuilderType::morton: return Builder::build_hierarchy_morton(prims);
    }
    return Builder::build_hierarchy(prims);
}

// The scene box and camera of src/main.cpp:305-318: min/max over every
// vertex, centre = (min + max) * 0.5, camera = (cx, cy, 2*min.z - cz).
vec3f1 reference_camera(const std::vector<Triangle>& prims)
{
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (const Triangle& t : prims) {
        const vec3f1* v[3] = {&t.v0, &t.v1, &t.v2};
        for (int k = 0; k < 3; ++k) {
            const float c[3] = {v[k]->x, v[k]->y, v[k]->z};
            for (int a = 0; a < 3; ++a) {
                lo[a] = c[a] < lo[a] ? c[a] : lo[a];
                hi[a] = hi[a] < c[a] ? c[a] : hi[a];
            }
        }
    }
    const float cx = (lo[0] + hi[0]) * 0.5f, cy = (lo[1] + hi[1]) * 0.5f, cz = (lo[2] + hi[2]) * 0.5f;
    return vec3f1(cx, cy, 2.0f * lo[2] - cz);
}

uint8_t* run_tracer(const Arguments& a, Hierarchy& h, vec3f1 camera)
{
    if (a.mode == SQ_TRACE_REF) {
        // src/main.cpp:279-300
        switch (a.tracer) {
        case TracerType::basic: return trace(h, a.w, a.h, camera);
        case TracerType::packet:
            switch (a.packet_width) {
            case 1: return trace_packet<1>(h, a.w, a.h, camera);
            case 2: return trace_packet<2>(h, a.w, a.h, camera);
            case 4: return trace_packet<4>(h, a.w, a.h, camera);
            case 8: return trace_packet<8>(h, a.w, a.h, camera);
            default: throw Error(SQ_ERR_INVALID, "invalid packet width (1, 2, 4 or 8)");
            }
        case TracerType::bundle:
            if (a.bundle_width == 16) return trace_bundle<16>(h, a.w, a.h, camera);
            return trace_bundle<64>(h, a.w, a.h, camera);
        }
    }
    sq_bvh* bvh = device_tree(h);
    if (!bvh) throw Error(SQ_ERR_INVALID, "no device tree for this hierarchy");
    sq_ray_source rs;
    memset(&rs, 0, sizeof(rs));
    rs.kind = SQ_RAYS_REFERENCE_CAMERA;
    rs.width = a.w;
    rs.height = a.h;
    rs.origin[0] = camera.x;
    rs.origin[1] = camera.y;
    rs.origin[2] = camera.z;
    uint8_t* img = new uint8_t[3ull * a.w * a.h];
    const sq_status s = sq_trace(context(), bvh, &rs, a.mode, nullptr, img);
    if (s != SQ_OK) {
        delete[] img;
        throw Error(s, std::string("sq_trace: ") + sq_last_error(context()));
    }
    return img;
}

void write_image(const char* path, uint32_t w, uint32_t h, const uint8_t* img)
{
    if (sq_bmp_write(path, w, h, img) != SQ_OK) fprintf(stderr, "Error: %s\n", sq_host_last_error());
}

void configure(const Arguments& a)
{
    sq_build_params p = build_params();
    p.sah_bins = a.bins;
    p.leaf_size = a.leaf;
    p.flags = a.wide ? SQ_BUILD_WIDE8 : 0u;
    set_build_params(p);
    set_host_threads(a.threads);
}

void run(const Arguments& a)
{
    double t = now_ms();
    std::vector<Triangle> prims = loadOBJFromFile(a.filename);
    printf("Load time:     %.0fms\n", now_ms() - t);
    const vec3f1 camera = reference_camera(prims);

    t = now_ms();
    Hierarchy h = run_builder(a.builder, prims);
    const double build = now_ms() - t;
    float st[8];
    last_timings(st);
    printf("Build time:    %.2fms (device %.3fms)\n", build, st[0]);

    t = now_ms();
    uint8_t* image = run_tracer(a, h, camera);
    const double tr = now_ms() - t;
    last_timings(st);
    printf("Traverse time: %.2fms (device %.3fms, %.1f Mrays/s)\n", tr, st[4],
           st[4] > 0 ? (double)a.w * a.h / (st[4] * 1e3) : 0.0);

    write_image(a.out.c_str(), a.w, a.h, image);
    delete[] image;
    release(h);
}

void benchmark(const Arguments& a)
{
    double t0 = now_ms();
    std::vector<Triangle> prims = loadOBJFromFile(a.filename);
    const double load = now_ms() - t0;
    const vec3f1 camera = reference_camera(prims);

    double wall[6], dev[6];
    Hierarchy sah{};
    for (int b = 0; b < 6; ++b) {
        const double t = now_ms();
        Hierarchy h = run_builder((BuilderType)b, prims);
        wall[b] = now_ms() - t;
        float st[8];
        last_timings(st);
        dev[b] = st[0];
        if (b == 0) sah = h;
        else release(h);
    }
    const uint32_t w = 1920, hh = 1080;
    Arguments ta = a;
    ta.w = w;
    ta.h = hh;
    double twall[3], tdev[3];
    uint8_t* img[3];
    // basic, packet<8>, bundle<64> (src/main.cpp:368-373)
    const TracerType kinds[3] = {TracerType::basic, TracerType::packet, TracerType::bundle};
    ta.packet_width = 8;
    ta.bundle_width = 64;
    for (int k = 0; k < 3; ++k) {
        ta.tracer = kinds[k];
        const double t = now_ms();
        img[k] = run_tracer(ta, sah, camera);
        twall[k] = now_ms() - t;
        float st[8];
        last_timings(st);
        tdev[k] = st[4];
    }
    const double n = (double)prims.size();
    printf("Load time: %.2fs\n\n", load / 1e3);
    printf("             recursive horizontal       grid   grid_sse   grid_avx     morton\n");
    printf("build time: ");
    for (int b = 0; b < 6; ++b) printf(" % 8.2fms", wall[b]);
    printf("\ndevice    : ");
    for (int b = 0; b < 6; ++b) printf(" % 8.3fms", dev[b]);
    printf("\ntri/s     : ");
    for (int b = 0; b < 6; ++b) printf(" % 9.0fm", n / (1e3 * wall[b]));
    printf("\n\n             basic packet bundle\n");
    printf("trace time: % 6.2fms % 6.2fms % 6.2fms\n", twall[0], twall[1], twall[2]);
    printf("mrps      : % 6.1f % 6.1f % 6.1f\n", w * hh / (1e3 * twall[0]), w * hh / (1e3 * twall[1]),
           w * hh / (1e3 * twall[2]));
    printf("device    : % 6.3fms % 6.3fms % 6.3fms\n", tdev[0], tdev[1], tdev[2]);
    const char* names[3] = {"benchmark1.bmp", "benchmark2.bmp", "benchmark3.bmp"};
    for (int k = 0; k < 3; ++k) {
        write_image(names[k], w, hh, img[k]);
        delete[] img[k];
    }
    release(sah);
}

}  // namespace

int main(int argc, char** argv)
{
    const Arguments a = parse_arguments(argc, argv);
    try {
        configure(a);
        if (a.benchmark) benchmark(a);
        else run(a);
    } catch (const Error& e) {
        fprintf(stderr, "sequoia: %s\n", e.what());
        return 1;
    }
    return 0;
}
