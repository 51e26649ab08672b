"""Generate the golden fixtures in this directory from the Sequoia reference
itself (oracle/_ref/libseqref_*.so, built by oracle/build_ref.sh from the
reference's own sources).  Run on x86-64 where the reference tree exists:

    make -C oracle ref && python tests/golden/make_golden.py

Each fixture is a compressed .npz holding the input triangles and what the
reference's own functions return for them:
  codes, code_index, scene      setup_morton          (src/builder.cpp:2204)
  sorted_codes, sorted_index    radix_sort            (src/algorithms.h:89)
  sah{8,16,32}_nodes / _root    Builder::build_hierarchy (src/builder.cpp:1576),
                                only where the reference's tree is valid
  grid_nodes / grid_root        Builder::build_hierarchy_grid (src/builder.cpp:2133)
  horizontal_*, grid_sse_*,     build_hierarchy_horizontal / _grid_sse / _grid_m128
  grid_avx_*                    (src/builder.cpp:1621, 1993, 2064), where valid
  cam, w, h, heat               trace() heatmap on the 8-bin SAH tree
                                (src/tracer.cpp:195)
  packet{1,2,4,8}_heat,         trace_packet<k> / trace_bundle<k> heatmaps of
  bundle{16,64}_heat            that tree and camera (src/tracer.cpp:232, 292)
  ref_hit, ref_tests            traverse() per ray     (src/tracer.cpp:47) for
                                the reference-camera rays (regenerated by the
                                oracle; trace()'s heatmap pins that generation)
  splits_*                      find_split_morton on sub-ranges
  codes64, sorted_codes64,      setup_morton2 / radix_sort<uint64_t> /
  sorted_index64, splits64      find_split_morton2 (src/builder.cpp:2247-2349)
                                on the same sub-ranges
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from sequoia_gb300 import scenes  # noqa: E402


def valid(nodes, root, n):
    try:
        return bool((O.leaf_reach(nodes, root, n) == 1).all())
    except ValueError:
        return False


def make(name, tris, w=160, h=120):
    n = len(tris)
    out = {"tris": tris}
    codes, index, box = O.ref_setup_morton(tris)
    out.update(codes=codes, code_index=index, scene=box)
    sc, si = O.ref_radix_sort(codes, index)
    out.update(sorted_codes=sc, sorted_index=si)
    rng = np.random.default_rng(11)
    starts, ends, splits = [], [], []
    for _ in range(256):
        a = int(rng.integers(0, max(1, n - 2)))
        b = int(rng.integers(a + 2, min(n, a + 4000) + 1))
        starts.append(a); ends.append(b); splits.append(O.ref_find_split_morton(sc[a:b]))
    out.update(splits_begin=np.array(starts, np.uint32), splits_end=np.array(ends, np.uint32),
               splits=np.array(splits, np.uint32))
    # the 60-bit path of build_hierarchy_morton2
    codes64, index64, _ = O.ref_setup_morton2(tris)
    sc64, si64 = O.ref_radix_sort64(codes64, index64)
    out.update(codes64=codes64, sorted_codes64=sc64, sorted_index64=si64,
               splits64=np.array([O.ref_find_split_morton2(sc64[a:b]) for a, b in zip(starts, ends)], np.uint32))
    for bins, variant in ((8, "b8"), (16, "b16"), (32, "b32")):
        nodes, root = O.ref_build("recursive", tris, variant)
        if valid(nodes, root, n):
            out["sah%d_nodes" % bins] = nodes
            out["sah%d_root" % bins] = np.uint32(root)
    gnodes, groot = O.ref_build("grid", tris, "b8")
    if valid(gnodes, groot, n):
        out["grid_nodes"] = gnodes
        out["grid_root"] = np.uint32(groot)
    # the builders the drop-in maps onto the ones above (horizontal -> SAH,
    # grid_sse / grid_avx -> grid with cell nodes bounded by their triangles)
    for key, kind in (("horizontal", "horizontal"), ("grid_sse", "grid_sse"), ("grid_avx", "grid_avx")):
        knodes, kroot = O.ref_build(kind, tris, "b8")
        if valid(knodes, kroot, n):
            out[key + "_nodes"] = knodes
            out[key + "_root"] = np.uint32(kroot)
    lo, hi = scenes.scene_box(tris)
    centre = (lo + hi) * np.float32(0.5)
    cam = np.array([centre[0], centre[1], np.float32(2) * lo[2] - centre[2]], np.float32)
    nodes, root = O.ref_build("recursive", tris, "b8")
    assert valid(nodes, root, n), name
    out.update(cam=cam, w=np.uint32(w), h=np.uint32(h))
    out["heat"] = O.ref_trace(nodes, root, tris, w, h, cam, 0)
    # trace_packet<k> / trace_bundle<k> heatmaps of the same tree and camera
    for k in (1, 2, 4, 8):
        out["packet%d_heat" % k] = O.ref_trace(nodes, root, tris, w, h, cam, 100 + k)
    for k in (16, 64):
        out["bundle%d_heat" % k] = O.ref_trace(nodes, root, tris, w, h, cam, 200 + k)
    rays = O.rays_reference_camera(w, h, cam)
    hit, tests = O.ref_traverse(nodes, root, tris, rays)
    out.update(ref_hit=hit, ref_tests=tests)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), sorted(k for k in out if k.endswith("_root")))


def main():
    if not O.ref_available("b8"):
        raise SystemExit("reference not built: run `make -C oracle ref` first")
    O.ref("b8").ref_set_threads(8)
    make("ico3", scenes.displaced_icosphere(3, seed=1))
    make("ico4", scenes.displaced_icosphere(4, seed=1))
    make("soup3k", scenes.gaussian_soup(3000, clusters=4, seed=7))
    # duplicate-heavy: many triangles share a centroid cell
    t = scenes.gaussian_soup(2000, clusters=2, seed=9)
    t[:600] = t[0]
    make("dups2k", t)


if __name__ == "__main__":
    main()
