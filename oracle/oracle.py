"""ctypes bindings for the CPU oracle (liboracle.so) and, where it was built,
the reference's own code (_ref/libseqref_*.so).

TEST INFRASTRUCTURE ONLY: imported by tests, the smoke check and the
benchmark's CPU-baseline leg, never by the library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NO_HIT = 0xFFFFFFFF
NODE1 = np.dtype([("min", "<f4", 3), ("count", "<u2"), ("flags", "<u2"),
                  ("max", "<f4", 3), ("child", "<u4")])
assert NODE1.itemsize == 32

_lib = None


def build():
    """Compile liboracle.so (and nothing else)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _declare(L):
    vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int, C.c_float
    sig = {
        "sqo_set_threads": (None, [i32]),
        "sqo_get_threads": (i32, []),
        "sqo_tri_aabbs": (None, [vp, u32, vp, vp]),
        "sqo_morton_codes": (None, [vp, u32, i32, vp, vp]),
        "sqo_bit_interleave_32": (u32, [u32, u32, u32]),
        "sqo_sort_pairs": (None, [vp, vp, u32, u32, u32]),
        "sqo_find_split_morton": (u32, [vp, u32]),
        "sqo_bit_interleave_64": (C.c_uint64, [C.c_uint64, C.c_uint64, C.c_uint64]),
        "sqo_morton_codes64": (None, [vp, u32, i32, vp, vp]),
        "sqo_sort_pairs64": (None, [vp, vp, u32]),
        "sqo_find_split_morton64": (u32, [vp, u32]),
        "sqo_build_morton64": (u32, [vp, u32, i32, vp, vp, vp]),
        "sqo_node_capacity": (u32, [u32, i32]),
        "sqo_build_morton": (u32, [vp, u32, i32, vp, vp, vp]),
        "sqo_build_sah": (u32, [vp, u32, u32, u32, vp, vp]),
        "sqo_build_grid": (u32, [vp, u32, u32, u32, i32, vp, vp]),
        "sqo_rays_reference_camera": (None, [u32, u32, vp, vp]),
        "sqo_pinhole_basis": (None, [vp, vp, vp, f32, u32, u32, vp]),
        "sqo_rays_pinhole": (None, [u32, u32, vp, vp]),
        "sqo_trace": (i32, [vp, u32, vp, vp, u32, i32, vp, vp, vp]),
        "sqo_brute_closest": (None, [vp, u32, vp, u32, vp, vp]),
        "sqo_heatmap": (None, [vp, u32, vp]),
        "sqo_heatmap_colour": (None, [f32, vp]),
        "sqo_heatmap_ramp": (None, [vp, u32, vp]),
        "sqo_trace_coherent": (i32, [vp, u32, u32, u32, vp, i32, u32, vp]),
        "sqo_reintersect_f64": (None, [vp, vp, u32, vp, vp]),
        "sqo_canonical_bfs": (u32, [vp, u32, u32, vp, u32]),
        "sqo_leaf_reach": (u32, [vp, u32, u32, u32, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def _tris(t):
    t = np.ascontiguousarray(t, dtype=np.float32)
    assert t.ndim == 2 and t.shape[1] == 9
    return t


def set_threads(n):
    lib().sqo_set_threads(int(n))


def threads():
    return int(lib().sqo_get_threads())


def morton_codes(tris, bounds_mode=0):
    tris = _tris(tris)
    codes = np.empty(len(tris), np.uint32)
    box = np.empty(6, np.float32)
    lib().sqo_morton_codes(_p(tris), len(tris), bounds_mode, _p(codes), _p(box))
    return codes, box


def bit_interleave_32(x, y, z):
    return int(lib().sqo_bit_interleave_32(x, y, z))


def sort_pairs(keys, values, key_bits=32, digit_bits=8):
    k = np.array(keys, np.uint32, copy=True)
    v = np.array(values, np.uint32, copy=True)
    lib().sqo_sort_pairs(_p(k), _p(v), len(k), key_bits, digit_bits)
    return k, v


def find_split_morton(codes):
    codes = np.ascontiguousarray(codes, np.uint32)
    return int(lib().sqo_find_split_morton(_p(codes), len(codes)))


def morton_codes64(tris, bounds_mode=0):
    tris = _tris(tris)
    codes = np.empty(len(tris), np.uint64)
    box = np.empty(6, np.float32)
    lib().sqo_morton_codes64(_p(tris), len(tris), bounds_mode, _p(codes), _p(box))
    return codes, box


def sort_pairs64(keys, values):
    k = np.array(keys, np.uint64, copy=True)
    v = np.array(values, np.uint32, copy=True)
    lib().sqo_sort_pairs64(_p(k), _p(v), len(k))
    return k, v


def find_split_morton64(codes):
    codes = np.ascontiguousarray(codes, np.uint64)
    return int(lib().sqo_find_split_morton64(_p(codes), len(codes)))


def build_morton64(tris, bounds_mode=0):
    tris = _tris(tris)
    n = len(tris)
    nodes = np.zeros(node_capacity(n, 0), NODE1)
    codes = np.empty(n, np.uint64)
    perm = np.empty(n, np.uint32)
    root = lib().sqo_build_morton64(_p(tris), n, bounds_mode, _p(nodes), _p(codes), _p(perm))
    return nodes, int(root), codes, perm


def node_capacity(n, kind):
    return int(lib().sqo_node_capacity(n, kind))


def build_morton(tris, bounds_mode=0):
    tris = _tris(tris)
    n = len(tris)
    nodes = np.zeros(node_capacity(n, 0), NODE1)
    codes = np.empty(n, np.uint32)
    perm = np.empty(n, np.uint32)
    root = lib().sqo_build_morton(_p(tris), n, bounds_mode, _p(nodes), _p(codes), _p(perm))
    return nodes, int(root), codes, perm


def build_sah(tris, bins=8, leaf=8):
    tris = _tris(tris)
    n = len(tris)
    nodes = np.zeros(node_capacity(n, 1), NODE1)
    perm = np.empty(n, np.uint32)
    root = lib().sqo_build_sah(_p(tris), n, bins, leaf, _p(nodes), _p(perm))
    if root == NO_HIT:
        raise ValueError("SAH leaf exceeds 65535 triangles")
    return nodes, int(root), perm


def build_grid(tris, bins=8, leaf=8, scene_bounds_cells=False):
    tris = _tris(tris)
    n = len(tris)
    nodes = np.zeros(node_capacity(n, 2), NODE1)
    perm = np.empty(n, np.uint32)
    root = lib().sqo_build_grid(_p(tris), n, bins, leaf, int(scene_bounds_cells), _p(nodes), _p(perm))
    if root == NO_HIT:
        raise ValueError("SAH leaf exceeds 65535 triangles")
    return nodes, int(root), perm


def rays_reference_camera(w, h, origin):
    o = np.asarray(origin, np.float32)
    rays = np.empty((w * h, 8), np.float32)
    lib().sqo_rays_reference_camera(w, h, _p(o), _p(rays))
    return rays


def pinhole_basis(eye, target, up, vfov, w, h):
    b = np.empty(14, np.float32)
    e, t, u = (np.asarray(x, np.float32) for x in (eye, target, up))
    lib().sqo_pinhole_basis(_p(e), _p(t), _p(u), float(vfov), w, h, _p(b))
    return b


def rays_pinhole(w, h, eye, target, up, vfov):
    b = pinhole_basis(eye, target, up, vfov, w, h)
    rays = np.empty((w * h, 8), np.float32)
    lib().sqo_rays_pinhole(w, h, _p(b), _p(rays))
    return rays


def trace(nodes, root, tris, rays, mode):
    tris = _tris(tris)
    rays = np.ascontiguousarray(rays, np.float32)
    n = len(rays)
    ids = np.empty(n, np.uint32)
    ts = np.empty(n, np.float32)
    tests = np.empty(n, np.uint32)
    err = lib().sqo_trace(_p(nodes), root, _p(tris), _p(rays), n, mode, _p(ids), _p(ts), _p(tests))
    if err:
        raise RuntimeError("oracle traversal stack limit reached")
    return ids, ts, tests


def brute_closest(tris, rays):
    tris = _tris(tris)
    rays = np.ascontiguousarray(rays, np.float32)
    ids = np.empty(len(rays), np.uint32)
    ts = np.empty(len(rays), np.float32)
    lib().sqo_brute_closest(_p(tris), len(tris), _p(rays), len(rays), _p(ids), _p(ts))
    return ids, ts


def heatmap(tests):
    tests = np.ascontiguousarray(tests, np.uint32)
    rgb = np.empty(len(tests) * 3, np.uint8)
    lib().sqo_heatmap(_p(tests), len(tests), _p(rgb))
    return rgb


def heatmap_colour(xs):
    """get_heatmap_colour (src/tracer.cpp:25-45) of each x: float32 (n, 3)."""
    xs = np.ascontiguousarray(xs, np.float32).ravel()
    out = np.empty((len(xs), 3), np.float32)
    for i, x in enumerate(xs):
        lib().sqo_heatmap_colour(float(x), _p(out[i]))
    return out


def heatmap_ramp(values):
    """Colour-ramp heatmap bytes (n * 3) of box-test values (counts)."""
    v = np.ascontiguousarray(values, np.float32)
    rgb = np.empty(len(v) * 3, np.uint8)
    lib().sqo_heatmap_ramp(_p(v), len(v), _p(rgb))
    return rgb


def trace_coherent(nodes, root, w, h, origin, bundle, k):
    """trace_packet<k> / trace_bundle<k> heatmap bytes (w*h*3)."""
    o = np.asarray(origin, np.float32)
    rgb = np.zeros(w * h * 3, np.uint8)
    rc = lib().sqo_trace_coherent(_p(np.ascontiguousarray(nodes)), root, w, h, _p(o), int(bundle), k, _p(rgb))
    if rc != 0:
        raise ValueError("sqo_trace_coherent failed (%d)" % rc)
    return rgb


def reintersect_f64(tris, rays, ids):
    tris = _tris(tris)
    rays = np.ascontiguousarray(rays, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    out = np.empty(len(rays), np.float64)
    lib().sqo_reintersect_f64(_p(tris), _p(rays), len(rays), _p(ids), _p(out))
    return out


def canonical_bfs(nodes, root):
    out = np.zeros(len(nodes), NODE1)
    m = lib().sqo_canonical_bfs(_p(nodes), len(nodes), root, _p(out), len(out))
    if m == NO_HIT:
        raise ValueError("malformed tree")
    return out[:m]


def leaf_reach(nodes, root, n):
    counts = np.zeros(n, np.uint32)
    m = lib().sqo_leaf_reach(_p(nodes), len(nodes), root, n, _p(counts))
    if m == NO_HIT:
        raise ValueError("malformed tree")
    return counts


# ---------------------------------------------------------------- reference

REF_BUILDERS = {"recursive": 0, "horizontal": 1, "grid": 2, "grid_sse": 3, "grid_avx": 4, "morton": 5,
                "morton2": 6}
_refs = {}


def ref_available(variant="b8"):
    return os.path.exists(os.path.join(HERE, "_ref", "libseqref_%s.so" % variant))


def ref(variant="b8"):
    if variant not in _refs:
        L = C.CDLL(os.path.join(HERE, "_ref", "libseqref_%s.so" % variant))
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        L.ref_set_threads.argtypes = [i32]
        L.ref_setup_morton.argtypes = [vp, u32, vp, vp, vp]
        L.ref_radix_sort.argtypes = [vp, vp, u32]
        L.ref_find_split_morton.argtypes = [vp, u32]
        L.ref_find_split_morton.restype = u32
        L.ref_build.argtypes = [i32, vp, u32, vp, u32, vp, vp]
        L.ref_build.restype = i32
        L.ref_build_only.argtypes = [i32, vp, u32]
        L.ref_trace.argtypes = [i32, vp, u32, u32, vp, u32, u32, u32, vp, vp]
        L.ref_traverse.argtypes = [vp, u32, u32, vp, u32, vp, u32, vp, vp]
        L.ref_load_obj.argtypes = [C.c_char_p, vp, u32]
        L.ref_load_obj.restype = u32
        L.ref_write_bmp.argtypes = [C.c_char_p, u32, u32, vp]
        L.ref_write_bmp.restype = i32
        L.ref_setup_morton2.argtypes = [vp, u32, vp, vp, vp]
        L.ref_radix_sort64.argtypes = [vp, vp, u32]
        L.ref_find_split_morton2.argtypes = [vp, u32]
        L.ref_find_split_morton2.restype = u32
        L.ref_heatmap_colour.argtypes = [vp, u32, vp]
        _refs[variant] = L
    return _refs[variant]


def ref_setup_morton(tris, variant="b8"):
    tris = _tris(tris)
    n = len(tris)
    codes = np.empty(n, np.uint32)
    index = np.empty(n, np.uint32)
    box = np.empty(6, np.float32)
    ref(variant).ref_setup_morton(_p(tris), n, _p(codes), _p(index), _p(box))
    return codes, index, box


def ref_setup_morton2(tris, variant="b8"):
    tris = _tris(tris)
    n = len(tris)
    codes = np.empty(n, np.uint64)
    index = np.empty(n, np.uint32)
    box = np.empty(6, np.float32)
    ref(variant).ref_setup_morton2(_p(tris), n, _p(codes), _p(index), _p(box))
    return codes, index, box


def ref_radix_sort64(codes, index, variant="b8"):
    c = np.array(codes, np.uint64, copy=True)
    i = np.array(index, np.uint32, copy=True)
    ref(variant).ref_radix_sort64(_p(c), _p(i), len(c))
    return c, i


def ref_find_split_morton2(codes, variant="b8"):
    codes = np.ascontiguousarray(codes, np.uint64)
    return int(ref(variant).ref_find_split_morton2(_p(codes), len(codes)))


def ref_radix_sort(codes, index, variant="b8"):
    c = np.array(codes, np.uint32, copy=True)
    i = np.array(index, np.uint32, copy=True)
    ref(variant).ref_radix_sort(_p(c), _p(i), len(c))
    return c, i


def ref_find_split_morton(codes, variant="b8"):
    codes = np.ascontiguousarray(codes, np.uint32)
    return int(ref(variant).ref_find_split_morton(_p(codes), len(codes)))


def ref_build(builder, tris, variant="b8"):
    tris = _tris(tris)
    n = len(tris)
    cap = 2 * n + 128
    nodes = np.zeros(cap, NODE1)
    cnt = np.zeros(1, np.uint32)
    root = np.zeros(1, np.uint32)
    ref(variant).ref_build(REF_BUILDERS[builder], _p(tris), n, _p(nodes), cap, _p(cnt), _p(root))
    return nodes[: int(cnt[0])], int(root[0])


def ref_trace(nodes, root, tris, w, h, origin, tracer=0, variant="b8"):
    tris = _tris(tris)
    o = np.asarray(origin, np.float32)
    img = np.empty(w * h * 3, np.uint8)
    ref(variant).ref_trace(tracer, _p(nodes), len(nodes), root, _p(tris), len(tris), w, h, _p(o), _p(img))
    return img


def ref_traverse(nodes, root, tris, rays, variant="b8"):
    tris = _tris(tris)
    rays = np.ascontiguousarray(rays, np.float32)
    hit = np.empty(len(rays), np.uint32)
    tests = np.empty(len(rays), np.uint32)
    ref(variant).ref_traverse(_p(nodes), len(nodes), root, _p(tris), len(tris), _p(rays), len(rays),
                              _p(hit), _p(tests))
    return hit, tests


def ref_heatmap_colour(xs, variant="b8"):
    """The reference's own get_heatmap_colour of each x: float32 (n, 3)."""
    xs = np.ascontiguousarray(xs, np.float32).ravel()
    out = np.empty((len(xs), 3), np.float32)
    ref(variant).ref_heatmap_colour(_p(xs), len(xs), _p(out))
    return out


def ref_write_bmp(path, w, h, rgb, variant="b8"):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    return int(ref(variant).ref_write_bmp(path.encode(), w, h, _p(rgb)))


def ref_load_obj(path, cap=1 << 26, variant="b8"):
    buf = np.empty((cap, 9), np.float32)
    n = ref(variant).ref_load_obj(path.encode(), _p(buf), cap)
    return buf[: min(n, cap)].copy()
