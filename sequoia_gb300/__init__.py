"""sequoia_gb300 -- GB300-native BVH build and ray trace behind Sequoia's interface.

Python host binding of libsequoia_gpu.so (the C ABI in include/sequoia_gpu.h).
The classes mirror the reference's host interface (src/builder.h:81-104,
src/tracer.h:118-135): `Builder.build_hierarchy*` return a `Hierarchy` and
`trace()` returns the heatmap bytes, but every call runs the CUDA kernels
through the C ABI.  There is no CPU fallback: if the library is missing or
no GPU is present, calls raise.

Arrays: host arguments are numpy arrays; device arguments are any object with
`__cuda_array_interface__` (e.g. a torch CUDA tensor) or a raw integer
address.  Triangles are float32 (n, 9); rays float32 (n, 8)
{ox, oy, oz, tmin, dx, dy, dz, tmax}.
"""
from __future__ import annotations

import ctypes as C
import weakref
import os

import numpy as np

__all__ = ["Context", "Bvh", "Hierarchy", "Builder", "trace", "trace_packet", "trace_bundle", "traverse", "SequoiaError",
           "NODE1", "HIT", "NO_HIT", "library_path", "load_library", "load_obj", "parse_obj",
           "encode_bmp", "write_bmp"]

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "libsequoia_gpu.so")
NO_HIT = 0xFFFFFFFF
NODE1 = np.dtype([("min", "<f4", 3), ("count", "<u2"), ("flags", "<u2"), ("max", "<f4", 3), ("child", "<u4")])
HIT = np.dtype([("id", "<u4"), ("t", "<f4"), ("tests", "<u4")])

MODES = {"ref": 0, "closest": 1, "anyhit": 2, "packet": 3, "bundle": 4}
SCHEDS = {None: 0, "refill": 0x200, "tiles": 0x400}
BUILDERS = {"morton": 0, "sah": 1, "recursive": 1, "grid": 2}
STATUS = {0: "OK", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "device error",
          5: "unsupported", 6: "no CUDA device", 7: "exceeds a fixed capacity"}


class SequoiaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, msg))
        self.status = status


class _Options(C.Structure):
    _fields_ = [("device", C.c_int), ("stream", C.c_void_p), ("flags", C.c_uint32)]


class _BuildParams(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("sah_bins", C.c_uint32), ("leaf_size", C.c_uint32),
                ("sort_digit_bits", C.c_uint32), ("morton_bounds", C.c_uint32), ("flags", C.c_uint32)]


class _BvhInfo(C.Structure):
    _fields_ = [("node_capacity", C.c_uint32), ("root", C.c_uint32), ("tri_count", C.c_uint32),
                ("kind", C.c_uint32), ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3),
                ("wide_nodes", C.c_uint32), ("wide_levels", C.c_uint32), ("wide_launches", C.c_uint32)]


class _RaySource(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("origin", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("vfov_deg", C.c_float), ("rays", C.c_void_p), ("ray_count", C.c_uint32)]


class _BatchMesh(C.Structure):
    _fields_ = [("tris", C.c_void_p), ("tri_count", C.c_uint32), ("rays", _RaySource)]


class _BatchParams(C.Structure):
    _fields_ = [("builder", C.c_uint32), ("sort_digit_bits", C.c_uint32), ("wide", C.c_uint32),
                ("block_threads", C.c_uint32), ("mode", C.c_uint32), ("flags", C.c_uint32),
                ("sah_bins", C.c_uint32), ("leaf_size", C.c_uint32)]


class _ObjInfo(C.Structure):
    _fields_ = [("faces", C.c_uint32), ("vertices", C.c_uint32), ("lines", C.c_uint32), ("threads", C.c_uint32)]


class _BatchInfo(C.Structure):
    _fields_ = [("meshes", C.c_uint32), ("tris", C.c_uint32), ("rays", C.c_uint32), ("graph", C.c_uint32),
                ("params", _BatchParams)]


_lib = None


def library_path():
    return _LIB_PATH


def load_library():
    """Load libsequoia_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise RuntimeError("libsequoia_gpu.so is not built (run `python -c \"import __graft_entry__ as g; g.build()\"`)")
    L = C.CDLL(_LIB_PATH)
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
    sig = {
        "sq_abi_version": (u32, []),
        "sq_create": (i32, [C.POINTER(vp), C.POINTER(_Options)]),
        "sq_destroy": (i32, [vp]),
        "sq_last_error": (C.c_char_p, [vp]),
        "sq_sync": (i32, [vp, C.POINTER(u32)]),
        "sq_build": (i32, [vp, vp, u32, C.POINTER(_BuildParams), C.POINTER(vp)]),
        "sq_bvh_free": (i32, [vp]),
        "sq_bvh_get_info": (i32, [vp, C.POINTER(_BvhInfo)]),
        "sq_bvh_export_node1": (i32, [vp, vp, u32, C.POINTER(u32), C.POINTER(u32)]),
        "sq_bvh_import_node1": (i32, [vp, vp, u32, u32, vp, u32, C.POINTER(vp)]),
        "sq_morton_codes": (i32, [vp, vp, u32, u32, vp, vp]),
        "sq_radix_sort_pairs": (i32, [vp, vp, vp, u32, u32, u32, vp, vp]),
        "sq_bvh_export_sorted": (i32, [vp, vp, vp]),
        "sq_bvh_export_sorted64": (i32, [vp, vp, vp]),
        "sq_trace": (i32, [vp, vp, C.POINTER(_RaySource), u32, vp, vp]),
        "sq_trace_batches": (i32, [vp, vp, C.POINTER(_RaySource), u32, u32, vp, vp]),
        "sq_traverse": (i32, [vp, vp, u32, u32, vp, u32, vp]),
        "sq_debug_inject": (i32, [vp, u32, u32]),
        "sq_debug_memory": (i32, [vp, vp]),
        "sq_last_timings": (i32, [vp, C.POINTER(C.c_float * 8)]),
        "sq_last_trace_stats": (i32, [vp, C.POINTER(C.c_uint64 * 4)]),
        "sq_batch_create": (i32, [vp, C.POINTER(_BatchMesh), u32, C.POINTER(_BatchParams), C.POINTER(vp)]),
        "sq_batch_run": (i32, [vp, vp, vp]),
        "sq_batch_info_get": (i32, [vp, C.POINTER(_BatchInfo)]),
        "sq_batch_free": (i32, [vp]),
        "sq_batch_autotune": (i32, [vp, C.c_char_p, C.POINTER(_BatchParams), C.POINTER(C.c_float)]),
        "sq_obj_load": (i32, [C.c_char_p, u32, C.POINTER(vp), C.POINTER(u32), C.POINTER(_ObjInfo)]),
        "sq_obj_parse": (i32, [vp, C.c_uint64, u32, C.POINTER(vp), C.POINTER(u32), C.POINTER(_ObjInfo)]),
        "sq_obj_free": (None, [vp]),
        "sq_bmp_write": (i32, [C.c_char_p, u32, u32, vp]),
        "sq_bmp_size": (C.c_uint64, [u32, u32]),
        "sq_bmp_encode": (i32, [u32, u32, vp, vp]),
        "sq_host_last_error": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _addr(x):
    """Address of a host numpy array, a device array or an int (None -> None)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return x.ctypes.data
    cai = getattr(x, "__cuda_array_interface__", None)
    if cai is not None:
        return int(cai["data"][0])
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    raise TypeError("unsupported buffer type %r" % type(x))


def _len(x, width):
    if isinstance(x, np.ndarray):
        return x.size // width
    shape = getattr(x, "shape", None)
    if shape is not None:
        total = 1
        for s in shape:
            total *= int(s)
        return total // width
    raise TypeError("cannot infer the length of %r" % type(x))


class Bvh:
    """A device-resident BVH (sq_bvh)."""

    def __init__(self, ctx, handle, tris_ref=None):
        self.ctx = ctx
        self.handle = handle
        self._tris_ref = tris_ref  # keeps a device triangle buffer alive
        ctx._owned.add(self)

    def info(self):
        info = _BvhInfo()
        self.ctx._check(load_library().sq_bvh_get_info(self.handle, C.byref(info)))
        return info

    @property
    def node_capacity(self):
        return self.info().node_capacity

    @property
    def root(self):
        return self.info().root

    def export_node1(self):
        L = load_library()
        cap = self.info().node_capacity
        nodes = np.zeros(cap, NODE1)
        cnt, root = C.c_uint32(), C.c_uint32()
        self.ctx._check(L.sq_bvh_export_node1(self.handle, nodes.ctypes.data, cap, C.byref(cnt), C.byref(root)))
        return nodes, int(root.value)

    def export_sorted(self):
        n = self.info().tri_count
        codes = np.empty(n, np.uint32)
        perm = np.empty(n, np.uint32)
        self.ctx._check(load_library().sq_bvh_export_sorted(self.handle, codes.ctypes.data, perm.ctypes.data))
        return codes, perm

    def export_sorted64(self):
        n = self.info().tri_count
        codes = np.empty(n, np.uint64)
        perm = np.empty(n, np.uint32)
        self.ctx._check(load_library().sq_bvh_export_sorted64(self.handle, codes.ctypes.data, perm.ctypes.data))
        return codes, perm

    def free(self):
        # after the context is closed the library has released the BVH's
        # memory; the handle must not reach sq_bvh_free then
        if self.handle and self.ctx.handle:
            load_library().sq_bvh_free(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Many meshes and ray tiles built and traced by one launch sequence
    (sq_batch), replayed as a CUDA graph."""

    def __init__(self, ctx, handle, keep):
        self.ctx = ctx
        self.handle = handle
        self._keep = keep
        ctx._owned.add(self)

    def info(self):
        i = _BatchInfo()
        self.ctx._check(load_library().sq_batch_info_get(self.handle, C.byref(i)))
        p = i.params
        return {"meshes": i.meshes, "tris": i.tris, "rays": i.rays, "graph": bool(i.graph), "builder": p.builder,
                "sort_digit_bits": p.sort_digit_bits, "sah_bins": p.sah_bins, "leaf_size": p.leaf_size,
                "wide": p.wide, "block_threads": p.block_threads, "mode": p.mode}

    def run(self, hits=True, heatmap=False):
        n = self.info()["rays"]
        h_arr = np.empty(n, HIT) if hits is True else (hits if hits is not False else None)
        m_arr = np.empty(n * 3, np.uint8) if heatmap is True else (heatmap if heatmap is not False else None)
        self.ctx._check(load_library().sq_batch_run(self.handle, _addr(h_arr), _addr(m_arr)))
        return h_arr, m_arr

    def autotune(self, cache_path=None):
        best = _BatchParams()
        ms = C.c_float()
        path = cache_path.encode() if cache_path else None
        self.ctx._check(load_library().sq_batch_autotune(self.handle, path, C.byref(best), C.byref(ms)))
        out = {"wide": best.wide, "block_threads": best.block_threads}
        if best.builder == BUILDERS["sah"]:
            out["sah_bins"] = best.sah_bins
        else:
            out["sort_digit_bits"] = best.sort_digit_bits
        return out, ms.value

    def free(self):
        if self.handle and self.ctx.handle:
            load_library().sq_batch_free(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """A CUDA context wrapper (sq_ctx): one device, one stream."""

    def __init__(self, device: int = 0, stream=None):
        L = load_library()
        opt = _Options(device, stream if stream is not None else None, 1 if stream is not None else 0)
        h = C.c_void_p()
        self.handle = None
        self._owned = weakref.WeakSet()  # BVHs and batches made on this context
        st = L.sq_create(C.byref(h), C.byref(opt))
        if st != 0:
            raise SequoiaError(st, "sq_create failed")
        self.handle = h

    def _check(self, st):
        if st != 0:
            msg = load_library().sq_last_error(self.handle)
            raise SequoiaError(st, msg.decode() if msg else "")

    def close(self):
        """Free every BVH and batch still open on the context, then the
        context (sq_destroy)."""
        if getattr(self, "handle", None):
            for obj in list(self._owned):
                obj.free()
            load_library().sq_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        bits = C.c_uint32()
        self._check(load_library().sq_sync(self.handle, C.byref(bits)))
        return bits.value

    def build(self, tris, builder="morton", bins=8, leaf=8, digit_bits=8, morton_bounds=0, flags=0, wide=False,
              morton64=False):
        n = _len(tris, 9)
        if wide:
            flags |= 2
        if morton64:
            flags |= 4  # 60-bit codes (build_hierarchy_morton2)
        p = _BuildParams(BUILDERS[builder] if isinstance(builder, str) else int(builder), bins, leaf,
                         digit_bits, morton_bounds, flags)
        h = C.c_void_p()
        self._check(load_library().sq_build(self.handle, _addr(tris), n, C.byref(p), C.byref(h)))
        keep = None if isinstance(tris, np.ndarray) else tris
        return Bvh(self, h, keep)

    def import_node1(self, nodes, root, tris):
        nodes = np.ascontiguousarray(nodes, NODE1)
        tris = np.ascontiguousarray(tris, np.float32)
        h = C.c_void_p()
        self._check(load_library().sq_bvh_import_node1(self.handle, nodes.ctypes.data, len(nodes), int(root),
                                                        tris.ctypes.data, len(tris), C.byref(h)))
        return Bvh(self, h)

    def morton_codes(self, tris, bounds_mode=0):
        n = _len(tris, 9)
        codes = np.empty(n, np.uint32)
        box = np.empty(6, np.float32)
        self._check(load_library().sq_morton_codes(self.handle, _addr(tris), n, bounds_mode,
                                                   codes.ctypes.data, box.ctypes.data))
        return codes, box

    def radix_sort_pairs(self, keys, values, key_bits=32, digit_bits=8, keys_out=None, values_out=None):
        n = _len(keys, 1)
        host = keys_out is None
        if host:
            keys_out = np.empty(n, np.uint32)
            values_out = np.empty(n, np.uint32)
        self._check(load_library().sq_radix_sort_pairs(self.handle, _addr(keys), _addr(values), n, key_bits,
                                                       digit_bits, _addr(keys_out), _addr(values_out)))
        return keys_out, values_out

    def _ray_source(self, rays=None, camera=None, width=0, height=0, origin=(0, 0, 0), target=(0, 0, -1),
                    up=(0, 1, 0), vfov=60.0):
        src = _RaySource()
        if rays is not None:
            src.kind = 2
            src.rays = _addr(rays)
            src.ray_count = _len(rays, 8)
            return src, src.ray_count
        src.kind = 0 if camera == "reference" else 1
        src.width, src.height = width, height
        src.origin[:] = [float(v) for v in origin]
        src.target[:] = [float(v) for v in target]
        src.up[:] = [float(v) for v in up]
        src.vfov_deg = float(vfov)
        return src, width * height

    def trace(self, bvh, mode="closest", rays=None, camera=None, width=0, height=0, origin=(0, 0, 0),
              target=(0, 0, -1), up=(0, 1, 0), vfov=60.0, hits=True, heatmap=False, binary=False, k=0,
              sched=None, ramp=False):
        """Trace rays; returns (hits structured array or None, heatmap bytes or None).
        `hits` / `heatmap` may also be device buffers to write into.  `binary`
        forces the binary tree when the BVH also has an 8-wide one.  `sched`
        ("refill" or "tiles", closest / any-hit) chooses how rays are given
        to GPU lanes; the results do not depend on it.  `ramp`: heatmap in
        the reference's colour ramp instead of grey.  Modes "packet" and
        "bundle" (trace_packet<k> / trace_bundle<k>) take the packet size
        `k`, the reference camera and produce the heatmap only."""
        if mode in ("packet", "bundle"):
            hits, heatmap = False, (True if heatmap is False else heatmap)
        src, count = self._ray_source(rays, camera, width, height, origin, target, up, vfov)
        h_arr = np.empty(count, HIT) if hits is True else (hits if hits is not False else None)
        m_arr = np.empty(count * 3, np.uint8) if heatmap is True else (heatmap if heatmap is not False else None)
        m = MODES[mode] | (0x100 if binary else 0) | (int(k) << 16) | SCHEDS[sched] | (0x800 if ramp else 0)
        self._check(load_library().sq_trace(self.handle, bvh.handle, C.byref(src), m, _addr(h_arr), _addr(m_arr)))
        return h_arr, m_arr

    def trace_batches(self, bvh, mode="closest", batches=(), hits=True, heatmap=False, binary=False, sched=None):
        """Trace many ray batches against one BVH in one launch
        (sq_trace_batches).  `batches`: a list whose items are explicit ray
        arrays (numpy or device tensors, (n, 8) float32) or camera dicts
        (`camera`, `width`, `height`, `origin`, `target`, `up`, `vfov`).
        Returns (hits, heatmap) laid out batch after batch."""
        arr = (_RaySource * max(1, len(batches)))()
        total = 0
        for k, item in enumerate(batches):
            if isinstance(item, dict):
                src, cnt = self._ray_source(**item)
            else:
                src, cnt = self._ray_source(rays=item)
            arr[k] = src
            total += cnt
        h_arr = np.empty(total, HIT) if hits is True else (hits if hits is not False else None)
        m_arr = np.empty(total * 3, np.uint8) if heatmap is True else (heatmap if heatmap is not False else None)
        m = MODES[mode] | (0x100 if binary else 0) | SCHEDS[sched]
        self._check(load_library().sq_trace_batches(self.handle, bvh.handle, arr, len(batches), m, _addr(h_arr),
                                                    _addr(m_arr)))
        return h_arr, m_arr

    def traverse(self, bvh, index, count, rays, hits=True):
        """traverse() from the node group [index, index + count) for explicit
        rays (sq_traverse): per ray the hit flag (id 0 or NO_HIT) and the
        box-test count."""
        n = _len(rays, 8)
        h_arr = np.empty(n, HIT) if hits is True else hits
        self._check(load_library().sq_traverse(self.handle, bvh.handle, int(index), int(count), _addr(rays), n,
                                               _addr(h_arr)))
        return h_arr

    # failure-detection test hooks (sq_debug_inject / sq_debug_memory)
    INJECT = {"off": 0, "stall_lookback": 1, "stall_barrier": 2, "fail_alloc": 3}

    def debug_inject(self, what, limit=0):
        self._check(load_library().sq_debug_inject(self.handle, self.INJECT[what], int(limit)))

    def debug_memory(self):
        """{live_blocks, live_bytes, cached_blocks, cached_bytes} of the
        context's device allocator."""
        arr = (C.c_uint64 * 4)()
        self._check(load_library().sq_debug_memory(self.handle, C.byref(arr)))
        return {"live_blocks": arr[0], "live_bytes": arr[1], "cached_blocks": arr[2], "cached_bytes": arr[3]}

    def trace_stats(self):
        arr = (C.c_uint64 * 4)()
        self._check(load_library().sq_last_trace_stats(self.handle, C.byref(arr)))
        return {"box_tests": arr[0], "tri_tests": arr[1], "bytes": arr[2], "nodes": arr[3]}

    def batch(self, meshes, mode="closest", wide=True, digit_bits=8, block=128, graph=True, builder="morton",
              bins=8, leaf=8):
        """meshes: list of dicts with `tris` and either `rays` (explicit) or a
        camera (`camera`, `width`, `height`, `origin`, `target`, `up`, `vfov`).
        builder: "morton" (digit_bits) or "sah" (bins, leaf)."""
        arr = (_BatchMesh * len(meshes))()
        keep = []
        for k, m in enumerate(meshes):
            t = m["tris"]
            if isinstance(t, np.ndarray):
                t = np.ascontiguousarray(t, np.float32)
            keep.append(t)
            arr[k].tris = _addr(t)
            arr[k].tri_count = _len(t, 9)
            cam = {kk: m[kk] for kk in ("camera", "width", "height", "origin", "target", "up", "vfov") if kk in m}
            src, _ = self._ray_source(rays=m.get("rays"), **cam)
            if m.get("rays") is not None:
                keep.append(m["rays"])
            arr[k].rays = src
        p = _BatchParams(BUILDERS[builder], digit_bits, 1 if wide else 0, block, MODES[mode], 1 if graph else 0,
                         bins, leaf)
        h = C.c_void_p()
        self._check(load_library().sq_batch_create(self.handle, arr, len(meshes), C.byref(p), C.byref(h)))
        return Batch(self, h, keep)

    def timings(self):
        arr = (C.c_float * 8)()
        self._check(load_library().sq_last_timings(self.handle, C.byref(arr)))
        return {"build": arr[0], "codes": arr[1], "sort": arr[2], "topology": arr[3], "trace": arr[4],
                "box_tests": arr[5], "tri_tests": arr[6], "wide": arr[7]}


# ---------------------------------------------------------------------------
# Mirror of the reference's host interface (src/builder.h:81-104,
# src/tracer.h:118-135, src/aabb.h:197-205).

_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class Hierarchy:
    """Host view of a BVH in the reference's layout: node_base (Node1 array),
    node_count, tri_base (the triangles), tri_count, root_index."""

    def __init__(self, node_base, root_index, tri_base, bvh=None):
        self.node_base = node_base
        self.node_count = len(node_base)
        self.tri_base = tri_base
        self.tri_count = len(tri_base)
        self.root_index = root_index
        self.bvh = bvh


class Builder:
    """Builder::build_hierarchy* (src/builder.h:81-104), on the GPU."""

    @staticmethod
    def _build(primitives, builder, **kw):
        ctx = default_context()
        tris = np.ascontiguousarray(primitives, np.float32).reshape(-1, 9)
        bvh = ctx.build(tris, builder, **kw)
        nodes, root = bvh.export_node1()
        return Hierarchy(nodes, root, tris, bvh)

    @staticmethod
    def build_hierarchy(primitives, bins=8, leaf=8):
        return Builder._build(primitives, "sah", bins=bins, leaf=leaf)

    @staticmethod
    def build_hierarchy_morton(primitives):
        return Builder._build(primitives, "morton")

    @staticmethod
    def build_hierarchy_grid(primitives, bins=8, leaf=8, scene_bounds_cells=True):
        return Builder._build(primitives, "grid", bins=bins, leaf=leaf, flags=1 if scene_bounds_cells else 0)


def _bvh_of(h):
    ctx = default_context()
    if h.bvh is not None:
        return ctx, h.bvh
    h.bvh = ctx.import_node1(h.node_base, h.root_index, h.tri_base)
    return ctx, h.bvh


def trace(hierarchy, w, h, origin):
    """trace() (src/tracer.cpp:195-230): reference camera at `origin`, w x h
    primary rays; returns the w*h*3 heatmap bytes."""
    ctx, bvh = _bvh_of(hierarchy)
    _, heat = ctx.trace(bvh, mode="ref", camera="reference", width=w, height=h, origin=origin,
                        hits=False, heatmap=True)
    return heat


def trace_packet(hierarchy, w, h, origin, k=8):
    """trace_packet<k> (src/tracer.cpp:232-281): the heatmap bytes of packets
    of k rays (1, 2, 4 or 8) counting box tests together."""
    ctx, bvh = _bvh_of(hierarchy)
    _, heat = ctx.trace(bvh, mode="packet", k=k, camera="reference", width=w, height=h, origin=origin)
    return heat


def trace_bundle(hierarchy, w, h, origin, k=64):
    """trace_bundle<k> (src/tracer.cpp:292-362): the heatmap bytes of bundles
    of k rays (16 or 64) split into packets of 8."""
    ctx, bvh = _bvh_of(hierarchy)
    _, heat = ctx.trace(bvh, mode="bundle", k=k, camera="reference", width=w, height=h, origin=origin)
    return heat


def traverse(hierarchy, rays):
    """traverse() (src/tracer.cpp:47-65) for explicit rays: returns (hit flag,
    number of ray-box tests) per ray."""
    ctx, bvh = _bvh_of(hierarchy)
    hits, _ = ctx.trace(bvh, mode="ref", rays=np.ascontiguousarray(rays, np.float32))
    return (hits["id"] != NO_HIT).astype(np.uint32), hits["tests"].copy()


# ---------------------------------------------------------------- host I/O

def _host_check(status):
    if status != 0:
        raise SequoiaError(status, load_library().sq_host_last_error().decode(errors="replace"))


def _obj_result(L, tp, n, info):
    try:
        tris = np.empty((n.value, 9), np.float32)
        if n.value:
            C.memmove(tris.ctypes.data, tp.value, tris.nbytes)
    finally:
        L.sq_obj_free(tp)
    return tris, {"faces": info.faces, "vertices": info.vertices, "lines": info.lines, "threads": info.threads}


def load_obj(path, threads=0):
    """loadOBJFromFile (src/main.cpp:108-179) with the reference's parse:
    returns (float32 (n, 9) triangles, {faces, vertices, lines, threads})."""
    L = load_library()
    tp, n, info = C.c_void_p(), C.c_uint32(), _ObjInfo()
    _host_check(L.sq_obj_load(os.fsencode(path), threads, C.byref(tp), C.byref(n), C.byref(info)))
    return _obj_result(L, tp, n, info)


def parse_obj(data, threads=0):
    """The same parse over OBJ text in memory (bytes)."""
    L = load_library()
    buf = np.frombuffer(bytes(data), np.uint8) if len(data) else np.zeros(1, np.uint8)
    tp, n, info = C.c_void_p(), C.c_uint32(), _ObjInfo()
    _host_check(L.sq_obj_parse(buf.ctypes.data, len(data), threads, C.byref(tp), C.byref(n), C.byref(info)))
    return _obj_result(L, tp, n, info)


def encode_bmp(rgb, w, h):
    """The reference's render.bmp (src/main.cpp:335-336) as bytes."""
    L = load_library()
    rgb = np.ascontiguousarray(rgb, np.uint8).reshape(-1)
    if rgb.size != 3 * w * h:
        raise ValueError("rgb must hold w*h*3 bytes")
    out = np.empty(int(L.sq_bmp_size(w, h)), np.uint8)
    _host_check(L.sq_bmp_encode(w, h, rgb.ctypes.data if rgb.size else None, out.ctypes.data))
    return out.tobytes()


def write_bmp(path, rgb, w, h):
    L = load_library()
    rgb = np.ascontiguousarray(rgb, np.uint8).reshape(-1)
    if rgb.size != 3 * w * h:
        raise ValueError("rgb must hold w*h*3 bytes")
    _host_check(L.sq_bmp_write(os.fsencode(path), w, h, rgb.ctypes.data if rgb.size else None))
