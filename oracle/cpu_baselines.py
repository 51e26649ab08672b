"""CPU baselines of the build and trace path, timed on this host.

TEST AND BASELINE INFRASTRUCTURE ONLY: used by the benchmark's CPU legs and
run by hand to tabulate the reference's own code beside the oracle's
restatement of it.  Two implementations are timed where they exist:

  port       the oracle (liboracle.so): the C restatement of the
             reference's builders and tracers, OpenMP over the host's cores
  reference  the reference's own code (oracle/_ref/libseqref_*.so), built
             from its sources by oracle/build_ref.sh where they are present

Builders are timed as the median of `reps` calls after one warm-up; a
reference builder that crashes (the reference's grid builders corrupt the
heap on some inputs) is reported as such, because every reference call runs
in a child process.  Tracers use the reference camera (src/tracer.cpp:202-
216) at 1920x1080 on the 8-bin SAH tree of the scene, so their heatmaps are
the ones the reference's trace(), trace_packet<8> and trace_bundle<64> make.

    python oracle/cpu_baselines.py [--reps 3] [--scenes icosphere_l6,soup_2m]

prints a markdown table of both implementations on this host.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402

# reference builder kinds (ref_build / ref_time_build) and the variant built
# with the matching NUM_BINS
REF_BUILDS = {
    "sah8": (0, "b8"), "sah16": (0, "b16"), "sah32": (0, "b32"), "horizontal": (1, "b8"), "grid": (2, "b8"),
    "grid_sse": (3, "b8"), "grid_avx": (4, "b8"), "morton": (5, "b8"), "morton60": (6, "b8"),
}
REF_TRACERS = {"trace": 0, "packet8": 1, "bundle64": 2}
TRACE_W, TRACE_H = 1920, 1080


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def scene(name):
    from sequoia_gb300 import scenes
    if name == "icosphere_l6":
        return scenes.displaced_icosphere(6, seed=1)
    if name == "soup_2m":
        return scenes.gaussian_soup(2_000_000, 64, seed=2)
    if name == "terrain_4m":
        return scenes.heightfield(2048, 1024, seed=3)
    raise ValueError(name)


def reference_camera(tris):
    """trace()'s camera for a scene (src/main.cpp:312-318)."""
    v = tris.reshape(-1, 3)
    lo, hi = v.min(0), v.max(0)
    c = (lo + hi) * np.float32(0.5)
    return np.array([c[0], c[1], np.float32(2) * lo[2] - c[2]], np.float32)


def _median(f, reps):
    f()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        f()
        ts.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(ts)


# ------------------------------------------------------------------ port

def port_builders(tris, reps=3, which=("sah8", "sah16", "sah32", "grid", "morton", "morton60")):
    """Oracle builder times in ms (median of reps).  sahB: B bins, leaf <= 8
    as the reference; sah16_leaf4: 16 bins, leaf <= 4."""
    out = {}
    jobs = {"sah8": lambda: O.build_sah(tris, 8, 8), "sah16": lambda: O.build_sah(tris, 16, 8),
            "sah16_leaf4": lambda: O.build_sah(tris, 16, 4),
            "sah32": lambda: O.build_sah(tris, 32, 8), "grid": lambda: O.build_grid(tris, 8, 8),
            "morton": lambda: O.build_morton(tris), "morton60": lambda: O.build_morton64(tris)}
    for k in which:
        out[k] = _median(jobs[k], reps)
    return out


def port_tracers(tris, reps=3, which=("trace", "packet8", "bundle64")):
    """Oracle tracer times in ms on the 8-bin SAH tree, reference camera,
    1920x1080 (ray generation outside the timing for the scalar trace)."""
    nodes, root, _ = O.build_sah(tris, 8, 8)
    cam = reference_camera(tris)
    rays = O.rays_reference_camera(TRACE_W, TRACE_H, cam)
    jobs = {"trace": lambda: O.trace(nodes, root, tris, rays, 0),
            "packet8": lambda: O.trace_coherent(nodes, root, TRACE_W, TRACE_H, cam, False, 8),
            "bundle64": lambda: O.trace_coherent(nodes, root, TRACE_W, TRACE_H, cam, True, 64)}
    return {k: _median(jobs[k], reps) for k in which}


def port_step(tris, cfg):
    """One step of the benchmark's workload on the CPU: Morton build of all
    triangles, then closest-hit trace of every pinhole ray with the
    test-count heatmap.  Returns (build s, trace s, rays)."""
    t0 = time.perf_counter()
    nodes, root, _, _ = O.build_morton(tris)
    t1 = time.perf_counter()
    rays = O.rays_pinhole(cfg["width"], cfg["height"], cfg["eye"], cfg["target"], cfg["up"], cfg["vfov"])
    t2 = time.perf_counter()
    _, _, tests = O.trace(nodes, root, tris, rays, 1)
    O.heatmap(tests)
    t3 = time.perf_counter()
    return t1 - t0, t3 - t2, len(rays)


# ------------------------------------------------------------- reference

def _ref_lib(variant):
    L = O.ref(variant)
    import ctypes as C
    L.ref_time_build.argtypes = [C.c_int, C.c_void_p, C.c_uint32]
    L.ref_time_build.restype = C.c_double
    L.ref_time_trace.argtypes = [C.c_int, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32,
                                 C.c_uint32, C.c_void_p]
    L.ref_time_trace.restype = C.c_double
    L.ref_set_threads(min(64, host_threads()))
    return L


def _ref_one(kind, item, scene_name, reps):
    """Runs in a child process: one reference builder or tracer, median ms."""
    tris = np.ascontiguousarray(scene(scene_name), np.float32)
    if kind == "build":
        code, variant = REF_BUILDS[item]
        L = _ref_lib(variant)
        ts = [L.ref_time_build(code, tris.ctypes.data, len(tris)) for _ in range(reps + 1)][1:]
        return statistics.median(ts)
    L = _ref_lib("b8")
    nodes, root = O.ref_build("recursive", tris, "b8")
    cam = reference_camera(tris)
    ts = [L.ref_time_trace(REF_TRACERS[item], nodes.ctypes.data, len(nodes), root, tris.ctypes.data, len(tris),
                           TRACE_W, TRACE_H, cam.ctypes.data) for _ in range(reps + 1)][1:]
    return statistics.median(ts)


def reference_item(kind, item, scene_name, reps=3, timeout=600):
    """Median ms of one reference builder / tracer in a child process, or a
    string saying why there is none (crash, not built)."""
    if not O.ref_available("b8"):
        return "not built"
    cmd = [sys.executable, os.path.abspath(__file__), "--one", kind, item, scene_name, "--reps", str(reps)]
    try:
        p = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    except subprocess.TimeoutExpired:
        return "timed out"
    if p.returncode != 0:
        return "crashed (exit %d: %s)" % (p.returncode, (p.stderr.strip().splitlines() or ["?"])[-1][:80])
    return float(p.stdout.strip().splitlines()[-1])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--scenes", default="icosphere_l6,soup_2m")
    ap.add_argument("--one", nargs=3, metavar=("KIND", "ITEM", "SCENE"))
    args = ap.parse_args()
    if args.one:
        print(_ref_one(args.one[0], args.one[1], args.one[2], args.reps))
        return
    O.set_threads(host_threads())
    rows = []
    for sc in args.scenes.split(","):
        tris = scene(sc)
        pb = port_builders(tris, args.reps)
        pt = port_tracers(tris, args.reps)
        for item in ("sah8", "sah16", "sah32", "horizontal", "grid", "grid_sse", "grid_avx", "morton", "morton60"):
            port = pb.get(item)
            rows.append((sc, "build " + item, reference_item("build", item, sc, args.reps), port))
        for item in REF_TRACERS:
            rows.append((sc, item, reference_item("trace", item, sc, args.reps), pt[item]))
    print("host: %s, %d threads" % (os.uname().machine, host_threads()))
    print("| scene | item | reference (ms) | port (ms) |")
    print("|---|---|---|---|")
    for sc, item, r, p in rows:
        fr = "%.1f" % r if isinstance(r, float) else r
        fp = "%.1f" % p if p is not None else "-"
        print("| %s | %s | %s | %s |" % (sc, item, fr, fp))
    print(json.dumps([dict(scene=a, item=b, reference=c, port=d) for a, b, c, d in rows]))


if __name__ == "__main__":
    main()
