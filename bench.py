#!/usr/bin/env python3
"""Benchmark: LBVH build + closest-hit trace on one GB300 (per rank).

Workload (one step): Morton/LBVH build of a 2,000,000-triangle Gaussian soup
(64 clusters, seed 2) resident in HBM, then a closest-hit trace of
3840x2160 pinhole primary rays from (0, 0, -40) aimed at the origin, with
per-ray hit records and the test-count heatmap written to HBM.

  value     Mrays/s for the whole step (rays / (build + trace) device time)
  e2e       the same through the C ABI with pinned host buffers: triangle
            upload, build, trace, hit + heatmap download inside the timing
  roofline  the trace kernel: algorithmic bytes (hit record + heatmap +
            32 B per ray-box test + 36 B per triangle test) / kernel time
            against the measured HBM copy bandwidth
  cpu_baseline  the CPU implementation (the reference built from its sources
            where available, else the oracle's restatement) on a bounded
            sample of the same workload, all host threads

`--impl reference` times only the CPU implementation and prints its line.
Multi-GPU (torchrun): independent replicas, one per GPU (the path does not
exchange data); value sums the rays of all ranks over the slowest rank.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "Mrays/s traced & Mtris/s built on 1 GB300: quantized+batched vs plain FP32, same hits"
WORKLOAD = dict(name="soup_2m", tris=2_000_000, clusters=64, seed=2, width=3840, height=2160,
                eye=(0.0, 0.0, -40.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), vfov=60.0)
KERNELS_PER_STEP = 8  # scene bounds, Morton codes, 4 onesweep passes, climb, trace


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_scene():
    from sequoia_gb300 import scenes
    w = WORKLOAD
    return scenes.gaussian_soup(w["tris"], w["clusters"], seed=w["seed"])


def cpu_trace_sample(tris, impl, threads, row_step):
    """Build on the CPU and trace every `row_step`-th image row; returns
    (build seconds, trace seconds, sampled rays, kind)."""
    import oracle as O
    w = WORKLOAD
    O.set_threads(threads)
    kind = "port"
    t0 = time.perf_counter()
    nodes, root, _, _ = O.build_morton(tris)
    t1 = time.perf_counter()
    rays = O.rays_pinhole(w["width"], w["height"], w["eye"], w["target"], w["up"], w["vfov"])
    rays = rays.reshape(w["height"], w["width"], 8)[::row_step].reshape(-1, 8).copy()
    t2 = time.perf_counter()
    O.trace(nodes, root, tris, rays, 1)
    t3 = time.perf_counter()
    return t1 - t0, t3 - t2, len(rays), kind


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    tris = make_scene()
    w = WORKLOAD
    rays_total = w["width"] * w["height"]
    threads = host_threads()
    row_step = 16
    times = []
    for i in range(args.warmup + args.steps):
        tb, tt, ns, kind = cpu_trace_sample(tris, "port", threads, row_step)
        if i >= args.warmup:
            times.append(tb + tt * (rays_total / ns))
    step_s = statistics.mean(times)
    value = rays_total / step_s / 1e6
    sample = "Morton build of all %d tris + closest-hit trace of every %dth image row (%d rays), " \
             "extrapolated to %d rays; oracle restatement (the reference's x86 code does not build here)" % (
                 w["tris"], row_step, rays_total // row_step, rays_total)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "soup_2m: 2M-triangle Gaussian soup, 3840x2160 pinhole primary rays",
                       "builder": "morton", "trace": "closest"},
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import sequoia_gb300 as sq

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl")
        dist = dist_mod
    w = WORKLOAD
    tris = make_scene()
    n = len(tris)
    rays_total = w["width"] * w["height"]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)  # torch work (L2 flush, events) and the library share one stream
    ctx = sq.Context(local, stream=stream.cuda_stream)
    d_tris = torch.from_numpy(tris).to("cuda")
    d_hits = torch.empty(rays_total * 3, dtype=torch.int32, device="cuda")
    d_heat = torch.empty(rays_total * 3, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    cam = dict(camera="pinhole", width=w["width"], height=w["height"], origin=w["eye"], target=w["target"],
               up=w["up"], vfov=w["vfov"])

    def step(src_tris, hits, heat):
        bvh = ctx.build(src_tris, "morton")
        ctx.trace(bvh, "closest", hits=hits, heatmap=heat, **cam)
        return bvh

    # warm-up
    for _ in range(args.warmup):
        step(d_tris, d_hits, d_heat).free()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    step_ms, build_ms, trace_ms, box_tests, tri_tests = [], [], [], [], []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bvh = step(d_tris, d_hits, d_heat)
        e1.record(stream)
        tm = ctx.timings()  # synchronises
        step_ms.append(e0.elapsed_time(e1))
        build_ms.append(tm["build"])
        trace_ms.append(tm["trace"])
        box_tests.append(tm["box_tests"])
        tri_tests.append(tm["tri_tests"])
        bvh.free()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = float(sum(step_ms))
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * rays_total * args.steps / (total_ms / 1e3) / 1e6

    # end to end through the public API with pinned host buffers
    h_tris = torch.from_numpy(tris).pin_memory()
    h_hits = torch.empty(rays_total * 3, dtype=torch.int32).pin_memory()
    h_heat = torch.empty(rays_total * 3, dtype=torch.uint8).pin_memory()
    e2e_ms = []
    if not args.no_e2e:
        step(h_tris, h_hits, h_heat).free()
    for _ in range(0 if args.no_e2e else args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bvh = step(h_tris, h_hits, h_heat)
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        bvh.free()
    e2e_total = float(sum(e2e_ms)) if e2e_ms else float("nan")
    if dist:
        t = torch.tensor([e2e_total], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = world * rays_total * args.steps / (e2e_total / 1e3) / 1e6

    # every builder once on the same scene (not part of the timed steps)
    builders = {}
    for name, kw in (("morton", {}), ("sah32_leaf4", dict(bins=32, leaf=4)), ("sah8_leaf8", dict(bins=8, leaf=8)),
                     ("grid", dict(bins=8, leaf=8))):
        kind = "morton" if name == "morton" else ("grid" if name == "grid" else "sah")
        ctx.build(d_tris, kind, **kw).free()  # warm
        flush.zero_()
        bvh = ctx.build(d_tris, kind, **kw)
        tb = ctx.timings()["build"]
        flush.zero_()
        ctx.trace(bvh, "closest", hits=d_hits, heatmap=d_heat, **cam)
        tm = ctx.timings()
        builders[name] = {"build_ms": tb, "trace_ms": tm["trace"], "box_tests_per_ray": tm["box_tests"] / rays_total,
                          "tri_tests_per_ray": tm["tri_tests"] / rays_total}
        bvh.free()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peak, peak_kind = measured_peaks()
    tr_ms = statistics.mean(trace_ms)
    bt = statistics.mean(box_tests)
    tt = statistics.mean(tri_tests)
    trace_bytes = rays_total * (12 + 3) + bt * 32 + tt * 36
    achieved = trace_bytes / (tr_ms / 1e3) / 1e9
    b_ms = statistics.mean(build_ms)
    build_bytes = n * (200 + 16 * 4)
    build_gbs = build_bytes / (b_ms / 1e3) / 1e9
    hits_np = d_hits.view(-1, 3).cpu().numpy()
    nhit = int((hits_np[:, 0] != -1).sum())

    cpu = None
    if not args.no_cpu_baseline:
        threads = host_threads()
        row_step = 16
        tb, tt_s, ns, kind = cpu_trace_sample(tris, "port", threads, row_step)
        cpu_value = rays_total / (tb + tt_s * (rays_total / ns)) / 1e6
        cpu = {"value": cpu_value, "unit": "Mrays/s", "cores": threads, "kind": kind,
               "sample": "Morton build of all %d tris (%.2f s) + closest-hit trace of every %dth row "
                         "(%d rays, %.2f s), extrapolated to the full image" % (n, tb, row_step, ns, tt_s)}

    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded 64-cluster Gaussian triangle soup (no dataset ships with the reference)",
        "config": {"workload": "soup_2m: %d-triangle Gaussian soup, %dx%d pinhole primary rays from (0,0,-40)"
                               % (n, w["width"], w["height"]),
                   "builder": "morton (LBVH)", "trace": "closest hit + heatmap", "tris": n, "rays": rays_total,
                   "l2": "flushed between steps (512 MB write)", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "build_mtris_s": n / (b_ms / 1e3) / 1e6,
        "trace_mrays_s": rays_total / (tr_ms / 1e3) / 1e6,
        "stage_ms": {"build": b_ms, "trace": tr_ms, "step": ms_per_step},
        "box_tests_per_ray": bt / rays_total, "tri_tests_per_ray": tt / rays_total, "hit_rays": nhit,
        "roofline": {"bound": "hbm", "kernel": "k_trace<closest>", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                     "bytes_model": "15 B/ray out + 32 B per box test + 36 B per triangle test"},
        "build_roofline": {"bound": "hbm", "achieved": build_gbs, "peak": peak, "unit": "GB/s",
                           "frac": build_gbs / peak, "bytes_model": "264 B/tri (200 + 16 x 4 sort passes)"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": n * 36,
                "d2h_bytes_per_step": rays_total * 15, "ms_per_step": e2e_total / args.steps},
        "builders": builders,
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
