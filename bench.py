#!/usr/bin/env python3
"""Benchmark: BVH build + ray trace on one GB300 (per rank).

Timed step (the 2M-triangle configuration): build a Morton LBVH of a
2,000,000-triangle Gaussian soup (64 clusters, seed 2) resident in HBM,
collapse it into the 8-wide BVH with 8-bit outward-rounded child boxes, then
trace 3840x2160 pinhole primary rays from (0, 0, -40) aimed at the origin
(closest hit), writing per-ray hit records and the test-count heatmap to HBM.
L2 is flushed between steps (512 MB write).

  value      Mrays/s of the whole step: rays / (build + collapse + trace)
  e2e        the same step through the C ABI with pinned host buffers:
             triangle upload, build, trace, hit + heatmap download inside
  plain_fp32 the same rays on the same tree traced as the plain FP32 binary
             BVH, with the hit ids and t of both forms compared
  stress     8,000,000-triangle soup (256 clusters, seed 5) and 2^24 rays with
             origins uniform in the scene box and directions uniform on the
             sphere, in 64 batches of log-uniform size [16K, 1M] traced by
             one launch: 8-wide quantised vs plain FP32, closest and any-hit
  batch      256 meshes (displaced icospheres and soups, 1K-200K triangles
             each, log-uniform, seeds 4000+i) with one square primary-ray
             tile each (side log-uniform in [64, 512]): built and traced by
             one CUDA-graph launch with the autotuned sort digit width, BVH
             width and block shape, against 256 separate build+trace calls
  roofline   the dominant kernel (the 8-wide trace): bytes it requested
             (counted by the kernel: node loads, triangle loads, ray records
             and outputs) / kernel time, against the measured HBM bandwidth
  cpu_baseline  the CPU implementation (the reference's own code where it
             builds, else the oracle's restatement) on a bounded sample

`--impl reference` times only the CPU implementation.  Multi-GPU (torchrun):
independent replicas, one per GPU; value sums all ranks' rays over the
slowest rank.
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

import numpy as np  # noqa: E402,F401

METRIC = "Mrays/s traced & Mtris/s built on 1 GB300: quantized+batched vs plain FP32, same hits"
WORKLOAD = dict(name="soup_2m", tris=2_000_000, clusters=64, seed=2, width=3840, height=2160,
                eye=(0.0, 0.0, -40.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), vfov=60.0)
STRESS = dict(tris=8_000_000, clusters=256, seed=5, rays=1 << 24, batches=64)
LBVH_KERNELS = 8  # scene bounds, Morton codes, 4 onesweep passes, climb (local + global phase)
# DRAM bytes (read + write) of one k_trace8_tiles<closest> launch on this
# workload, from the ncu capture summarised in profiles/k_trace8_tiles_soup2m.md
TRACE8_DRAM_BYTES = 115.0e6 + 106.3e6
TRACE8_DRAM_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch (profiles/k_trace8_tiles_soup2m.md)"


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
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def reduce_max(x, dist, device="cuda"):
    """Max of a per-rank float over all ranks (the slowest rank's time)."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(rays_per_step, steps, world, total_ms):
    """Mrays/s of the whole job: every rank traces rays_per_step rays per step
    (independent replicas), timed by the slowest rank."""
    return world * rays_per_step * steps / (total_ms / 1e3) / 1e6


def make_scene():
    from sequoia_gb300 import scenes
    w = WORKLOAD
    return scenes.gaussian_soup(w["tris"], w["clusters"], seed=w["seed"])


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_sample(tris, threads, row_step):
    """CPU build of the whole scene and closest-hit trace of every
    `row_step`-th image row.  Returns (build s, trace s, sampled rays, kind)."""
    import oracle as O
    w = WORKLOAD
    O.set_threads(threads)
    t0 = time.perf_counter()
    nodes, root, _, _ = O.build_morton(tris)
    t1 = time.perf_counter()
    rays = O.rays_pinhole(w["width"], w["height"], w["eye"], w["target"], w["up"], w["vfov"])
    rays = rays.reshape(w["height"], w["width"], 8)[::row_step].reshape(-1, 8).copy()
    t2 = time.perf_counter()
    O.trace(nodes, root, tris, rays, 1)
    t3 = time.perf_counter()
    return t1 - t0, t3 - t2, len(rays), "port"


def cpu_line(tris, steps, warmup):
    w = WORKLOAD
    rays_total = w["width"] * w["height"]
    threads = host_threads()
    row_step = 16
    times = []
    for i in range(warmup + steps):
        tb, tt, ns, _ = cpu_sample(tris, threads, row_step)
        if i >= warmup:
            times.append(tb + tt * (rays_total / ns))
    step_s = statistics.mean(times)
    value = rays_total / step_s / 1e6
    sample = ("Morton build of all %d tris + closest-hit trace of every %dth image row (%d rays), extrapolated to "
              "%d rays; the oracle's C restatement with OpenMP (the reference's own code needs x86 intrinsics)"
              % (len(tris), row_step, rays_total // row_step, rays_total))
    return value, step_s, threads, sample


def run_reference(args):
    rank, _, _ = dist_info()
    if rank != 0:
        return
    tris = make_scene()
    value, step_s, threads, sample = cpu_line(tris, args.steps, args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "soup_2m: 2M-triangle Gaussian soup, 3840x2160 pinhole primary rays",
                       "builder": "morton", "trace": "closest"},
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def stress_leg(ctx, flush, torch):
    """8M-triangle soup, 2^24 incoherent rays in 64 batches, one launch per
    form: 8-wide quantised vs plain FP32 binary, closest and any-hit."""
    from sequoia_gb300 import scenes
    s = STRESS
    tris = scenes.gaussian_soup(s["tris"], s["clusters"], seed=s["seed"])
    lo, hi = scenes.scene_box(tris)
    sizes = scenes.batch_sizes(s["rays"], s["batches"], seed=s["seed"])
    rays = torch.from_numpy(scenes.random_rays(int(sizes.sum()), lo, hi, seed=s["seed"])).cuda()
    d_tris = torch.from_numpy(tris).cuda()
    h_a = torch.empty(s["rays"] * 3, dtype=torch.int32, device="cuda")
    h_b = torch.empty_like(h_a)
    bvh = ctx.build(d_tris, "morton", wide=True)
    out = {"tris": len(tris), "rays": int(sizes.sum()), "batches": len(sizes),
           "batch_sizes_min_max": [int(sizes.min()), int(sizes.max())], "build_ms": ctx.timings()["build"]}
    for mode in ("closest", "anyhit"):
        t = {}
        for form in ("binary", "wide"):
            best = None
            for _ in range(2):
                flush.zero_()
                ctx.trace(bvh, mode, rays=rays, hits=h_b if form == "binary" else h_a, binary=(form == "binary"))
                ms = ctx.timings()["trace"]
                best = ms if best is None else min(best, ms)
            t[form] = best
        a = h_a.view(-1, 3)
        b = h_b.view(-1, 3)
        if mode == "closest":
            same = bool(torch.equal(a[:, :2], b[:, :2]))
        else:
            same = bool(torch.equal(a[:, 0] != -1, b[:, 0] != -1))
        out[mode] = {"wide_mrays_s": s["rays"] / t["wide"] / 1e3, "plain_fp32_mrays_s": s["rays"] / t["binary"] / 1e3,
                     "speedup": t["binary"] / t["wide"], "same_hits": same}
    bvh.free()
    return out


def batch_leg(ctx, flush, torch, sq):
    """256 meshes with one ray tile each: one graph launch (autotuned) vs 256
    separate plain build + trace calls, same hits."""
    from sequoia_gb300 import scenes
    meshes, tiles = scenes.mesh_batch(256, seed=4000)
    d_meshes = [torch.from_numpy(m).cuda() for m in meshes]
    descs = []
    for m, dm, side in zip(meshes, d_meshes, tiles):
        lo, hi = scenes.scene_box(m)
        c = (lo + hi) * 0.5
        ext = float(max(hi - lo))
        eye = (float(c[0]), float(c[1]) + 0.5 * ext, float(c[2]) - 2.5 * ext)
        descs.append(dict(tris=dm, camera="pinhole", width=int(side), height=int(side), origin=eye,
                          target=tuple(float(x) for x in c), up=(0.0, 1.0, 0.0), vfov=50.0))
    n_tris = sum(len(m) for m in meshes)
    n_rays = sum(int(t) * int(t) for t in tiles)
    b = ctx.batch(descs, mode="closest", wide=True, graph=True)
    best, tune_ms = b.autotune()
    for _ in range(3):
        b.run(hits=False)
    times = []
    stream = torch.cuda.current_stream()
    for _ in range(5):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(hits=False)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    got, _ = b.run()
    b.free()
    # 256 separate plain (binary FP32, default digits) build + trace calls
    d_hits = torch.empty(n_rays * 3, dtype=torch.int32, device="cuda")
    def separate():
        off = 0
        for d in descs:
            bvh = ctx.build(d["tris"], "morton")
            cnt = d["width"] * d["height"]
            ctx.trace(bvh, "closest", hits=d_hits[3 * off:3 * (off + cnt)], camera="pinhole", width=d["width"],
                      height=d["height"], origin=d["origin"], target=d["target"], up=d["up"], vfov=d["vfov"])
            bvh.free()
            off += cnt
    separate()
    sep = []
    for _ in range(3):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        separate()
        e1.record(stream)
        e1.synchronize()
        sep.append(e0.elapsed_time(e1))
    ref = d_hits.view(-1, 3).cpu().numpy()
    same = bool(np.array_equal(got["id"], ref[:, 0].view(np.uint32)) and np.array_equal(got["t"], ref[:, 1].view(np.float32)))
    ms, sms = min(times), min(sep)
    return {"meshes": len(meshes), "tris": n_tris, "rays": n_rays, "autotuned": best,
            "graph_ms": ms, "graph_mrays_s": n_rays / ms / 1e3, "graph_mtris_s": n_tris / ms / 1e3,
            "separate_launches_ms": sms, "separate_mrays_s": n_rays / sms / 1e3, "speedup": sms / ms,
            "same_hits": same}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-extra", action="store_true", help="skip the comparison legs (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
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
        bvh = ctx.build(src_tris, "morton", wide=True)
        ctx.trace(bvh, "closest", hits=hits, heatmap=heat, **cam)
        return bvh

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
    step_ms, build_ms, wide_ms, trace_ms, stats, launches = [], [], [], [], [], 0
    lbvh_stage = {"codes": [], "sort": [], "topology": []}
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bvh = step(d_tris, d_hits, d_heat)
        e1.record(stream)
        tm = ctx.timings()  # synchronises
        st = ctx.trace_stats()
        step_ms.append(e0.elapsed_time(e1))
        build_ms.append(tm["build"])
        wide_ms.append(tm["wide"])
        for k in lbvh_stage:
            lbvh_stage[k].append(tm[k])
        trace_ms.append(tm["trace"])
        stats.append(st)
        launches += LBVH_KERNELS + bvh.info().wide_launches + 1
        bvh.free()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = reduce_max(sum(step_ms), dist)
    ms_per_step = total_ms / args.steps
    value = whole_job_value(rays_total, args.steps, world, total_ms)

    # end to end through the public API with pinned host buffers
    e2e_ms = []
    if not args.no_e2e:
        h_tris = torch.from_numpy(tris).pin_memory()
        h_hits = torch.empty(rays_total * 3, dtype=torch.int32).pin_memory()
        h_heat = torch.empty(rays_total * 3, dtype=torch.uint8).pin_memory()
        step(h_tris, h_hits, h_heat).free()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            bvh = step(h_tris, h_hits, h_heat)
            torch.cuda.synchronize()
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
            bvh.free()
    e2e_total = reduce_max(sum(e2e_ms) if e2e_ms else float("nan"), dist)
    e2e_value = whole_job_value(rays_total, args.steps, world, e2e_total)

    plain = stress = batch = None
    if not args.no_extra:
        # plain FP32 binary traversal of the same tree, same rays; same hits?
        bvh = ctx.build(d_tris, "morton", wide=True)
        d_hits2 = torch.empty_like(d_hits)
        times = {"wide": [], "binary": []}
        for _ in range(3):
            for form in ("binary", "wide"):
                flush.zero_()
                ctx.trace(bvh, "closest", hits=d_hits if form == "wide" else d_hits2, binary=(form == "binary"), **cam)
                times[form].append(ctx.timings()["trace"])
        same = bool(torch.equal(d_hits.view(-1, 3)[:, :2], d_hits2.view(-1, 3)[:, :2]))
        bvh.free()
        plain = {"trace_ms": min(times["binary"]), "trace_mrays_s": rays_total / min(times["binary"]) / 1e3,
                 "wide_trace_ms": min(times["wide"]), "speedup": min(times["binary"]) / min(times["wide"]),
                 "same_hits": same}
        del d_hits2
        stress = stress_leg(ctx, flush, torch)
        batch = batch_leg(ctx, flush, torch, sq)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peak, peak_kind = measured_peaks()
    tr_ms = statistics.mean(trace_ms)
    req_bytes = statistics.mean(s["bytes"] for s in stats)
    achieved = req_bytes / (tr_ms / 1e3) / 1e9
    b_ms = statistics.mean(build_ms)
    lbvh_ms = b_ms - statistics.mean(wide_ms)
    build_gbs = n * (200 + 16 * 4) / (lbvh_ms / 1e3) / 1e9
    hits_np = d_hits.view(-1, 3).cpu().numpy()

    cpu = None
    if not args.no_cpu_baseline:
        value_c, _, threads, sample = cpu_line(tris, 1, 0)
        cpu = {"value": value_c, "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": sample}

    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded 64-cluster Gaussian triangle soup (no dataset ships with the reference)",
        "config": {"workload": "soup_2m: %d-triangle Gaussian soup, %dx%d pinhole primary rays from (0,0,-40)"
                               % (n, w["width"], w["height"]),
                   "builder": "Morton LBVH + 8-wide 8-bit quantised collapse", "trace": "closest hit + heatmap",
                   "tris": n, "rays": rays_total, "l2": "flushed between steps (512 MB write)",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "build_mtris_s": n / (b_ms / 1e3) / 1e6,
        "lbvh_mtris_s": n / (lbvh_ms / 1e3) / 1e6,
        "trace_mrays_s": rays_total / (tr_ms / 1e3) / 1e6,
        "stage_ms": {"build_total": b_ms, "lbvh": lbvh_ms, "wide_collapse": statistics.mean(wide_ms),
                     "trace": tr_ms, "step": ms_per_step,
                     "lbvh_stages": {k: statistics.mean(v) for k, v in lbvh_stage.items()}},
        "per_ray": {"box_tests": statistics.mean(s["box_tests"] for s in stats) / rays_total,
                    "tri_tests": statistics.mean(s["tri_tests"] for s in stats) / rays_total,
                    "wide_nodes": statistics.mean(s["nodes"] for s in stats) / rays_total,
                    "requested_bytes": req_bytes / rays_total},
        "hit_rays": int((hits_np[:, 0] != -1).sum()),
        "roofline": {"bound": "hbm", "kernel": "k_trace8<closest>", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": TRACE8_DRAM_BYTES, "traffic_source": TRACE8_DRAM_SOURCE,
                     "bytes_model": "kernel-counted requested bytes: 80 B per wide node loaded, 48 B per "
                                    "triangle tested, 15 B of outputs per ray"},
        "build_roofline": {"bound": "hbm", "achieved": build_gbs, "peak": peak, "unit": "GB/s",
                           "frac": build_gbs / peak, "bytes_model": "264 B/tri (200 + 16 x 4 sort passes)"},
        "plain_fp32": plain,
        "stress": stress,
        "batch": batch,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": n * 36,
                "d2h_bytes_per_step": rays_total * 15, "ms_per_step": e2e_total / args.steps},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
