"""GPU traversal against the reference's golden heatmaps and the oracle."""
import os

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["ico3", "ico4", "soup3k", "dups2k"])
def test_reference_tree_heatmap_golden(ctx, name):
    """The reference's own SAH tree, uploaded unchanged and traced on the GPU
    with the reference's camera: heatmap bytes identical to trace()."""
    g = load_golden(name)
    bvh = ctx.import_node1(g["sah8_nodes"], int(g["sah8_root"]), g["tris"])
    w, h = int(g["w"]), int(g["h"])
    hits, heat = ctx.trace(bvh, "ref", camera="reference", width=w, height=h, origin=g["cam"], heatmap=True)
    assert np.array_equal(heat, g["heat"])
    assert np.array_equal(hits["tests"], g["ref_tests"])
    assert np.array_equal((hits["id"] != 0xFFFFFFFF).astype(np.uint32), g["ref_hit"])


def test_drop_in_trace(lib_built):
    """The reference-named interface: trace(hierarchy, w, h, origin)."""
    import sequoia_gb300 as sq
    g = load_golden("ico4")
    hier = sq.Hierarchy(g["sah8_nodes"], int(g["sah8_root"]), g["tris"])
    heat = sq.trace(hier, int(g["w"]), int(g["h"]), g["cam"])
    assert np.array_equal(heat, g["heat"])


def scenes_for_trace():
    from sequoia_gb300 import scenes
    return {
        "ico4": scenes.displaced_icosphere(4, seed=1),
        "soup20k": scenes.gaussian_soup(20_000, 8, seed=21),
    }


@pytest.mark.parametrize("name", ["ico4", "soup20k"])
@pytest.mark.parametrize("mode", ["ref", "closest", "anyhit"])
def test_trace_matches_oracle_pinhole(ctx, oracle, name, mode):
    tris = scenes_for_trace()[name]
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    eye = (0.0, 0.0, float(lo[2]) - 2.0 * float(hi[2] - lo[2]))
    w, h = 320, 200
    bvh = ctx.build(tris, "morton")
    nodes, root = bvh.export_node1()
    hits, heat = ctx.trace(bvh, mode, camera="pinhole", width=w, height=h, origin=eye, target=(0, 0, 0),
                           up=(0, 1, 0), vfov=60.0, heatmap=True)
    rays = oracle.rays_pinhole(w, h, eye, (0, 0, 0), (0, 1, 0), 60.0)
    m = {"ref": 0, "closest": 1, "anyhit": 2}[mode]
    ids, ts, tests = oracle.trace(nodes, root, tris, rays, m)
    assert np.array_equal(hits["id"], ids)
    assert np.array_equal(hits["tests"], tests)
    assert np.array_equal(hits["t"], ts)
    assert np.array_equal(heat, oracle.heatmap(tests))
    if mode == "closest":
        bids, bts = oracle.brute_closest(tris, rays[::7])
        assert np.array_equal(hits["id"][::7], bids)


def test_trace_explicit_random_rays(ctx, oracle):
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(50_000, 16, seed=31)
    lo, hi = scenes.scene_box(tris)
    rays = scenes.random_rays(100_000, lo, hi, seed=32)
    bvh = ctx.build(tris, "morton")
    nodes, root = bvh.export_node1()
    for mode, m in (("closest", 1), ("anyhit", 2), ("ref", 0)):
        hits, _ = ctx.trace(bvh, mode, rays=rays)
        ids, ts, tests = oracle.trace(nodes, root, tris, rays, m)
        assert np.array_equal(hits["id"], ids), mode
        assert np.array_equal(hits["tests"], tests), mode
        assert np.array_equal(hits["t"], ts), mode
    bids, bts = oracle.brute_closest(tris, rays[:2000])
    hits, _ = ctx.trace(bvh, "closest", rays=rays[:2000].copy())
    assert np.array_equal(hits["id"], bids)
    assert np.array_equal(hits["t"], bts)


def test_trace_into_pinned_host_buffers(ctx):
    """Page-locked host outputs are written by the kernel in place; the
    results equal those written to pageable host arrays (through a copy)."""
    torch = pytest.importorskip("torch")
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(200_000, 16, seed=33)
    lo, hi = scenes.scene_box(tris)
    rays = scenes.random_rays(60_000, lo, hi, seed=34)
    for wide in (False, True):
        bvh = ctx.build(tris, "morton", wide=wide)
        for kw in (dict(rays=rays), dict(camera="pinhole", width=320, height=200, origin=(0, 0, -40), target=(0, 0, 0))):
            ref_hits, ref_heat = ctx.trace(bvh, "closest", heatmap=True, **kw)
            count = len(ref_hits)
            p_hits = torch.zeros(count * 3, dtype=torch.int32).pin_memory()
            p_heat = torch.zeros(count * 3, dtype=torch.uint8).pin_memory()
            ctx.trace(bvh, "closest", hits=p_hits, heatmap=p_heat, **kw)
            assert np.array_equal(p_hits.numpy().view(np.uint8), ref_hits.view(np.uint8))
            assert np.array_equal(p_heat.numpy(), ref_heat)


def test_banded_trace_into_pinned_host_buffers(ctx):
    """A camera image of 2^21 rays or more with page-locked host outputs on
    the 8-wide tree is traced in row bands whose results are copied to the
    host while later bands trace.  Every combination of pinned and device
    outputs gives the bytes a single trace into device buffers gives, on an
    image whose width and height are not multiples of the 8x4 tile."""
    torch = pytest.importorskip("torch")
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(300_000, 16, seed=35)
    bvh = ctx.build(tris, "morton", wide=True)
    cam = dict(camera="pinhole", width=2050, height=1031, origin=(0.0, 1.0, -40.0), target=(0, 0, 0), vfov=45.0)
    count = 2050 * 1031
    assert count >= 1 << 21
    d_hits = torch.zeros(count * 3, dtype=torch.int32, device="cuda")
    d_heat = torch.zeros(count * 3, dtype=torch.uint8, device="cuda")
    ctx.trace(bvh, "closest", hits=d_hits, heatmap=d_heat, **cam)
    ctx.sync()
    want_hits, want_heat = d_hits.cpu().numpy(), d_heat.cpu().numpy()
    assert (want_hits.reshape(-1, 3)[:, 0] != -1).sum() > 0
    for pin_hits, pin_heat in ((True, True), (True, False), (False, True)):
        h = torch.full((count * 3,), 7, dtype=torch.int32)
        m = torch.full((count * 3,), 7, dtype=torch.uint8)
        h = h.pin_memory() if pin_hits else h.cuda()
        m = m.pin_memory() if pin_heat else m.cuda()
        ctx.trace(bvh, "closest", hits=h, heatmap=m, **cam)
        ctx.sync()
        assert np.array_equal(h.cpu().numpy(), want_hits), (pin_hits, pin_heat)
        assert np.array_equal(m.cpu().numpy(), want_heat), (pin_hits, pin_heat)
    # hits only, and the colour ramp, pinned
    h = torch.zeros(count * 3, dtype=torch.int32).pin_memory()
    ctx.trace(bvh, "closest", hits=h, **cam)
    assert np.array_equal(h.numpy(), want_hits)
    ramp_d = torch.zeros(count * 3, dtype=torch.uint8, device="cuda")
    ctx.trace(bvh, "closest", hits=False, heatmap=ramp_d, ramp=True, **cam)
    ctx.sync()
    ramp_p = torch.zeros(count * 3, dtype=torch.uint8).pin_memory()
    ctx.trace(bvh, "closest", hits=False, heatmap=ramp_p, ramp=True, **cam)
    assert np.array_equal(ramp_p.numpy(), ramp_d.cpu().numpy())
    assert ctx.sync() == 0


def test_closest_t_vs_fp64(ctx, oracle):
    """Closest-hit t is bit-identical to the oracle (so within any relative
    tolerance of it, 1e-6 included); its error against an FP64 re-intersection
    of the same (ray, triangle) is stated: printed, and bounded loosely at
    1e-5 relative (the watertight test's shear adds a few ulp)."""
    from sequoia_gb300 import scenes
    tris = scenes.displaced_icosphere(5, seed=1)
    w, h = 256, 256
    bvh = ctx.build(tris, "morton")
    hits, _ = ctx.trace(bvh, "closest", camera="pinhole", width=w, height=h, origin=(0, 0, 3), target=(0, 0, 0),
                        up=(0, 1, 0), vfov=60.0)
    rays = oracle.rays_pinhole(w, h, (0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0)
    nodes, root = bvh.export_node1()
    ids, ts, _ = oracle.trace(nodes, root, tris, rays, 1)
    assert np.array_equal(hits["id"], ids)
    m = hits["id"] != 0xFFFFFFFF
    rel_oracle = np.abs(hits["t"][m].astype(np.float64) - ts[m]) / np.abs(ts[m])
    assert rel_oracle.max() <= 1e-6
    t64 = oracle.reintersect_f64(tris, rays, hits["id"])
    rel = np.abs(hits["t"][m].astype(np.float64) - t64[m]) / np.abs(t64[m])
    print("t error vs FP64 re-intersection: max %.3g, mean %.3g relative over %d hits" % (rel.max(), rel.mean(), m.sum()))
    assert rel.max() < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ico3", "ico4", "soup3k", "dups2k"])
@pytest.mark.parametrize("mode,k", [("packet", 1), ("packet", 2), ("packet", 4), ("packet", 8),
                                    ("bundle", 16), ("bundle", 64)])
def test_packet_bundle_heatmap_golden(ctx, name, mode, k):
    """trace_packet<k> / trace_bundle<k> on the reference's own SAH tree: the
    reference's heatmap bytes (tests/golden)."""
    from conftest import load_golden
    g = load_golden(name)
    w, h = int(g["w"]), int(g["h"])
    bvh = ctx.import_node1(g["sah8_nodes"], int(g["sah8_root"]), g["tris"])
    _, heat = ctx.trace(bvh, mode, k=k, camera="reference", width=w, height=h, origin=g["cam"])
    assert np.array_equal(heat, g["%s%d_heat" % (mode, k)])
    assert ctx.sync() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode,k", [("packet", 8), ("bundle", 64), ("bundle", 16), ("packet", 2)])
def test_packet_bundle_matches_oracle_large(ctx, oracle, mode, k):
    """A GPU-built SAH tree of the level-6 icosphere at 640x480, against the
    oracle's restatement of the reference's packet / bundle tracers."""
    from sequoia_gb300 import scenes
    tris = scenes.displaced_icosphere(6, seed=1)
    bvh = ctx.build(tris, "sah", bins=8, leaf=8)
    nodes, root = bvh.export_node1()
    lo, hi = scenes.scene_box(tris)
    c = (lo + hi) * np.float32(0.5)
    cam = np.array([c[0], c[1], np.float32(2) * lo[2] - c[2]], np.float32)
    w, h = 640, 480
    _, heat = ctx.trace(bvh, mode, k=k, camera="reference", width=w, height=h, origin=cam)
    want = oracle.trace_coherent(nodes, root, w, h, cam, mode == "bundle", k)
    assert np.array_equal(heat, want)


@pytest.mark.gpu
def test_packet_bundle_argument_checks(ctx):
    import sequoia_gb300 as sq
    from sequoia_gb300 import scenes
    tris = scenes.displaced_icosphere(3, seed=1)
    bvh = ctx.build(tris, "sah")
    for mode, k, w, h in (("packet", 3, 64, 64), ("packet", 8, 63, 64), ("bundle", 64, 64, 60), ("bundle", 8, 64, 64)):
        with pytest.raises(sq.SequoiaError):
            ctx.trace(bvh, mode, k=k, camera="reference", width=w, height=h, origin=(0, 0, -3))


@pytest.mark.gpu
def test_heatmap_colour_ramp(ctx, oracle):
    """SQ_TRACE_HEAT_RAMP: heatmap pixels in the reference's colour ramp
    (get_heatmap_colour, src/tracer.cpp:25-45) of the same box-test counts,
    byte for byte the oracle's, for the reference tracer on the reference's
    own tree and for closest hit on both tree forms."""
    from conftest import load_golden
    g = load_golden("ico4")
    w, h = int(g["w"]), int(g["h"])
    bvh = ctx.import_node1(g["sah8_nodes"], int(g["sah8_root"]), g["tris"])
    hits, heat = ctx.trace(bvh, "ref", camera="reference", width=w, height=h, origin=g["cam"], heatmap=True,
                           ramp=True)
    assert np.array_equal(hits["tests"], g["ref_tests"])
    assert np.array_equal(heat, oracle.heatmap_ramp(g["ref_tests"].astype(np.float32)))
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(200_000, 16, seed=91)
    wbvh = ctx.build(tris, "morton", wide=True)
    cam = dict(camera="pinhole", width=320, height=200, origin=(0, 0, -40), target=(0, 0, 0))
    for binary in (True, False):
        hh, hm = ctx.trace(wbvh, "closest", heatmap=True, ramp=True, binary=binary, **cam)
        assert np.array_equal(hm, oracle.heatmap_ramp(hh["tests"].astype(np.float32)))
        # the grey heatmap of the same counts is unchanged
        _, grey = ctx.trace(wbvh, "closest", heatmap=True, binary=binary, **cam)
        assert np.array_equal(grey, oracle.heatmap(hh["tests"]))
    assert ctx.sync() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ico3", "soup3k"])
def test_traverse_node_groups(ctx, name):
    """sq_traverse (traverse(), src/tracer.cpp:47-65) on the reference's own
    SAH tree: from (root, 1) it gives the reference's per-ray counts and hit
    flags (tests/golden); from a node group it gives the sum of the counts
    and the OR of the hits of its nodes taken one by one, and from the root's
    child group exactly the root's counts minus the root's own test."""
    from conftest import load_golden
    import oracle as O
    g = load_golden(name)
    nodes, root = g["sah8_nodes"], int(g["sah8_root"])
    bvh = ctx.import_node1(nodes, root, g["tris"])
    rays = O.rays_reference_camera(int(g["w"]), int(g["h"]), g["cam"])
    h = ctx.traverse(bvh, root, 1, rays)
    assert np.array_equal(h["tests"], g["ref_tests"])
    assert np.array_equal((h["id"] == 0).astype(np.uint32), g["ref_hit"])
    first, count = int(nodes[root]["child"]), int(nodes[root]["count"])
    grp = ctx.traverse(bvh, first, count, rays)
    singles = [ctx.traverse(bvh, first + j, 1, rays) for j in range(count)]
    assert np.array_equal(grp["tests"], sum(s["tests"] for s in singles))
    hit_any = np.zeros(len(rays), bool)
    for s in singles:
        hit_any |= s["id"] == 0
    assert np.array_equal(grp["id"] == 0, hit_any)
    root_hit = h["tests"] > 1
    assert np.array_equal(h["tests"][root_hit], 1 + grp["tests"][root_hit])
    import sequoia_gb300 as sq
    with pytest.raises(sq.SequoiaError):
        ctx.traverse(bvh, len(nodes) - 1, 2, rays)  # a group past the node array
    assert ctx.sync() == 0


@pytest.mark.gpu
def test_drop_in_traverse(lib_built, tmp_path, oracle):
    """The C++ drop-in's traverse() (single ray and many rays) on a tree from
    Builder::build_hierarchy: the oracle's reference-mode counts and hit
    flags on the same tree; attributes accumulate over calls."""
    import subprocess
    from conftest import ROOT
    from sequoia_gb300 import scenes
    tris = scenes.displaced_icosphere(4, seed=1)
    lo, hi = scenes.scene_box(tris)
    rays = scenes.random_rays(5000, lo, hi, seed=19)
    rays[:, 7] = 1e4
    (tmp_path / "tris.bin").write_bytes(tris.tobytes())
    (tmp_path / "rays.bin").write_bytes(rays.tobytes())
    exe = str(tmp_path / "drop_in_traverse")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "sequoia_gb300", "host")]
    lib = os.path.join(ROOT, "sequoia_gb300")
    subprocess.run(["g++", "-std=c++17", "-O1", *inc, os.path.join(ROOT, "tests", "drop_in_traverse.cpp"), "-o", exe,
                    "-L" + lib, "-lsequoia_gpu", "-Wl,-rpath," + lib], check=True)
    subprocess.run([exe, str(tmp_path / "tris.bin"), str(tmp_path / "rays.bin"), str(tmp_path / "out.bin")],
                   check=True, timeout=300)
    out = np.fromfile(str(tmp_path / "out.bin"), np.int32).reshape(-1, 2)
    one, many, twice = out[:64], out[64:64 + len(rays)], out[64 + len(rays):]
    nodes, root, _ = oracle.build_sah(tris, 8, 8)
    _, _, tests = oracle.trace(nodes, root, tris, rays, 0)
    rids, _, _ = oracle.trace(nodes, root, tris, rays, 0)
    assert np.array_equal(many[:, 1], tests.astype(np.int32))
    assert np.array_equal(many[:, 0], np.where(rids != 0xFFFFFFFF, -1, 0))
    assert np.array_equal(one, many[:64])
    assert np.array_equal(twice[:, 1], 2 * one[:, 1]) and np.array_equal(twice[:, 0], one[:, 0])
