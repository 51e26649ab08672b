"""GPU traversal against the reference's golden heatmaps and the oracle."""
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
