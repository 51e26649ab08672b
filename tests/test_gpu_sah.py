"""GPU binned-SAH and grid builders against the oracle (record for record in
the range-tree layout) and the reference's golden trees (canonical form)."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_lbvh import assert_same_tree

pytestmark = pytest.mark.gpu


def scenes_sah():
    from sequoia_gb300 import scenes
    out = {
        "ico4": scenes.displaced_icosphere(4, seed=1),
        "soup30k": scenes.gaussian_soup(30_000, 8, seed=41),
        "few": scenes.gaussian_soup(5, 1, seed=42),
        "nine": scenes.gaussian_soup(9, 1, seed=43),
        "one": scenes.gaussian_soup(1, 1, seed=44),
    }
    t = scenes.gaussian_soup(4000, 2, seed=45)
    t[:2500] = t[0]            # 2500 coincident centroids: a zero-area leaf of 2500
    out["coincident"] = t
    t = scenes.gaussian_soup(3000, 2, seed=46)
    t[:, 1::3] = 0.0           # a flat scene (all y = 0)
    out["flat"] = t
    return out


@pytest.mark.parametrize("name", list(scenes_sah().keys()))
@pytest.mark.parametrize("bins,leaf", [(8, 8), (16, 4), (32, 4)])
def test_sah_matches_oracle(ctx, oracle, name, bins, leaf):
    tris = scenes_sah()[name]
    bvh = ctx.build(tris, "sah", bins=bins, leaf=leaf)
    nodes, root = bvh.export_node1()
    onodes, oroot, _ = oracle.build_sah(tris, bins, leaf)
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    assert (oracle.leaf_reach(nodes, root, len(tris)) == 1).all()
    assert ctx.sync() == 0


@pytest.mark.parametrize("name", ["ico4", "soup30k", "coincident", "one"])
@pytest.mark.parametrize("scene_box", [False, True])
def test_grid_matches_oracle(ctx, oracle, name, scene_box):
    tris = scenes_sah()[name]
    bvh = ctx.build(tris, "grid", bins=8, leaf=8, flags=1 if scene_box else 0)
    nodes, root = bvh.export_node1()
    onodes, oroot, _ = oracle.build_grid(tris, 8, 8, scene_bounds_cells=scene_box)
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    assert (oracle.leaf_reach(nodes, root, len(tris)) == 1).all()


@pytest.mark.parametrize("name", ["ico3", "ico4", "soup3k", "dups2k"])
def test_sah_matches_reference_golden(ctx, name):
    """Canonical (layout-free) comparison with the reference's own SAH trees."""
    import sys
    sys.setrecursionlimit(100000)
    from test_oracle_golden import canon
    g = load_golden(name)
    for bins in (8, 16, 32):
        key = "sah%d_nodes" % bins
        if key not in g:
            continue
        bvh = ctx.build(g["tris"], "sah", bins=bins, leaf=8)
        nodes, root = bvh.export_node1()
        assert canon(nodes, root) == canon(g[key], int(g["sah%d_root" % bins])), bins
    if "grid_nodes" in g:
        bvh = ctx.build(g["tris"], "grid", bins=8, leaf=8, flags=1)
        nodes, root = bvh.export_node1()
        assert canon(nodes, root) == canon(g["grid_nodes"], int(g["grid_root"]))
    # the builders the C++ drop-in maps onto these (horizontal -> SAH,
    # grid_sse / grid_m128 -> grid with cell nodes bounded by their triangles)
    if "horizontal_nodes" in g:
        bvh = ctx.build(g["tris"], "sah", bins=8, leaf=8)
        nodes, root = bvh.export_node1()
        assert canon(nodes, root) == canon(g["horizontal_nodes"], int(g["horizontal_root"]))
    for key in ("grid_sse", "grid_avx"):
        if key + "_nodes" in g:
            bvh = ctx.build(g["tris"], "grid", bins=8, leaf=8, flags=0)
            nodes, root = bvh.export_node1()
            assert canon(nodes, root) == canon(g[key + "_nodes"], int(g[key + "_root"])), key


def test_sah_soup_2m_32bins(ctx, oracle):
    """The 2M-triangle soup with 32 bins at full size, against the oracle."""
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(2_000_000, 64, seed=2)
    bvh = ctx.build(tris, "sah", bins=32, leaf=4)
    nodes, root = bvh.export_node1()
    onodes, oroot, _ = oracle.build_sah(tris, 32, 4)
    assert_same_tree(oracle, nodes, root, onodes, oroot)


def test_sah_trace_matches_oracle(ctx, oracle):
    from sequoia_gb300 import scenes
    tris = scenes.displaced_icosphere(5, seed=1)
    bvh = ctx.build(tris, "sah", bins=16, leaf=4)
    nodes, root = bvh.export_node1()
    hits, _ = ctx.trace(bvh, "closest", camera="pinhole", width=256, height=192, origin=(0, 0, 3),
                        target=(0, 0, 0), up=(0, 1, 0), vfov=60.0)
    rays = oracle.rays_pinhole(256, 192, (0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0)
    ids, ts, tests = oracle.trace(nodes, root, tris, rays, 1)
    assert np.array_equal(hits["id"], ids)
    assert np.array_equal(hits["t"], ts)
    assert np.array_equal(hits["tests"], tests)
