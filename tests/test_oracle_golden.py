"""The CPU oracle against golden outputs of the Sequoia reference itself
(tests/golden, produced by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import load_golden


def canon(nodes, idx, depth=0):
    nd = nodes[idx]
    b = tuple(nd["min"].tolist()) + tuple(nd["max"].tolist())
    if nd["flags"] & 1:
        return ("L", int(nd["child"]), b)
    ch = sorted((canon(nodes, int(nd["child"]) + k, depth + 1) for k in range(int(nd["count"]))), key=repr)
    return ("N", b, tuple(ch))


def test_morton_codes(oracle, golden):
    codes, box = oracle.morton_codes(golden["tris"])
    assert np.array_equal(codes, golden["codes"])
    assert np.array_equal(box, golden["scene"])


def test_radix_sort(oracle, golden):
    n = len(golden["codes"])
    k, v = oracle.sort_pairs(golden["codes"], golden["code_index"])
    assert np.array_equal(k, golden["sorted_codes"])
    assert np.array_equal(v, golden["sorted_index"])
    # the sorted permutation is the unique stable one
    order = np.lexsort((np.arange(n), golden["codes"]))
    assert np.array_equal(v, order.astype(np.uint32))


def test_find_split(oracle, golden):
    sc = golden["sorted_codes"]
    for a, b, s in zip(golden["splits_begin"], golden["splits_end"], golden["splits"]):
        assert oracle.find_split_morton(sc[a:b]) == s


def test_sah_tree_matches_reference(oracle, golden):
    import sys
    sys.setrecursionlimit(100000)
    found = 0
    for bins in (8, 16, 32):
        key = "sah%d_nodes" % bins
        if key not in golden:
            continue
        found += 1
        rn, rroot = golden[key], int(golden["sah%d_root" % bins])
        on, oroot, _ = oracle.build_sah(golden["tris"], bins, 8)
        assert canon(rn, rroot) == canon(on, oroot), bins
    assert found >= 1


def test_grid_tree_matches_reference(oracle, golden):
    import sys
    sys.setrecursionlimit(100000)
    if "grid_nodes" not in golden:
        return
    on, oroot, _ = oracle.build_grid(golden["tris"], 8, 8, scene_bounds_cells=True)
    assert canon(golden["grid_nodes"], int(golden["grid_root"])) == canon(on, oroot)


def test_reference_trace_heatmap(oracle, golden):
    """trace() on the reference's own SAH tree: per-ray test counts, hit
    flags and the heatmap bytes, bit-exact."""
    w, h = int(golden["w"]), int(golden["h"])
    rays = oracle.rays_reference_camera(w, h, golden["cam"])
    nodes, root = golden["sah8_nodes"], int(golden["sah8_root"])
    ids, _, tests = oracle.trace(nodes, root, golden["tris"], rays, 0)
    assert np.array_equal(tests, golden["ref_tests"])
    assert np.array_equal((ids != oracle.NO_HIT).astype(np.uint32), golden["ref_hit"])
    assert np.array_equal(oracle.heatmap(tests), golden["heat"])


def test_oracle_trees_valid(oracle, golden):
    n = len(golden["tris"])
    for build in (lambda t: oracle.build_morton(t)[:2], lambda t: oracle.build_sah(t, 16, 4)[:2],
                  lambda t: oracle.build_grid(t, 8, 8)[:2]):
        nodes, root = build(golden["tris"])
        assert (oracle.leaf_reach(nodes, root, n) == 1).all()


def test_mapped_builders_match_reference(oracle, golden):
    """The drop-in builds the SAH tree for build_hierarchy_horizontal and the
    grid tree with cell nodes bounded by their own triangles for
    build_hierarchy_grid_sse / _grid_m128: the reference's own trees for those
    builders are the same logical trees (where the reference's layout is
    valid)."""
    import sys
    sys.setrecursionlimit(100000)
    checked = 0
    if "horizontal_nodes" in golden:
        on, oroot, _ = oracle.build_sah(golden["tris"], 8, 8)
        assert canon(golden["horizontal_nodes"], int(golden["horizontal_root"])) == canon(on, oroot)
        checked += 1
    for key in ("grid_sse", "grid_avx"):
        if key + "_nodes" in golden:
            on, oroot, _ = oracle.build_grid(golden["tris"], 8, 8, scene_bounds_cells=False)
            assert canon(golden[key + "_nodes"], int(golden[key + "_root"])) == canon(on, oroot)
            checked += 1
    assert checked >= 1


@pytest.mark.parametrize("bundle,k", [(0, 1), (0, 2), (0, 4), (0, 8), (1, 16), (1, 64)])
def test_packet_and_bundle_heatmaps(oracle, golden, bundle, k):
    """trace_packet<k> / trace_bundle<k> (src/tracer.cpp:232-362): the
    oracle's restatement gives the reference's heatmap bytes."""
    w, h = int(golden["w"]), int(golden["h"])
    key = ("bundle%d_heat" if bundle else "packet%d_heat") % k
    got = oracle.trace_coherent(golden["sah8_nodes"], int(golden["sah8_root"]), w, h, golden["cam"], bundle, k)
    assert np.array_equal(got, golden[key])


def test_morton64_codes_sort_split(oracle, golden):
    """The 60-bit path of build_hierarchy_morton2: codes, stable sort and
    find_split_morton2, against the reference's own functions."""
    codes, box = oracle.morton_codes64(golden["tris"])
    assert np.array_equal(codes, golden["codes64"])
    assert np.array_equal(box, golden["scene"])
    k, v = oracle.sort_pairs64(golden["codes64"], np.arange(len(codes), dtype=np.uint32))
    assert np.array_equal(k, golden["sorted_codes64"])
    assert np.array_equal(v, golden["sorted_index64"])
    sc = golden["sorted_codes64"]
    for a, b, s in zip(golden["splits_begin"], golden["splits_end"], golden["splits64"]):
        assert oracle.find_split_morton64(sc[a:b]) == s


def test_morton64_tree_valid(oracle, golden):
    n = len(golden["tris"])
    nodes, root, codes, perm = oracle.build_morton64(golden["tris"])
    assert np.array_equal(codes, golden["sorted_codes64"]) and np.array_equal(perm, golden["sorted_index64"])
    assert (oracle.leaf_reach(nodes, root, n) == 1).all()


def test_heatmap_colour_matches_reference(oracle):
    """The oracle's restatement of get_heatmap_colour (src/tracer.cpp:25-45)
    equals the reference's own function bit for bit on the golden inputs
    (every count / 200 up to 1000, the stops and their float neighbours,
    out-of-range values, seeded uniform values)."""
    g = load_golden("heat_ramp")
    got = oracle.heatmap_colour(g["x"])
    assert np.array_equal(got.view(np.uint32), g["rgb"].view(np.uint32))
    if oracle.ref_available("b8"):
        ref = oracle.ref_heatmap_colour(g["x"], "b8")
        assert np.array_equal(ref.view(np.uint32), g["rgb"].view(np.uint32))
    # the heatmap bytes: black at 0, red from 200 tests on, grey-free ramp
    rgb = oracle.heatmap_ramp(np.array([0, 40, 100, 200, 5000], np.float32)).reshape(-1, 3)
    assert rgb[0].tolist() == [0, 0, 0] and rgb[3].tolist() == [255, 0, 0] and rgb[4].tolist() == [255, 0, 0]
    assert rgb[1].tolist() == [0, 0, 255]  # 40 / 200 = 0.2: the blue stop
