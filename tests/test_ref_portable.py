"""The reference's own code built through the portable intrinsics.

oracle/build_ref.sh compiles the unmodified reference sources against
oracle/x86compat/immintrin.h (a restatement of the x86 intrinsics it uses)
wherever the host is not x86-64.  On an x86-64 host it also builds that way
as variant x8, so this file can check the restatement: every output of the
x8 build must equal the golden outputs recorded from the x86 build with the
compiler's own intrinsics (tests/golden) -- Morton codes (pdep), the sort,
find_split_morton (lzcnt), every builder including grid_sse and grid_avx
(SSE/AVX2 gathers, permutes, masked loads, move masks), and the trace,
packet and bundle heatmaps.  Skipped where the reference was not built.
"""
import numpy as np
import pytest

from conftest import load_golden

NAMES = ["ico3", "ico4", "soup3k", "dups2k"]


@pytest.fixture(scope="module")
def x8(oracle):
    if not oracle.ref_available("x8"):
        pytest.skip("reference sources not present here: the portable-intrinsics build was not made")
    oracle.ref("x8").ref_set_threads(4)
    return "x8"


@pytest.mark.parametrize("name", NAMES)
def test_morton_sort_split(x8, name):
    import oracle as O
    g = load_golden(name)
    codes, index, box = O.ref_setup_morton(g["tris"], x8)
    assert np.array_equal(codes, g["codes"]) and np.array_equal(index, g["code_index"])
    assert np.array_equal(box, g["scene"])
    sc, si = O.ref_radix_sort(codes, index, x8)
    assert np.array_equal(sc, g["sorted_codes"]) and np.array_equal(si, g["sorted_index"])
    for a, b, s in zip(g["splits_begin"], g["splits_end"], g["splits"]):
        assert O.ref_find_split_morton(sc[a:b], x8) == s
    c64, i64, _ = O.ref_setup_morton2(g["tris"], x8)
    assert np.array_equal(c64, g["codes64"])
    s64, si64 = O.ref_radix_sort64(c64, i64, x8)
    assert np.array_equal(s64, g["sorted_codes64"]) and np.array_equal(si64, g["sorted_index64"])
    for a, b, s in zip(g["splits_begin"], g["splits_end"], g["splits64"]):
        assert O.ref_find_split_morton2(s64[a:b], x8) == s


@pytest.mark.parametrize("name", NAMES)
def test_builders(x8, name):
    """Every builder's tree, record for record over what the root reaches
    (node arrays are not zeroed by the reference, so unreached slots hold
    whatever the allocator left; the golden trees were kept only where the
    x86 build's tree is valid)."""
    import sys
    import oracle as O
    from test_oracle_golden import canon
    sys.setrecursionlimit(100000)
    g = load_golden(name)
    pairs = [("sah8", "recursive"), ("grid", "grid"), ("horizontal", "horizontal"), ("grid_sse", "grid_sse"),
             ("grid_avx", "grid_avx")]
    checked = 0
    for key, kind in pairs:
        if key + "_nodes" not in g:
            continue
        nodes, root = O.ref_build(kind, g["tris"], x8)
        want = g[key + "_nodes"]
        assert root == int(g[key + "_root"]), kind
        assert len(nodes) == len(want), kind
        assert canon(nodes, root) == canon(want, root), kind
        checked += 1
    assert checked >= 2


@pytest.mark.parametrize("name", NAMES)
def test_tracers(x8, name):
    """trace(), trace_packet<k>, trace_bundle<k> heatmaps and traverse()'s
    per-ray counts on the reference's own SAH tree."""
    import oracle as O
    g = load_golden(name)
    nodes, root = g["sah8_nodes"], int(g["sah8_root"])
    w, h, cam = int(g["w"]), int(g["h"]), g["cam"]
    assert np.array_equal(O.ref_trace(nodes, root, g["tris"], w, h, cam, 0, x8), g["heat"])
    for k in (1, 2, 4, 8):
        assert np.array_equal(O.ref_trace(nodes, root, g["tris"], w, h, cam, 100 + k, x8), g["packet%d_heat" % k])
    for k in (16, 64):
        assert np.array_equal(O.ref_trace(nodes, root, g["tris"], w, h, cam, 200 + k, x8), g["bundle%d_heat" % k])
    rays = O.rays_reference_camera(w, h, cam)
    hit, tests = O.ref_traverse(nodes, root, g["tris"], rays, x8)
    assert np.array_equal(hit, g["ref_hit"]) and np.array_equal(tests, g["ref_tests"])
