"""GPU LBVH build (Morton codes, onesweep sort, topology + refit) against the
oracle and the reference's golden outputs, through the C ABI."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def bfs(oracle, nodes, root):
    return oracle.canonical_bfs(nodes, root)


def assert_same_tree(oracle, a_nodes, a_root, b_nodes, b_root):
    a = bfs(oracle, a_nodes, a_root)
    b = bfs(oracle, b_nodes, b_root)
    assert len(a) == len(b)
    for f in ("count", "flags", "child"):
        assert np.array_equal(a[f], b[f]), f
    # bounds compare as floats (+0 == -0)
    assert np.array_equal(a["min"], b["min"])
    assert np.array_equal(a["max"], b["max"])


@pytest.mark.parametrize("name", ["ico3", "ico4", "soup3k", "dups2k"])
def test_morton_codes_golden(ctx, name):
    g = load_golden(name)
    codes, box = ctx.morton_codes(g["tris"])
    assert np.array_equal(codes, g["codes"])
    assert np.array_equal(box, g["scene"])


# tile edges of every tile size (4096, 8192 and 16384 keys), and sizes on
# both sides of the switch from one tile per SM to smaller tiles (on a 152-SM
# GB300: 2,490,368 keys for 8-bit digits, 16384 per SM; 2,023,424 for 10-bit
# digits, 13,312 per SM)
@pytest.mark.parametrize("n", [1, 2, 7, 8, 9, 255, 256, 257, 4095, 4096, 4097, 8191, 8192, 8193, 16383, 16384, 16385,
                               100_003, 1_000_000, 2_000_000, 2_023_424, 2_023_425, 2_490_368, 2_490_369, 3_000_017])
@pytest.mark.parametrize("digit_bits", [6, 8, 10])
def test_radix_sort_random(ctx, oracle, n, digit_bits):
    rng = np.random.default_rng(n + digit_bits)
    keys = rng.integers(0, 1 << 30, n, dtype=np.uint32)
    keys[: n // 3] = keys[0]  # many duplicates: stability matters
    vals = np.arange(n, dtype=np.uint32)
    k, v = ctx.radix_sort_pairs(keys, vals, 30, digit_bits)
    ek, ev = oracle.sort_pairs(keys, vals, 30, 8)
    assert np.array_equal(k, ek)
    assert np.array_equal(v, ev)


@pytest.mark.parametrize("n", [1, 255, 256, 257, 511, 512, 513, 77_777, 300_000])
def test_codes_and_tree_from_unaligned_device_triangles(ctx, oracle, n):
    """The bounds and codes kernels stage triangle tiles with bulk copies when
    the array starts on a 16-byte boundary and with plain loads otherwise
    (and for a partial last tile): device triangles at a 16-byte and at a
    4-byte offset give the oracle's codes, scene box and tree."""
    torch = pytest.importorskip("torch")
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(n, 4, seed=n)
    want_codes, _ = oracle.morton_codes(tris)
    onodes, oroot, _, _ = oracle.build_morton(tris)
    want = oracle.canonical_bfs(onodes, oroot)
    flat = torch.from_numpy(tris.reshape(-1)).cuda()
    buf = torch.zeros(flat.numel() + 4, dtype=torch.float32, device="cuda")
    for off in (0, 1, 4):  # 0 and 16 bytes: aligned; 4 bytes: not
        view = buf[off:off + flat.numel()]
        view.copy_(flat)
        codes, _ = ctx.morton_codes(view)
        assert np.array_equal(codes, want_codes), off
        bvh = ctx.build(view, "morton")
        nodes, root = bvh.export_node1()
        got = oracle.canonical_bfs(nodes, root)
        assert len(got) == len(want) and np.array_equal(got["child"], want["child"]), off
        assert np.array_equal(got["min"], want["min"]) and np.array_equal(got["max"], want["max"]), off
        bvh.free()
    assert ctx.sync() == 0


def test_radix_sort_full_32bit(ctx, oracle):
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 1 << 32, 300_001, dtype=np.uint64).astype(np.uint32)
    vals = rng.integers(0, 1 << 32, 300_001, dtype=np.uint64).astype(np.uint32)
    k, v = ctx.radix_sort_pairs(keys, vals, 32, 8)
    ek, ev = oracle.sort_pairs(keys, vals, 32, 8)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


@pytest.mark.parametrize("name", ["ico3", "ico4", "soup3k", "dups2k"])
def test_sorted_golden(ctx, name):
    g = load_golden(name)
    bvh = ctx.build(g["tris"], "morton")
    codes, perm = bvh.export_sorted()
    assert np.array_equal(codes, g["sorted_codes"])
    assert np.array_equal(perm, g["sorted_index"])


def scenes_small():
    from sequoia_gb300 import scenes
    out = {
        "ico3": scenes.displaced_icosphere(3, seed=1),
        "soup5k": scenes.gaussian_soup(5000, 8, seed=3),
        "one": scenes.gaussian_soup(1, 1, seed=4),
        "seven": scenes.gaussian_soup(7, 1, seed=4),
        "eight": scenes.gaussian_soup(8, 1, seed=4),
        "nine": scenes.gaussian_soup(9, 1, seed=4),
    }
    t = scenes.gaussian_soup(3000, 2, seed=9)
    t[:1500] = t[0]            # one run of 1500 equal codes
    out["dup_run"] = t
    t = scenes.gaussian_soup(64, 1, seed=10)
    t[:] = t[0]                # every code equal
    out["all_equal"] = t
    return out


@pytest.mark.parametrize("name", list(scenes_small().keys()))
def test_lbvh_matches_oracle(ctx, oracle, name):
    tris = scenes_small()[name]
    bvh = ctx.build(tris, "morton")
    nodes, root = bvh.export_node1()
    onodes, oroot, ocodes, operm = oracle.build_morton(tris)
    codes, perm = bvh.export_sorted()
    assert np.array_equal(codes, ocodes) and np.array_equal(perm, operm)
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    assert (oracle.leaf_reach(nodes, root, len(tris)) == 1).all()
    assert ctx.sync() == 0


@pytest.mark.parametrize("digit_bits", [6, 8, 10])
def test_lbvh_digit_widths(ctx, oracle, digit_bits):
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(200_000, 16, seed=12)
    bvh = ctx.build(tris, "morton", digit_bits=digit_bits)
    nodes, root = bvh.export_node1()
    onodes, oroot, _, _ = oracle.build_morton(tris)
    assert_same_tree(oracle, nodes, root, onodes, oroot)


def test_lbvh_icosphere_l6(ctx, oracle):
    from sequoia_gb300 import scenes
    tris = scenes.displaced_icosphere(6, seed=1)
    bvh = ctx.build(tris, "morton")
    nodes, root = bvh.export_node1()
    onodes, oroot, _, _ = oracle.build_morton(tris)
    assert_same_tree(oracle, nodes, root, onodes, oroot)


def test_lbvh_soup_2m_full_size(ctx, oracle):
    """The 2M-triangle soup at full size: exact against the oracle."""
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(2_000_000, 64, seed=2)
    bvh = ctx.build(tris, "morton")
    nodes, root = bvh.export_node1()
    onodes, oroot, _, _ = oracle.build_morton(tris)
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    assert (oracle.leaf_reach(nodes, root, len(tris)) == 1).all()


def test_lbvh_device_input(ctx, oracle):
    torch = pytest.importorskip("torch")
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(50_000, 8, seed=13)
    dt = torch.from_numpy(tris).cuda()
    bvh = ctx.build(dt, "morton")
    nodes, root = bvh.export_node1()
    onodes, oroot, _, _ = oracle.build_morton(tris)
    assert_same_tree(oracle, nodes, root, onodes, oroot)


def test_empty_build(ctx):
    bvh = ctx.build(np.zeros((0, 9), np.float32), "morton")
    nodes, root = bvh.export_node1()
    assert nodes[root]["count"] == 0
    hits, _ = ctx.trace(bvh, "closest", rays=np.array([[0, 0, -1, 0, 0, 0, 1, 1e30]], np.float32))
    assert hits["id"][0] == 0xFFFFFFFF


def test_invalid_arguments(ctx):
    import sequoia_gb300 as sq
    with pytest.raises(sq.SequoiaError):
        ctx.build(np.zeros((4, 9), np.float32), "morton", digit_bits=7)
    with pytest.raises(sq.SequoiaError):
        ctx.radix_sort_pairs(np.zeros(4, np.uint32), np.zeros(4, np.uint32), 0, 8)


def test_wide_triangle_limit(ctx):
    """The 8-wide form addresses at most 2^27 triangles (27-bit leaf entries):
    a larger build is refused before the input is looked at.  No buffer comes
    with the request (a null triangle pointer), so the call cannot read
    memory whatever order its checks run in; the handle is cleared."""
    import ctypes as C
    import sequoia_gb300 as sq
    p = sq._BuildParams(sq.BUILDERS["morton"], 8, 8, 8, 0, 2)
    h = C.c_void_p(0x1000)  # not null: the call must clear it
    st = sq.load_library().sq_build(ctx.handle, None, (1 << 27) + 1, C.byref(p), C.byref(h))
    assert st == 5 and not h.value  # SQ_ERR_UNSUPPORTED, no BVH
    # within the limit, a null triangle pointer is an invalid argument
    h = C.c_void_p(0x1000)
    st = sq.load_library().sq_build(ctx.handle, None, 16, C.byref(p), C.byref(h))
    assert st == 1 and not h.value
    assert ctx.sync() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ico3", "ico4", "soup3k", "dups2k"])
def test_morton64_golden(ctx, oracle, name):
    """build_hierarchy_morton2's 60-bit path: sorted codes and permutation
    equal the reference's setup_morton2 + radix_sort<uint64_t>, and the tree
    the oracle's record for record."""
    g = load_golden(name)
    bvh = ctx.build(g["tris"], "morton", morton64=True)
    codes, perm = bvh.export_sorted64()
    assert np.array_equal(codes, g["sorted_codes64"])
    assert np.array_equal(perm, g["sorted_index64"])
    nodes, root = bvh.export_node1()
    onodes, oroot, _, _ = oracle.build_morton64(g["tris"])
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    assert (oracle.leaf_reach(nodes, root, len(g["tris"])) == 1).all()
    assert ctx.sync() == 0


@pytest.mark.gpu
def test_morton64_soup_2m(ctx, oracle):
    """The 2M-triangle soup at full size: 60-bit codes, permutation and every
    record equal the oracle's; the 60-bit tree separates what the 30-bit one
    leaves in runs of equal codes."""
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(2_000_000, 64, seed=2)
    bvh = ctx.build(tris, "morton", morton64=True)
    codes, perm = bvh.export_sorted64()
    onodes, oroot, ocodes, operm = oracle.build_morton64(tris)
    assert np.array_equal(codes, ocodes) and np.array_equal(perm, operm)
    nodes, root = bvh.export_node1()
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    c32, _ = ctx.build(tris, "morton").export_sorted()
    assert len(np.unique(codes)) >= len(np.unique(c32))
