"""Batched build + trace (many meshes, one launch sequence, CUDA graph)
against separate per-mesh builds and traces: identical hits and test counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_meshes():
    from sequoia_gb300 import scenes
    rng = np.random.default_rng(77)
    meshes = []
    for i in range(12):
        if i == 3:
            tris = np.zeros((0, 9), np.float32)             # empty mesh
        elif i == 5:
            tris = scenes.gaussian_soup(5, 1, seed=100 + i)  # fewer than 8 triangles
        elif i % 2 == 0:
            tris = scenes.displaced_icosphere(3 + (i % 3), seed=100 + i)
        else:
            tris = scenes.gaussian_soup(int(rng.integers(1000, 40000)), 8, seed=100 + i)
        lo, hi = (tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)) if len(tris) else (np.zeros(3), np.ones(3))
        c = (lo + hi) / 2
        side = int(rng.integers(20, 90))
        if i in (4, 9):
            rays = scenes.random_rays(3000 + 7 * i, lo, hi, seed=200 + i)
            meshes.append(dict(tris=tris, rays=rays))
        else:
            eye = (float(c[0]), float(c[1]), float(lo[2] - 2.0 * (hi[2] - lo[2] + 1.0)))
            meshes.append(dict(tris=tris, camera="pinhole", width=side, height=side + 3, origin=eye,
                               target=tuple(float(x) for x in c), up=(0, 1, 0), vfov=50.0))
    return meshes


def separate(ctx, meshes, mode, wide, builder="morton", **kw):
    out = []
    for m in meshes:
        bvh = ctx.build(m["tris"], builder, wide=wide, **kw)
        if "rays" in m:
            h, _ = ctx.trace(bvh, mode, rays=m["rays"])
        else:
            h, _ = ctx.trace(bvh, mode, camera="pinhole", width=m["width"], height=m["height"], origin=m["origin"],
                             target=m["target"], up=m["up"], vfov=m["vfov"])
        out.append(h)
    return np.concatenate(out)


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("digit_bits", [6, 8, 10])
def test_batch_matches_separate(ctx, wide, graph, digit_bits):
    meshes = make_meshes()
    want = separate(ctx, meshes, "closest", wide)
    b = ctx.batch(meshes, mode="closest", wide=wide, digit_bits=digit_bits, graph=graph)
    assert b.info()["graph"] == graph
    for _ in range(2):  # replays give the same result
        got, _ = b.run()
        assert np.array_equal(got["id"], want["id"])
        assert np.array_equal(got["t"], want["t"])
        assert np.array_equal(got["tests"], want["tests"])
    assert ctx.sync() == 0
    b.free()


def test_batch_anyhit_and_ref(ctx):
    meshes = make_meshes()
    for mode in ("anyhit", "ref"):
        want = separate(ctx, meshes, mode, False)
        got, _ = ctx.batch(meshes, mode=mode, wide=False).run()
        if mode == "ref":
            assert np.array_equal(got["tests"], want["tests"])
        assert np.array_equal(got["id"] != 0xFFFFFFFF, want["id"] != 0xFFFFFFFF)


def test_batch_autotune_and_cache(ctx, tmp_path):
    meshes = make_meshes()
    want = separate(ctx, meshes, "closest", False)
    b = ctx.batch(meshes, mode="closest", wide=False)
    cache = str(tmp_path / "tune.jsonl")
    best, ms = b.autotune(cache)
    assert best["sort_digit_bits"] in (6, 8, 10) and best["wide"] in (0, 1) and best["block_threads"] in (64, 128, 256)
    assert ms > 0
    got, _ = b.run()
    assert np.array_equal(got["id"], want["id"]) and np.array_equal(got["t"], want["t"])
    lines = open(cache).read().strip().splitlines()
    assert len(lines) == 1
    best2, ms2 = ctx.batch(meshes, mode="closest", wide=False).autotune(cache)  # served from the cache
    assert best2 == best
    assert len(open(cache).read().strip().splitlines()) == 1


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("bins,leaf", [(8, 8), (16, 4), (32, 8)])
def test_sah_batch_matches_separate(ctx, wide, graph, bins, leaf):
    """SAH batches (one launch sequence, no host round trip, CUDA graph):
    every mesh's hits and box-test counts equal a separate SAH build of that
    mesh with the same bins and leaf size, so the trees are the same."""
    meshes = make_meshes()
    want = separate(ctx, meshes, "closest", wide, "sah", bins=bins, leaf=leaf)
    b = ctx.batch(meshes, mode="closest", wide=wide, graph=graph, builder="sah", bins=bins, leaf=leaf)
    assert b.info()["graph"] == graph and b.info()["sah_bins"] == bins
    for _ in range(2):
        got, _ = b.run()
        assert np.array_equal(got["id"], want["id"])
        assert np.array_equal(got["t"], want["t"])
        assert np.array_equal(got["tests"], want["tests"])
    assert ctx.sync() == 0
    b.free()


def large_depth(nodes, root, large=128):
    """Depth of the deepest inner record over more than `large` triangles
    (the root at depth 0) in a Node1 tree."""
    order, depth = [root], {root: 0}
    i = 0
    while i < len(order):
        nd = nodes[order[i]]
        i += 1
        if not (nd["flags"] & 1):
            for c in range(int(nd["child"]), int(nd["child"]) + int(nd["count"])):
                depth[c] = depth[order[i - 1]] + 1
                order.append(c)
    size = {}
    for k in reversed(order):
        nd = nodes[k]
        size[k] = 1 if nd["flags"] & 1 else sum(size[c] for c in range(int(nd["child"]),
                                                                       int(nd["child"]) + int(nd["count"])))
    return max((depth[k] for k in order if not (nodes[k]["flags"] & 1) and size[k] > large), default=0)


def test_sah_batch_deep_meshes(ctx):
    """Meshes whose SAH trees need more large-phase levels than the batch
    build runs (long chains of uneven splits): the rest is finished by the
    small phase, with the same trees as separate builds."""
    from sequoia_gb300 import scenes
    meshes = []
    for i in range(3):
        t = scenes.gaussian_soup(150_000, 1, seed=300 + i)
        # a geometric spread along x: every SAH split peels off a thin slab
        t = t.astype(np.float64)
        t[:, 0::3] = np.sign(t[:, 0::3]) * np.exp(np.abs(t[:, 0::3]) * 3.0)
        t = t.astype(np.float32)
        lo, hi = t.reshape(-1, 3).min(0), t.reshape(-1, 3).max(0)
        meshes.append(dict(tris=t, rays=scenes.random_rays(20_000, lo, hi, seed=400 + i)))
    # at least one tree has inner nodes of more than 128 triangles deeper
    # than the batch build's 24 large-phase levels
    deepest = max(large_depth(*ctx.build(m["tris"], "sah", bins=8, leaf=4).export_node1()) for m in meshes)
    assert deepest >= 24, deepest
    want = separate(ctx, meshes, "closest", False, "sah", bins=8, leaf=4)
    got, _ = ctx.batch(meshes, mode="closest", wide=False, builder="sah", bins=8, leaf=4).run()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert ctx.sync() == 0


def test_sah_batch_autotune(ctx, tmp_path):
    """The autotuner sweeps the SAH bin count for SAH batches; closest-hit
    ids and t do not depend on it."""
    meshes = make_meshes()
    want = separate(ctx, meshes, "closest", False, "sah", bins=8, leaf=8)
    b = ctx.batch(meshes, mode="closest", wide=False, builder="sah")
    best, ms = b.autotune(str(tmp_path / "tune.jsonl"))
    assert best["sah_bins"] in (8, 16, 32) and "sort_digit_bits" not in best and ms > 0
    got, _ = b.run()
    assert np.array_equal(got["id"], want["id"]) and np.array_equal(got["t"], want["t"])
    with pytest.raises(Exception):
        ctx.batch(meshes, builder="grid")
