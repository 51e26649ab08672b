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


def separate(ctx, meshes, mode, wide):
    out = []
    for m in meshes:
        bvh = ctx.build(m["tris"], "morton", wide=wide)
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
