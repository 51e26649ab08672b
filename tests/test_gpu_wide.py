"""8-wide quantised BVH (precision form) against the FP32 binary traversal
(itself pinned to the oracle) and brute force: identical closest-hit ids and
t, identical any-hit flags."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scenes_wide():
    from sequoia_gb300 import scenes
    return {
        "ico5": scenes.displaced_icosphere(5, seed=1),
        "soup200k": scenes.gaussian_soup(200_000, 16, seed=51),
        "terrain": scenes.heightfield(256, 128, seed=3),
        "tiny": scenes.gaussian_soup(5, 1, seed=52),
    }


def random_rays(tris, n, seed):
    from sequoia_gb300 import scenes
    lo, hi = scenes.scene_box(tris)
    return scenes.random_rays(n, lo, hi, seed=seed)


@pytest.mark.parametrize("name", list(scenes_wide().keys()))
@pytest.mark.parametrize("builder,kw", [("morton", {}), ("sah", dict(bins=16, leaf=4)), ("grid", dict(bins=8, leaf=8))])
def test_wide_matches_binary(ctx, oracle, name, builder, kw):
    tris = scenes_wide()[name]
    bvh = ctx.build(tris, builder, wide=True, **kw)
    assert bvh.info().wide_nodes > 0
    rays = random_rays(tris, 200_000, seed=7)
    h2, _ = ctx.trace(bvh, "closest", rays=rays, binary=True)
    h8, _ = ctx.trace(bvh, "closest", rays=rays)
    assert np.array_equal(h8["id"], h2["id"])
    assert np.array_equal(h8["t"], h2["t"])
    a2, _ = ctx.trace(bvh, "anyhit", rays=rays, binary=True)
    a8, _ = ctx.trace(bvh, "anyhit", rays=rays)
    assert np.array_equal(a8["id"] != 0xFFFFFFFF, a2["id"] != 0xFFFFFFFF)
    # primary rays from outside
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    eye = (float(lo[0] + hi[0]) / 2, float(hi[1]) + 1.0, float(lo[2]) - 2.0)
    p2, _ = ctx.trace(bvh, "closest", camera="pinhole", width=320, height=240, origin=eye, target=(0, 0, 0),
                      up=(0, 1, 0), vfov=60.0, binary=True)
    p8, _ = ctx.trace(bvh, "closest", camera="pinhole", width=320, height=240, origin=eye, target=(0, 0, 0),
                      up=(0, 1, 0), vfov=60.0)
    assert np.array_equal(p8["id"], p2["id"]) and np.array_equal(p8["t"], p2["t"])
    # the binary traversal itself against the oracle, and brute force on a sample
    nodes, root = bvh.export_node1()
    ids, ts, _ = oracle.trace(nodes, root, tris, rays[:20000], 1)
    assert np.array_equal(h2["id"][:20000], ids) and np.array_equal(h2["t"][:20000], ts)
    if len(tris) <= 20000:
        bids, bts = oracle.brute_closest(tris, rays[:5000])
        assert np.array_equal(h8["id"][:5000], bids) and np.array_equal(h8["t"][:5000], bts)
    assert ctx.sync() == 0


def test_wide_terrain_bounce(ctx, oracle):
    """Terrain, primary rays then one cosine-weighted bounce per hit."""
    from sequoia_gb300 import scenes
    tris = scenes.heightfield(512, 256, seed=3)
    bvh = ctx.build(tris, "morton", wide=True)
    w, h = 480, 270
    cam = dict(camera="pinhole", width=w, height=h, origin=(0.0, 0.6, -1.2), target=(0, 0, 0), up=(0, 1, 0), vfov=60.0)
    p2, _ = ctx.trace(bvh, "closest", binary=True, **cam)
    p8, _ = ctx.trace(bvh, "closest", **cam)
    assert np.array_equal(p8["id"], p2["id"]) and np.array_equal(p8["t"], p2["t"])
    rays = oracle.rays_pinhole(w, h, (0.0, 0.6, -1.2), (0, 0, 0), (0, 1, 0), 60.0)
    br, _ = scenes.bounce_rays(tris, rays, p2["id"], p2["t"], seed=3)
    b2, _ = ctx.trace(bvh, "closest", rays=br, binary=True)
    b8, _ = ctx.trace(bvh, "closest", rays=br)
    assert np.array_equal(b8["id"], b2["id"]) and np.array_equal(b8["t"], b2["t"])


@pytest.mark.parametrize("offset,scale", [((1.0e4, -3.0e3, 5.0e3), 0.01), ((-2.5e5, 7.0e4, 1.0e5), 0.5),
                                          ((0.0, 0.0, 0.0), 1.0e-3)])
def test_wide_far_from_origin(ctx, offset, scale):
    """Small geometry far from the origin, rays grazing it from nearby and
    from far away: the slab distances cancel heavily, which is where the
    affine child test's rounding margin matters.  Hits must stay identical to
    the FP32 binary traversal."""
    from sequoia_gb300 import scenes
    base = scenes.displaced_icosphere(4, seed=9).astype(np.float64)
    tris = (base * scale + np.tile(np.asarray(offset, np.float64), 3)).astype(np.float32)
    bvh = ctx.build(tris, "morton", wide=True)
    lo, hi = scenes.scene_box(tris)
    ext = float((hi - lo).max())
    rng = np.random.default_rng(11)
    n = 200_000
    rays = np.zeros((n, 8), np.float32)
    centre = (lo.astype(np.float64) + hi) / 2
    # origins on spheres of radius 0.6 .. 1000 extents, aimed at jittered points of the box
    rad = ext * np.exp(rng.uniform(np.log(0.6), np.log(1000.0), n))
    dirs = rng.standard_normal((n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    org = centre + dirs * rad[:, None]
    aim = centre + (rng.uniform(-0.6, 0.6, (n, 3)) * ext)
    d = aim - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 0:3] = org
    rays[:, 4:7] = d
    rays[:, 7] = 3.4e38
    h2, _ = ctx.trace(bvh, "closest", rays=rays, binary=True)
    h8, _ = ctx.trace(bvh, "closest", rays=rays)
    assert (h2["id"] != 0xFFFFFFFF).sum() > n // 10
    assert np.array_equal(h8["id"], h2["id"])
    assert np.array_equal(h8["t"], h2["t"])
    a2, _ = ctx.trace(bvh, "anyhit", rays=rays, binary=True)
    a8, _ = ctx.trace(bvh, "anyhit", rays=rays)
    assert np.array_equal(a8["id"] != 0xFFFFFFFF, a2["id"] != 0xFFFFFFFF)
    assert ctx.sync() == 0
