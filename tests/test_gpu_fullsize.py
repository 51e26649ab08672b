"""Parity at the full sizes of the benchmark configurations.

Each case builds on the GPU at the configuration's full size, traces the
configuration's rays on the GPU, and compares them ray by ray with the
oracle's closest-hit traversal of the same GPU-built tree (exported in the
reference's Node1 layout): hit id, t, box-test count and heatmap bytes must
be identical.  The tree itself is compared with the oracle's build where the
configuration names a builder.  The 8-wide quantised form must give the same
ids and t as the binary tree on every ray.  The t error of each hit against
an FP64 re-intersection of the same (ray, triangle) is printed and bounded;
the GPU's t equals the oracle's bit for bit, so it is within 1e-6 relative
of it by construction, and its FP64 error is no larger than that of the
reference's own FP32 Moller-Trumbore t on the same hits.

Configurations (seeded synthetic scenes of the stated shapes and sizes):

  icosphere_l6  81,920-triangle displaced icosphere; binned SAH at 16 bins,
                leaf <= 4, and Morton; 1920x1080 pinhole rays from distance 3.
  soup_2m       2,000,000-triangle 64-cluster Gaussian soup; Morton (all
                8,294,400 rays of 3840x2160), SAH at 32 bins and the grid
                builder (every 4th row and column).
  terrain_4m    2048x1024-quad height field (4,194,304 triangles); 1920x1080
                primary rays plus one cosine-weighted bounce per hit.
  stress_8m     8,000,000-triangle 256-cluster soup; 2^24 incoherent rays
                (wide against binary on all of them, the oracle on a sample).
"""
import numpy as np
import pytest

from test_gpu_lbvh import assert_same_tree

pytestmark = pytest.mark.gpu

NO_HIT = 0xFFFFFFFF
# bound on the relative t error against the FP64 re-intersection: the
# watertight test's shear and scaling round a few times, so t is a few ulp
# (2^-23 each) from the exact intersection of the float inputs
T_FP64_BOUND = 1e-5


def cam_rays(oracle, cfg, step=1):
    """The configuration's pinhole rays (one per pixel centre), every
    `step`-th row and column, with their pixel indices."""
    w, h = cfg["width"], cfg["height"]
    rays = oracle.rays_pinhole(w, h, cfg["eye"], cfg["target"], cfg["up"], cfg["vfov"])
    if step == 1:
        return rays, np.arange(w * h)
    ys, xs = np.meshgrid(np.arange(0, h, step), np.arange(0, w, step), indexing="ij")
    pix = (ys * w + xs).ravel()
    return rays[pix], pix


def cam_kw(cfg):
    return dict(camera="pinhole", width=cfg["width"], height=cfg["height"], origin=cfg["eye"],
                target=cfg["target"], up=cfg["up"], vfov=cfg["vfov"])


def assert_same_hits(hits, ids, ts, tests=None, what=""):
    bad = np.nonzero(hits["id"] != ids)[0]
    assert len(bad) == 0, "%s: %d rays differ in id, first %s" % (what, len(bad), bad[:5])
    assert np.array_equal(hits["t"].view(np.uint32), ts.view(np.uint32)), what + ": t"
    if tests is not None:
        assert np.array_equal(hits["tests"], tests), what + ": box-test counts"


def moller_trumbore_t(tris, rays, ids):
    """t of the reference's FP32 Moller-Trumbore formula (src/tracer.h:94-111:
    edge1, edge2, h = d x edge2, a = edge1 . h, f = 1/a, s = o - v0,
    q = s x edge1, t = f * (edge2 . q)), one rounding per operation, for
    stating how far the reference's own arithmetic is from FP64."""
    f32 = np.float32
    v = tris[ids].reshape(-1, 3, 3).astype(f32)
    o, d = rays[:, 0:3].astype(f32), rays[:, 4:7].astype(f32)

    def cross(a, b):
        return np.stack([a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2], a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0],
                         a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]], 1)

    def dot(a, b):
        return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]

    e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    a = dot(e1, cross(d, e2))
    q = cross(o - v[:, 0], e1)
    return (f32(1) / a) * dot(e2, q)


def fp64_error(oracle, tris, rays, hits, label):
    """Relative |t - t64| / |t64| of every hit against the FP64
    re-intersection of the same (ray, triangle), beside the same error of
    the reference's FP32 Moller-Trumbore t on those hits; printed, and
    returned as (max, mean, reference formula's max)."""
    m = hits["id"] != NO_HIT
    t64 = oracle.reintersect_f64(tris, rays[m], hits["id"][m])
    rel = np.abs(hits["t"][m].astype(np.float64) - t64) / np.abs(t64)
    mt = moller_trumbore_t(tris, rays[m], hits["id"][m]).astype(np.float64)
    rel_mt = np.abs(mt - t64) / np.abs(t64)
    print("%s: t error vs FP64 re-intersection: max %.3g, mean %.3g relative over %d hits "
          "(the reference's FP32 Moller-Trumbore t on the same hits: max %.3g, mean %.3g)"
          % (label, rel.max(), rel.mean(), int(m.sum()), rel_mt.max(), rel_mt.mean()))
    return float(rel.max()), float(rel.mean()), float(rel_mt.max())


def test_icosphere_l6_sah16_leaf4(ctx, oracle):
    """icosphere_l6: the SAH tree (16 bins, leaf <= 4) equals the oracle's;
    every one of the 2,073,600 rays gives the oracle's id, t, box-test count
    and heatmap byte on it; the 8-wide form gives the same ids and t; the
    Morton tree is traced the same way."""
    from sequoia_gb300 import scenes
    cfg = scenes.CONFIGS["icosphere_l6"]
    tris = scenes.displaced_icosphere(6, seed=1)
    assert len(tris) == 81_920
    rays, _ = cam_rays(oracle, cfg)
    for builder, kw in (("sah", dict(bins=16, leaf=4)), ("morton", {})):
        bvh = ctx.build(tris, builder, wide=True, **kw)
        nodes, root = bvh.export_node1()
        if builder == "sah":
            onodes, oroot, _ = oracle.build_sah(tris, 16, 4)
        else:
            onodes, oroot, _, _ = oracle.build_morton(tris)
        assert_same_tree(oracle, nodes, root, onodes, oroot)
        hits, heat = ctx.trace(bvh, "closest", heatmap=True, binary=True, **cam_kw(cfg))
        ids, ts, tests = oracle.trace(nodes, root, tris, rays, 1)
        assert_same_hits(hits, ids, ts, tests, builder)
        assert np.array_equal(heat, oracle.heatmap(tests))
        wide, _ = ctx.trace(bvh, "closest", **cam_kw(cfg))
        assert_same_hits(wide, ids, ts, None, builder + " 8-wide")
        assert (ids != NO_HIT).sum() > len(rays) // 10
        mx, _, mx_ref = fp64_error(oracle, tris, rays, hits, "icosphere_l6 " + builder)
        assert mx < T_FP64_BOUND and mx <= mx_ref
        bvh.free()
    assert ctx.sync() == 0


@pytest.fixture(scope="module")
def soup_2m():
    from sequoia_gb300 import scenes
    return scenes.gaussian_soup(2_000_000, 64, seed=2)


def test_soup_2m_morton_every_ray(ctx, oracle, soup_2m):
    """soup_2m as the benchmark runs it (Morton LBVH, 8-wide collapse,
    3840x2160): all 8,294,400 rays against the oracle on the binary tree,
    the 8-wide form against both."""
    from sequoia_gb300 import scenes
    cfg = scenes.CONFIGS["soup_2m"]
    tris = soup_2m
    bvh = ctx.build(tris, "morton", wide=True)
    nodes, root = bvh.export_node1()
    rays, _ = cam_rays(oracle, cfg)
    hits, heat = ctx.trace(bvh, "closest", heatmap=True, binary=True, **cam_kw(cfg))
    ids, ts, tests = oracle.trace(nodes, root, tris, rays, 1)
    assert_same_hits(hits, ids, ts, tests, "binary")
    assert np.array_equal(heat, oracle.heatmap(tests))
    wide, _ = ctx.trace(bvh, "closest", **cam_kw(cfg))
    assert_same_hits(wide, ids, ts, None, "8-wide")
    assert (ids != NO_HIT).sum() > len(rays) // 20
    mx, _, mx_ref = fp64_error(oracle, tris, rays, hits, "soup_2m morton")
    assert mx < T_FP64_BOUND and mx <= mx_ref
    bvh.free()
    assert ctx.sync() == 0


@pytest.mark.parametrize("builder,kw", [("sah", dict(bins=32, leaf=8)), ("grid", dict(bins=8, leaf=8))])
def test_soup_2m_sah_grid_sampled(ctx, oracle, soup_2m, builder, kw):
    """soup_2m's other builders: the tree equals the oracle's (SAH at 32
    bins, the grid builder), and the rays of every 4th row and column
    (518,400) give the oracle's hits and counts; the 8-wide form agrees on
    all 8,294,400."""
    from sequoia_gb300 import scenes
    cfg = scenes.CONFIGS["soup_2m"]
    tris = soup_2m
    bvh = ctx.build(tris, builder, wide=True, **kw)
    nodes, root = bvh.export_node1()
    if builder == "sah":
        onodes, oroot, _ = oracle.build_sah(tris, kw["bins"], kw["leaf"])
    else:
        onodes, oroot, _ = oracle.build_grid(tris, kw["bins"], kw["leaf"])
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    hits, heat = ctx.trace(bvh, "closest", heatmap=True, binary=True, **cam_kw(cfg))
    rays, pix = cam_rays(oracle, cfg, step=4)
    assert len(pix) == 518_400
    ids, ts, tests = oracle.trace(nodes, root, tris, rays, 1)
    assert_same_hits(hits[pix], ids, ts, tests, builder)
    assert np.array_equal(heat.reshape(-1, 3)[pix].ravel(), oracle.heatmap(tests))
    wide, _ = ctx.trace(bvh, "closest", **cam_kw(cfg))
    assert np.array_equal(wide["id"], hits["id"]) and np.array_equal(wide["t"], hits["t"])
    bvh.free()
    assert ctx.sync() == 0


def test_terrain_4m_primary_and_bounce(ctx, oracle):
    """terrain_4m: the Morton tree of all 4,194,304 triangles equals the
    oracle's; all 2,073,600 primary rays and every bounce ray give the
    oracle's id, t and counts on the binary tree and the same id and t on
    the 8-wide tree.  The FP64 t error of primary and bounce hits is
    printed and bounded."""
    from sequoia_gb300 import scenes
    cfg = scenes.CONFIGS["terrain_4m"]
    tris = scenes.heightfield(2048, 1024, seed=3)
    assert len(tris) == 4_194_304
    bvh = ctx.build(tris, "morton", wide=True)
    nodes, root = bvh.export_node1()
    onodes, oroot, _, _ = oracle.build_morton(tris)
    assert_same_tree(oracle, nodes, root, onodes, oroot)
    rays, _ = cam_rays(oracle, cfg)
    hits, heat = ctx.trace(bvh, "closest", heatmap=True, binary=True, **cam_kw(cfg))
    ids, ts, tests = oracle.trace(nodes, root, tris, rays, 1)
    assert_same_hits(hits, ids, ts, tests, "primary")
    assert np.array_equal(heat, oracle.heatmap(tests))
    wide, _ = ctx.trace(bvh, "closest", **cam_kw(cfg))
    assert_same_hits(wide, ids, ts, None, "primary 8-wide")
    assert (ids != NO_HIT).sum() > len(rays) // 4
    br, _ = scenes.bounce_rays(tris, rays, hits["id"], hits["t"], seed=3)
    assert len(br) == (ids != NO_HIT).sum()
    bh, _ = ctx.trace(bvh, "closest", rays=br, binary=True)
    bids, bts, btests = oracle.trace(nodes, root, tris, br, 1)
    assert_same_hits(bh, bids, bts, btests, "bounce")
    bw, _ = ctx.trace(bvh, "closest", rays=br)
    assert_same_hits(bw, bids, bts, None, "bounce 8-wide")
    mx_p, _, ref_p = fp64_error(oracle, tris, rays, hits, "terrain_4m primary")
    mx_b, _, ref_b = fp64_error(oracle, tris, br, bh, "terrain_4m bounce")
    assert mx_p < T_FP64_BOUND and mx_b < T_FP64_BOUND
    assert mx_p <= ref_p and mx_b <= ref_b
    bvh.free()
    assert ctx.sync() == 0


def test_stress_8m_incoherent(ctx, oracle):
    """stress_8m: 2^24 incoherent rays (origins uniform in the scene box,
    directions uniform on the sphere) in 64 batches.  The 8-wide and binary
    forms agree on every ray (closest ids and t, any-hit flags); a sample of
    every 32nd ray (524,288) gives the oracle's closest and any-hit results
    on the binary tree."""
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(8_000_000, 256, seed=5)
    lo, hi = scenes.scene_box(tris)
    sizes = scenes.batch_sizes(1 << 24, 64, seed=5)
    rays = scenes.random_rays(int(sizes.sum()), lo, hi, seed=5)
    assert len(rays) == 1 << 24
    bvh = ctx.build(tris, "morton", wide=True)
    nodes, root = bvh.export_node1()
    sample = slice(0, None, 32)
    for mode, m in (("closest", 1), ("anyhit", 2)):
        b, _ = ctx.trace(bvh, mode, rays=rays, binary=True)
        w, _ = ctx.trace(bvh, mode, rays=rays)
        if mode == "closest":
            assert np.array_equal(w["id"], b["id"]) and np.array_equal(w["t"], b["t"])
        else:
            assert np.array_equal(w["id"] != NO_HIT, b["id"] != NO_HIT)
        ids, ts, tests = oracle.trace(nodes, root, tris, rays[sample], m)
        assert_same_hits(b[sample], ids, ts, tests, mode)
    bvh.free()
    assert ctx.sync() == 0
