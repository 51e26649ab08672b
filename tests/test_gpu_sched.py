"""Ray schedules and batched tracing through the C ABI.

How rays are given to GPU lanes (a warp per 32 rays, or per-lane refill)
must not change any result: ids, t and box-test counts are compared between
schedules for both tree forms.  sq_trace_batches (many ray batches, one
launch) must write exactly what one sq_trace per batch writes, with batches
in device buffers of their own, in host memory, and as cameras.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def soup_and_rays(n_tris=300_000, n_rays=120_000, seed=61):
    from sequoia_gb300 import scenes
    tris = scenes.gaussian_soup(n_tris, 16, seed=seed)
    lo, hi = scenes.scene_box(tris)
    return tris, scenes.random_rays(n_rays, lo, hi, seed=seed + 1)


CAM = dict(camera="pinhole", width=333, height=201, origin=(0.0, 2.0, -40.0), target=(0, 0, 0), up=(0, 1, 0),
           vfov=55.0)


@pytest.mark.parametrize("mode", ["closest", "anyhit"])
def test_schedules_agree(ctx, oracle, mode):
    tris, rays = soup_and_rays()
    bvh = ctx.build(tris, "morton", wide=True)
    for kw in (dict(rays=rays), CAM):
        for binary in (True, False):
            base, bheat = ctx.trace(bvh, mode, binary=binary, heatmap=True, sched="tiles", **kw)
            other, oheat = ctx.trace(bvh, mode, binary=binary, heatmap=True, sched="refill", **kw)
            assert np.array_equal(base.view(np.uint32), other.view(np.uint32)), (binary, list(kw))
            assert np.array_equal(bheat, oheat)
            dflt, _ = ctx.trace(bvh, mode, binary=binary, **kw)
            assert np.array_equal(base.view(np.uint32), dflt.view(np.uint32))
    # the binary refill kernel against the oracle directly
    nodes, root = bvh.export_node1()
    h, _ = ctx.trace(bvh, mode, rays=rays, binary=True, sched="refill")
    ids, ts, tests = oracle.trace(nodes, root, tris, rays, 1 if mode == "closest" else 2)
    assert np.array_equal(h["id"], ids) and np.array_equal(h["t"], ts) and np.array_equal(h["tests"], tests)
    assert ctx.sync() == 0


def test_schedule_argument_checks(ctx):
    import ctypes as C
    import sequoia_gb300 as sq
    tris, rays = soup_and_rays(1000, 64)
    bvh = ctx.build(tris, "morton")
    src, _ = ctx._ray_source(rays=rays)
    out = np.empty(64, sq.HIT)
    st = sq.load_library().sq_trace(ctx.handle, bvh.handle, C.byref(src), 1 | 0x200 | 0x400,
                                    out.ctypes.data, None)
    assert st == 1  # both schedules at once: invalid


@pytest.mark.parametrize("mode", ["closest", "anyhit", "ref"])
@pytest.mark.parametrize("wide", [True, False])
def test_trace_batches_equal_separate_calls(ctx, mode, wide):
    torch = pytest.importorskip("torch")
    from sequoia_gb300 import scenes
    tris, rays = soup_and_rays()
    bvh = ctx.build(tris, "morton", wide=wide)
    sizes = scenes.batch_sizes(len(rays), 9, lo=100, hi=40_000, seed=3)
    cuts = np.concatenate([[0], np.cumsum(sizes)])
    batches, want = [], []
    for k in range(len(sizes)):
        r = np.ascontiguousarray(rays[cuts[k]:cuts[k + 1]])
        # alternate device buffers of their own and host arrays
        batches.append(torch.from_numpy(r).cuda() if k % 2 == 0 else r)
        want.append(ctx.trace(bvh, mode, rays=r, heatmap=True))
    if mode != "ref":
        batches.insert(3, CAM)
        want.insert(3, ctx.trace(bvh, mode, heatmap=True, **CAM))
    hits, heat = ctx.trace_batches(bvh, mode, batches, heatmap=True)
    wh = np.concatenate([w[0] for w in want])
    wm = np.concatenate([w[1] for w in want])
    if mode == "ref":
        assert np.array_equal(hits["id"], wh["id"]) and np.array_equal(hits["tests"], wh["tests"])
    else:
        assert np.array_equal(hits.view(np.uint32), wh.view(np.uint32))
    assert np.array_equal(heat, wm)
    # device outputs, schedules forced either way
    d_hits = torch.zeros(len(hits) * 3, dtype=torch.int32, device="cuda")
    for sched in ("refill", "tiles"):
        if mode == "ref":
            break
        d_hits.zero_()
        ctx.trace_batches(bvh, mode, batches, hits=d_hits, sched=sched)
        ctx.sync()  # device outputs are written on the context's stream
        assert np.array_equal(d_hits.cpu().numpy().view(np.uint32), hits.view(np.uint32).reshape(-1))
    # no batches: nothing to do
    h0, _ = ctx.trace_batches(bvh, mode, [])
    assert len(h0) == 0
    assert ctx.sync() == 0
