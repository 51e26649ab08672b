"""Failure detection without a GPU fault.

Every wait in the kernels is bounded; when one runs out, the kernel raises a
bit in the context's device error word and returns, the next synchronising
call reports SQ_ERR_DEVICE with that bit, and the context stays usable.
These tests make the waits run out on purpose through sq_debug_inject, in
the allowed form: a flag that nothing sets (a look-back word of a tile that
is never run, a grid barrier that counts one block more than the grid) and a
short poll limit.  Allocation failure is injected on the host, in the
library's device allocator: the call must report SQ_ERR_OOM and give back
every block it took.  Nothing here faults, traps or hangs the GPU.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_DEVICE = 4
ERR_OOM = 3
LOOKBACK_TIMEOUT = 0x2
BARRIER_TIMEOUT = 0x8  # SQ_DEVERR_SAH_QUEUE: a task queue or grid-barrier wait ran out


def raw_sync(ctx):
    import sequoia_gb300 as sq
    bits = C.c_uint32()
    st = sq.load_library().sq_sync(ctx.handle, C.byref(bits))
    return st, bits.value


def stable_sort(keys, vals):
    order = np.argsort(keys, kind="stable")
    return keys[order], vals[order]


def test_lookback_wait_runs_out(lib_built):
    import sequoia_gb300 as sq
    ctx = sq.Context(0)
    rng = np.random.default_rng(5)
    n = 200_000
    keys = rng.integers(0, 256, n, dtype=np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    ctx.debug_inject("stall_lookback", 256)
    with pytest.raises(sq.SequoiaError) as e:
        ctx.radix_sort_pairs(keys, vals, key_bits=8, digit_bits=8)
    assert e.value.status == ERR_DEVICE and "0x2" in str(e.value)
    assert raw_sync(ctx) == (0, 0)  # reported once, then cleared
    # the context still works, and the injection was used up
    k, v = ctx.radix_sort_pairs(keys, vals, key_bits=8, digit_bits=8)
    wk, wv = stable_sort(keys, vals)
    assert np.array_equal(k, wk) and np.array_equal(v, wv)
    # a multi-pass sort refuses the injection instead of risking a scatter
    # past the output
    ctx.debug_inject("stall_lookback", 256)
    with pytest.raises(sq.SequoiaError) as e:
        ctx.radix_sort_pairs(keys, vals, key_bits=16, digit_bits=8)
    assert e.value.status == 1
    ctx.close()


def test_collapse_barrier_wait_runs_out(lib_built):
    import sequoia_gb300 as sq
    from sequoia_gb300 import scenes
    ctx = sq.Context(0)
    tris = scenes.gaussian_soup(100_000, 8, seed=71)
    ctx.debug_inject("stall_barrier", 256)
    bvh = ctx.build(tris, "morton", wide=True)
    st, bits = raw_sync(ctx)
    assert st == ERR_DEVICE and bits & BARRIER_TIMEOUT, (st, bits)
    bvh.free()  # its 8-wide tree is not valid; it is never traced
    assert raw_sync(ctx) == (0, 0)
    # a normal build afterwards: the 8-wide hits equal the binary tree's
    bvh = ctx.build(tris, "morton", wide=True)
    lo, hi = scenes.scene_box(tris)
    rays = scenes.random_rays(20_000, lo, hi, seed=72)
    w, _ = ctx.trace(bvh, "closest", rays=rays)
    b, _ = ctx.trace(bvh, "closest", rays=rays, binary=True)
    assert np.array_equal(w["id"], b["id"]) and np.array_equal(w["t"], b["t"])
    assert raw_sync(ctx) == (0, 0)
    bvh.free()
    ctx.close()


def calls(ctx, tris, rays):
    """Each public call that allocates device memory, as (name, fn); fn
    returns the objects to free."""
    keys = np.random.default_rng(3).integers(0, 1 << 30, 50_000, dtype=np.uint32)
    vals = np.arange(50_000, dtype=np.uint32)
    bvh = ctx.build(tris, "morton")
    return bvh, [
        ("morton", lambda: [ctx.build(tris, "morton")]),
        ("morton_wide", lambda: [ctx.build(tris, "morton", wide=True)]),
        ("morton60", lambda: [ctx.build(tris, "morton", morton64=True)]),
        ("sah", lambda: [ctx.build(tris, "sah", bins=16, leaf=4)]),
        ("grid", lambda: [ctx.build(tris, "grid")]),
        ("trace", lambda: (ctx.trace(bvh, "closest", rays=rays, heatmap=True), [])[1]),
        ("trace_batches", lambda: (ctx.trace_batches(bvh, "closest", [rays[:1000], rays[1000:]]), [])[1]),
        ("sort", lambda: (ctx.radix_sort_pairs(keys, vals), [])[1]),
        ("codes", lambda: (ctx.morton_codes(tris), [])[1]),
    ]


def test_allocation_failure_reported_and_nothing_kept(lib_built):
    """For every call and every allocation it makes: failing that allocation
    gives SQ_ERR_OOM, and the context holds exactly the device blocks it held
    before the call; the next call succeeds."""
    import sequoia_gb300 as sq
    from sequoia_gb300 import scenes
    ctx = sq.Context(0)
    tris = scenes.gaussian_soup(30_000, 4, seed=81)
    lo, hi = scenes.scene_box(tris)
    rays = scenes.random_rays(5_000, lo, hi, seed=82)
    bvh, todo = calls(ctx, tris, rays)
    failures = 0
    for name, fn in todo:
        for obj in fn():  # warm the cache: later calls reuse its blocks
            obj.free()
        k = 0
        while True:
            ctx.sync()
            before = ctx.debug_memory()["live_blocks"]
            ctx.debug_inject("fail_alloc", k)
            try:
                made = fn()
            except sq.SequoiaError as e:
                assert e.status == ERR_OOM, (name, k, str(e))
                ctx.sync()
                assert ctx.debug_memory()["live_blocks"] == before, (name, k)
                failures += 1
                k += 1
                continue
            # the call made fewer than k + 1 allocations: done with it
            for obj in made:
                obj.free()
            ctx.debug_inject("off")
            break
        assert k >= 1, name  # every call allocates at least once
    assert failures >= len(todo)
    bvh.free()
    assert ctx.sync() == 0
    ctx.close()
