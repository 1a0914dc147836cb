"""Batched form: one persistent build launch for many scenes, one persistent
render launch for many images, CUDA-graph replay.  Everything must equal the
plain per-scene path bit for bit."""
import numpy as np
import pytest

from helpers import assert_canon_equal, tiny_terrain
from rtgb import capi, scenes

pytestmark = pytest.mark.gpu


def _items(ctx):
    rng = np.random.default_rng(7)
    scs = [scenes.soup(int(n), seed=100 + k) for k, n in
           enumerate([1, 3, 17, 1000, 4097, 20000, 60000])]
    scs.append(tiny_terrain(64, 32, 5).scene(2))
    gscenes = [capi.Scene(ctx, sc) for sc in scs]
    items = []
    for k, g in enumerate(gscenes):
        w, h = [(64, 64), (96, 40), (33, 47)][k % 3]
        cam = scenes.camera((0.0, 0.5, -4.0), (0.0, 0.0, 0.0), aspect=w / h)
        items.append((g, cam, w, h, int(rng.integers(0, 5))))
    # two extra views of shared scenes
    items.append((gscenes[5], scenes.camera((1.0, 1.0, -3.0), (0, 0, 0)), 80, 80, 3))
    items.append((gscenes[7], scenes.camera((0.0, 4.0, -10.0), (0, 0, 0)), 120, 70, 4))
    return scs, gscenes, items


def _plain(ctx, sc, cam, w, h, b):
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    rgba = ctx.alloc(4 * w * h)
    g.render(cam, w, h, b, rgba)
    ctx.sync()
    return g, rgba.read(np.uint8)


def test_batch_build_and_render_match_plain(ctx):
    scs, gscenes, items = _items(ctx)
    batch = capi.Batch(ctx)
    batch.set(items)
    n_scenes, n_tris, n_px = batch.info()
    assert n_scenes == len(scs) and n_tris == sum(s.n_tris for s in scs)
    batch.build()
    rgba = ctx.alloc(4 * batch.pixels)
    stats = ctx.alloc(32)
    stats.zero()
    batch.render(rgba, stats)
    ctx.sync()
    out = rgba.read(np.uint8)
    assert ctx.device_status() == 0
    # every scene's BVH equals a one-scene build
    for sc, g in zip(scs, gscenes):
        p, _ = _plain(ctx, sc, scenes.camera((0, 0, -4), (0, 0, 0)), 8, 8, 0)
        assert_canon_equal(g.canon(), p.canon())
        assert all(np.array_equal(a, b) for a, b in zip(g.sort_arrays(), p.sort_arrays()))
    # every image equals the plain render
    prim = 0
    for (g, cam, w, h, b), (off, _, _) in zip(items, batch.offsets):
        sc = scs[gscenes.index(g)]
        _, ref = _plain(ctx, sc, cam, w, h, b)
        assert np.array_equal(out[4 * off:4 * (off + w * h)], ref)
        prim += w * h
    st = stats.read(np.uint64)
    assert st[0] == prim


def test_batch_graph_replay(ctx):
    scs, gscenes, items = _items(ctx)
    batch = capi.Batch(ctx)
    batch.set(items)
    rgba = ctx.alloc(4 * batch.pixels)
    stats = ctx.alloc(32)
    batch.capture(rgba, stats)
    outs = []
    for _ in range(3):
        rgba.zero()
        batch.replay()
        ctx.sync()
        outs.append(rgba.read(np.uint8))
        assert stats.read(np.uint64)[0] == batch.pixels
    assert all(np.array_equal(outs[0], o) for o in outs[1:])
    for (g, cam, w, h, b), (off, _, _) in zip(items, batch.offsets):
        sc = scs[gscenes.index(g)]
        _, ref = _plain(ctx, sc, cam, w, h, b)
        assert np.array_equal(outs[0][4 * off:4 * (off + w * h)], ref)


def test_batch_rejects_bad_views(ctx):
    sc = scenes.soup(100, seed=1)
    g = capi.Scene(ctx, sc)
    batch = capi.Batch(ctx)
    cam = scenes.camera((0, 0, -4), (0, 0, 0))
    import ctypes as C
    from rtgb import abi
    arr = (abi.BatchView * 2)()
    for k in range(2):
        arr[k].scene = g.h
        arr[k].cam = cam
        arr[k].width = arr[k].height = 16
        arr[k].max_bounces = 1
    arr[1].rgba_offset = 7                          # not packed
    r = ctx.lib.rt_batch_set(ctx.h, batch.h, arr, 2, None)
    assert r == -2 and b"packed" in ctx.lib.rt_last_error()


@pytest.mark.parametrize("deepest", [4, 6, 8])
def test_batch_refraction_matches_plain(ctx, deepest):
    """Glass scenes in one batch: the pooled kernel whose ray pool holds the
    deepest view (4 or 6 bounces), or each pixel's ray tree beyond that; every
    image equals rt_render's (itself equal to the oracle's)."""
    scs = [scenes.with_glass(scenes.soup(6000, seed=70), frac=0.4, seed=1),
           scenes.soup(3000, seed=71),
           scenes.with_glass(tiny_terrain(48, 24, 4).scene(0), frac=0.5, seed=2)]
    gscenes = [capi.Scene(ctx, sc) for sc in scs]
    items = []
    for k, (g, b) in enumerate(zip(gscenes * 2, [deepest, 2, 3, 1, deepest - 1, 0])):
        w, h = [(96, 64), (64, 64), (80, 50)][k % 3]
        cam = scenes.camera((0.3 * k, 0.5, -4.0), (0.0, 0.0, 0.0), aspect=w / h)
        items.append((g, cam, w, h, b))
    batch = capi.Batch(ctx)
    batch.set(items)
    batch.build()
    rgba = ctx.alloc(4 * batch.pixels)
    batch.render(rgba)
    ctx.sync()
    out = rgba.read(np.uint8)
    assert ctx.device_status() == 0
    for (g, cam, w, h, b), (off, _, _) in zip(items, batch.offsets):
        sc = scs[gscenes.index(g)]
        _, ref = _plain(ctx, sc, cam, w, h, b)
        assert np.array_equal(out[4 * off:4 * (off + w * h)], ref)
