"""Served form: resident scenes, admission against a memory budget, LRU
eviction, continuous batching.  A request's image is the same alone, in a
mixed burst with uploads, and through the plain rt_render path."""
import numpy as np
import pytest

from helpers import tiny_terrain
from rtgb import capi, scenes

pytestmark = pytest.mark.gpu


def _plain(ctx, sc, cam, w, h, b):
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    rgba = ctx.alloc(4 * w * h)
    g.render(cam, w, h, b, rgba)
    ctx.sync()
    return rgba.read(np.uint8).reshape(-1, 4)


def _pool():
    return [scenes.soup(5000, seed=31), scenes.soup(40000, seed=32),
            tiny_terrain(64, 32, 6).scene(1)]


def test_result_alone_equals_mix_and_plain(ctx):
    pool = _pool()
    srv = capi.Server(ctx, budget=4 << 30, arena=256 << 20, max_views=64, max_inflight=2)
    ids = [srv.add_scene(sc) for sc in pool]
    cam = scenes.camera((0.5, 0.5, -4.0), (0, 0, 0), aspect=160 / 120)
    probe = (ids[1], cam, 160, 120, 3)
    alone, info = srv.result(srv.submit_render(*probe), 160, 120)
    assert info.status == 0 and info.batch_views == 1
    assert np.array_equal(alone, _plain(ctx, pool[1], cam, 160, 120, 3))
    # a mixed burst: renders of every scene and size, two uploads, the probe
    rng = np.random.default_rng(3)
    extra = [scenes.soup(20000, seed=40), tiny_terrain(32, 16, 2).scene(0)]
    tickets = []
    for k in range(40):
        if k in (7, 23):
            tickets.append(("up", srv.submit_upload(extra[k == 23]), None))
            continue
        if k == 20:
            tickets.append(("probe", srv.submit_render(*probe), (160, 120)))
            continue
        w, h = int(rng.integers(16, 200)), int(rng.integers(16, 200))
        sid = ids[int(rng.integers(0, 3))]
        c = scenes.camera(tuple(rng.normal(size=3) * 2 + [0, 0, -4]), (0, 0, 0), aspect=w / h)
        tickets.append(("r", srv.submit_render(sid, c, w, h, int(rng.integers(0, 5))), (w, h)))
    new_ids = []
    views = []
    for kind, t, wh in tickets:
        if kind == "up":
            _, inf = srv.result(t)
            assert inf.status == 0 and inf.scene_id > 0
            new_ids.append(inf.scene_id)
        else:
            img, inf = srv.result(t, *wh)
            assert inf.status == 0
            views.append(inf.batch_views)
            if kind == "probe":
                assert np.array_equal(img, alone)
    assert max(views) > 1                       # requests shared launches
    # the uploaded scenes render like the plain path
    for sid, sc in zip(new_ids, extra):
        img, _ = srv.result(srv.submit_render(sid, cam, 160, 120, 2), 160, 120)
        assert np.array_equal(img, _plain(ctx, sc, cam, 160, 120, 2))
    st = srv.stats()
    assert st.completed == 43 and st.rejected == 0   # probe alone + 40 in the burst + 2
    srv.close()


def test_admission_and_lru_eviction(ctx):
    small = [scenes.soup(20000, seed=50 + k) for k in range(3)]
    one = 20000 * 300                           # ~ bytes of one such scene
    srv = capi.Server(ctx, budget=(64 << 20) + int(2.5 * one), arena=64 << 20, max_views=16,
                      max_inflight=1)
    a = srv.add_scene(small[0])
    b = srv.add_scene(small[1])
    cam = scenes.camera((0, 0, -4), (0, 0, 0))
    srv.result(srv.submit_render(b, cam, 32, 32, 1), 32, 32)      # b used last -> a is LRU
    _, inf = srv.result(srv.submit_upload(small[2]))
    assert inf.status == 0
    st = srv.stats()
    assert st.evicted == 1 and st.resident_scenes == 2
    _, inf = srv.result(srv.submit_render(a, cam, 32, 32, 1), 32, 32, raise_on_error=False)
    assert inf.status == -2                     # evicted scene
    huge = scenes.soup(400000, seed=60)
    _, inf = srv.result(srv.submit_upload(huge), raise_on_error=False)
    assert inf.status == -8                     # does not fit even after eviction
    img, inf = srv.result(srv.submit_render(b, cam, 32, 32, 1), 32, 32)
    assert inf.status == 0
    srv.close()


def test_plain_mode_and_oversized_frame(ctx):
    pool = _pool()
    srv = capi.Server(ctx, budget=2 << 30, arena=1 << 20, max_views=1, max_inflight=4)
    ids = [srv.add_scene(sc) for sc in pool]
    cam = scenes.camera((0, 0, -4), (0, 0, 0))
    ts = [srv.submit_render(ids[k % 3], cam, 64, 64, 2) for k in range(9)]
    for k, t in enumerate(ts):
        img, inf = srv.result(t, 64, 64)
        assert inf.batch_views == 1
        assert np.array_equal(img, _plain(ctx, pool[k % 3], cam, 64, 64, 2))
    # a frame larger than the whole framebuffer arena is rejected, not queued
    _, inf = srv.result(srv.submit_render(ids[0], cam, 1024, 1024, 1), 1024, 1024,
                        raise_on_error=False)
    assert inf.status == -8
    srv.close()


def test_scene_cap_displaces_lru_at_submit(ctx):
    pool = [scenes.soup(3000, seed=70 + k) for k in range(3)]
    srv = capi.Server(ctx, budget=1 << 30, arena=16 << 20, max_views=8, max_inflight=2,
                      max_scenes=3)
    s0, s1, s2 = [srv.add_scene(sc) for sc in pool]
    cam = scenes.camera((0, 0, -4), (0, 0, 0))
    t0 = srv.submit_render(s0, cam, 48, 48, 1)          # s1 is now least recent
    t2 = srv.submit_render(s2, cam, 48, 48, 1)          # pending while s1 goes
    up = srv.submit_upload(scenes.soup(4000, seed=79))   # displaces s1 at submit
    t1 = srv.submit_render(s1, cam, 48, 48, 1)
    _, inf = srv.result(t1, 48, 48, raise_on_error=False)
    assert inf.status == -2                              # displaced scene
    for t in (t0, t2):
        assert srv.result(t, 48, 48)[1].status == 0
    _, inf = srv.result(up)
    new = inf.scene_id
    img, _ = srv.result(srv.submit_render(new, cam, 48, 48, 1), 48, 48)
    assert np.array_equal(img, _plain(ctx, scenes.soup(4000, seed=79), cam, 48, 48, 1))
    # s0 was used before s2: the next upload displaces s0 even though a render
    # of it is queued; the queued render is still served
    t0b = srv.submit_render(s0, cam, 48, 48, 2)
    srv.submit_render(s2, cam, 48, 48, 1)
    srv.submit_render(new, cam, 48, 48, 1)
    up2 = srv.submit_upload(scenes.soup(2000, seed=80))
    img, inf = srv.result(t0b, 48, 48)
    assert inf.status == 0 and np.array_equal(img, _plain(ctx, pool[0], cam, 48, 48, 2))
    assert srv.result(up2)[1].status == 0
    _, inf = srv.result(srv.submit_render(s0, cam, 48, 48, 1), 48, 48, raise_on_error=False)
    assert inf.status == -2
    st = srv.stats()
    assert st.evicted == 2 and st.resident_scenes == 3
    srv.close()


def test_stream_images_equal_plain_and_served(ctx):
    from rtgb import served
    wl = scenes.workload_served(seed=11, pool=6, uploads=3, n_min=2000, n_max=40000)
    cache = served.SceneCache(wl)
    reqs = scenes.served_requests(80, None, seed=12, upload_frac=0.08, min_px=24 * 24,
                                  max_px=200 * 150)
    a = served.run_stream(ctx, cache, reqs, max_views=1)
    b = served.run_stream(ctx, cache, reqs, max_views=32, max_inflight=3)
    assert a["failed"] == b["failed"] == 0 and a["upload_failed"] == b["upload_failed"] == 0
    assert a["uploads"] >= 3 and a["evicted"] == b["evicted"] == a["uploads"]
    assert a["crc"] == b["crc"] and len(a["crc"]) == a["renders"]
    assert b["mean_batch_views"] > 1 and a["mean_batch_views"] == 1


def test_served_refraction_equals_plain(ctx):
    """Scenes with glass are served like any other (launches that hold one
    walk each pixel's ray tree): every image equals rt_render's."""
    pool = [scenes.with_glass(scenes.soup(8000, seed=51), frac=0.4, seed=3),
            scenes.soup(6000, seed=52)]
    srv = capi.Server(ctx, budget=4 << 30, arena=256 << 20, max_views=64, max_inflight=2)
    ids = [srv.add_scene(sc) for sc in pool]
    rng = np.random.default_rng(5)
    reqs = []
    for k in range(16):
        w, h = int(rng.integers(24, 120)), int(rng.integers(24, 120))
        i = k % 2
        cam = scenes.camera(tuple(rng.normal(size=3) + [0, 0, -4]), (0, 0, 0), aspect=w / h)
        b = int(rng.integers(0, 6))
        reqs.append((i, cam, w, h, b, srv.submit_render(ids[i], cam, w, h, b)))
    for i, cam, w, h, b, t in reqs:
        img, inf = srv.result(t, w, h)
        assert inf.status == 0
        assert np.array_equal(img, _plain(ctx, pool[i], cam, w, h, b))
    srv.close()
    assert ctx.device_status() == 0
