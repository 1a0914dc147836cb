"""GPU parity of traversal, shading and the fused render (bit-exact against
the oracle; closest-hit ids against an FP64 brute-force intersector)."""
import numpy as np
import pytest

import pyoracle
from helpers import camera_small, single_light, tiny_terrain
from rtgb import abi, capi, scenes

pytestmark = pytest.mark.gpu


def _pair(ctx, orc, sc, depth=30):
    g = capi.Scene(ctx, sc)
    g.build(depth, 1)
    o = orc.new_scene(sc)
    o.build(depth, 1, 0)
    return g, o


def _primary(ctx, orc, cam, w, h):
    n = w * h
    d = ctx.alloc(80 * n)
    ctx.gen_primary(cam, w, h, d)
    ctx.sync()
    return d, pyoracle.gen_primary(orc, cam, w, h)


def test_primary_rays(ctx, orc):
    cam = camera_small()
    for (w, h) in [(512, 512), (100, 70), (33, 65)]:
        d, ref = _primary(ctx, orc, cam, w, h)
        got = d.read(abi.SAMPLE_DTYPE)
        assert got.tobytes() == ref.tobytes()


@pytest.mark.parametrize("light", ["point", "spot", "dir"])
def test_stages_match_oracle(ctx, orc, light):
    sc = scenes.soup(10000, seed=2)
    sc.lights = single_light(light)
    g, o = _pair(ctx, orc, sc)
    cam = camera_small()
    w = h = 256
    n = w * h
    smp_d, smp = _primary(ctx, orc, cam, w, h)
    hit_d = ctx.alloc(64 * n)
    hit_d.zero()
    g.trace(smp_d, n, hit_d)
    g.shadow(smp_d, n, hit_d)
    ctx.sync()
    got = hit_d.read(abi.HIT_DTYPE)
    ref = o.trace(smp)
    o.shadow(smp, ref)
    m = ref["hit"] == 1
    assert np.array_equal(got["hit"], ref["hit"])
    for f in ("id", "t", "inverse_n", "shadow_hit"):
        assert np.array_equal(got[f][m], ref[f][m]), f
    for f in ("n", "hit_point"):
        assert np.array_equal(got[f][m][:, :3], ref[f][m][:, :3]), f
    img_d = ctx.alloc(12 * n)
    img_d.zero()
    g.shade(smp_d, hit_d, n, img_d)
    ctx.sync()
    img = img_d.read(np.uint32).reshape(-1, 3)
    rimg = np.zeros((n, 3), np.uint32)
    o.shade(smp, ref, rimg)
    assert np.array_equal(img, rimg)
    out_d = ctx.alloc(80 * n)
    cnt_d = ctx.alloc(4)
    k = g.gen_secondary(smp_d, n, hit_d, out_d, n, cnt_d)
    ref_sec = o.gen_secondary(smp, ref)
    assert k == ref_sec.shape[0] and k > 0
    assert out_d.read(abi.SAMPLE_DTYPE, k).tobytes() == ref_sec.tobytes()
    rgba_d = ctx.alloc(4 * n)
    ctx.fb_copy(img_d, rgba_d, n)
    ctx.sync()
    assert np.array_equal(rgba_d.read(np.uint8).reshape(-1, 4), pyoracle.fb_copy(orc, rimg))


def _render_both(ctx, orc, sc, cam, w, h, bounces):
    g, o = _pair(ctx, orc, sc)
    n = w * h
    rgba_d, img_d = ctx.alloc(4 * n), ctx.alloc(12 * n)
    st_d = ctx.alloc(32)
    st_d.zero()
    g.render(cam, w, h, bounces, rgba_d, img_d, st_d)
    ctx.sync()
    img = img_d.read(np.uint32).reshape(-1, 3)
    rgba = rgba_d.read(np.uint8).reshape(-1, 4)
    st = st_d.read(np.uint64)
    rimg, rst = o.render(cam, w, h, bounces)
    return img, rgba, st, rimg, rst, g, o


def test_render_small_workload_bit_exact(ctx, orc):
    """512x512 soup, depth 3, one point light: identical fixed-point image."""
    wl = scenes.workload_small()
    img, rgba, st, rimg, rst, _, _ = _render_both(ctx, orc, wl["scene"], wl["camera"], 512, 512, 3)
    assert np.array_equal(img, rimg)
    assert np.array_equal(rgba, pyoracle.fb_copy(orc, rimg))
    assert st[0] == rst.primary_rays and st[1] == rst.secondary_rays
    assert st[2] == rst.shadow_rays and st[3] == rst.hits
    assert ctx.device_status() == 0


@pytest.mark.parametrize("bounces", [0, 1, 4])
def test_render_terrain_two_lights(ctx, orc, bounces):
    ter = tiny_terrain(96, 48, 12)
    sc = ter.scene(3)
    cam = scenes.camera((0.0, 4.0, -10.0), (0.0, 0.0, 0.0), aspect=160 / 90)
    img, rgba, st, rimg, rst, _, _ = _render_both(ctx, orc, sc, cam, 160, 90, bounces)
    assert np.array_equal(img, rimg)
    assert st[1] == rst.secondary_rays


def test_render_mid_scale_full_frame(ctx, orc):
    """The bench's mid-scale frame in full: 1920x1080, the 1.24M-triangle
    terrain with 200 mirror spheres, 2 point lights, depth 4.  Every pixel of
    the fixed-point image and of the RGBA8 frame, and the four ray counters
    (primary, secondary, shadow, hits) that the bench's Mrays/s is computed
    from, equal the oracle's full render."""
    wl = scenes.workload_mid()
    sc = wl["terrain"].scene(0)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    w, h = wl["width"], wl["height"]
    n = w * h
    rgba_d, img_d = ctx.alloc(4 * n), ctx.alloc(12 * n)
    st_d = ctx.alloc(32)
    st_d.zero()
    g.render(wl["camera"], w, h, wl["max_bounces"], rgba_d, img_d, st_d)
    ctx.sync()
    assert ctx.device_status() == 0
    img = img_d.read(np.uint32).reshape(-1, 3)
    rgba = rgba_d.read(np.uint8).reshape(-1, 4)
    st = st_d.read(np.uint64)
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    rimg, rst = o.render(wl["camera"], w, h, wl["max_bounces"])
    assert np.array_equal(img, rimg)
    assert np.array_equal(rgba, pyoracle.fb_copy(orc, rimg))
    assert (st[0], st[1], st[2], st[3]) == (rst.primary_rays, rst.secondary_rays,
                                            rst.shadow_rays, rst.hits)
    assert rst.secondary_rays > 500_000 and rst.hits > 1_000_000


def test_closest_hit_vs_fp64_mid_scale(ctx, orc):
    """Closest-hit ids of the mid-scale frame's primary rays against the FP64
    brute-force intersector, on 16,384 rays spread over the whole frame
    (every 126th sample): >= 99.99% equal, every mismatch a tie within 1e-6
    relative t; hit t within 1e-5 relative for >= 99.95% and within 1e-3 for
    all (the reference's FP32 Moller-Trumbore at grazing angles)."""
    wl = scenes.workload_mid()
    sc = wl["terrain"].scene(0)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    w, h = wl["width"], wl["height"]
    n = w * h
    smp_d, smp = _primary(ctx, orc, wl["camera"], w, h)
    hit_d = ctx.alloc(64 * n)
    hit_d.zero()
    g.trace(smp_d, n, hit_d)
    ctx.sync()
    pick = np.arange(0, n, 126)[:16384]
    hits = hit_d.read(abi.HIT_DTYPE)[pick]
    sub = smp[pick]
    _, _, _, orig = g.sort_arrays()
    gid = np.where(hits["hit"] == 1, orig.astype(np.int64)[np.clip(hits["id"], 0, None)], -1)
    gid = gid.astype(np.int32)
    fid, ft = o.fp64_closest(sub)
    match = gid == fid
    assert match.mean() >= 0.9999
    mism = np.nonzero(~match)[0]
    if mism.size:
        t_g = o.fp64_t_of(sub[mism], gid[mism])
        assert np.all(np.abs(t_g - ft[mism]) <= 1e-6 * np.abs(ft[mism]))
    hm = (gid >= 0) & match
    assert hm.sum() > 8000
    rel = np.abs(hits["t"][hm].astype(np.float64) - ft[hm]) / np.abs(ft[hm])
    assert (rel <= 1e-5).mean() >= 0.9995
    assert rel.max() <= 1e-3


def test_closest_hit_vs_fp64(ctx, orc):
    """Closest-hit ids vs an FP64 brute-force intersector: >= 99.99% equal,
    every mismatch a tie within 1e-6 relative t; hit t within 1e-5 relative
    for >= 99.95% of hits and within 1e-3 for all."""
    sc = scenes.soup(10000, seed=4)
    g, o = _pair(ctx, orc, sc)
    cam = camera_small()
    w = h = 256
    n = w * h
    smp_d, smp = _primary(ctx, orc, cam, w, h)
    hit_d = ctx.alloc(64 * n)
    hit_d.zero()
    g.trace(smp_d, n, hit_d)
    ctx.sync()
    hits = hit_d.read(abi.HIT_DTYPE)
    _, _, _, orig = g.sort_arrays()
    gid = np.where(hits["hit"] == 1, orig.astype(np.int64)[np.clip(hits["id"], 0, None)], -1)
    gid = gid.astype(np.int32)
    fid, ft = o.fp64_closest(smp)
    match = gid == fid
    assert match.mean() >= 0.9999
    mism = np.nonzero(~match)[0]
    if mism.size:
        t_g = o.fp64_t_of(smp[mism], gid[mism])
        assert np.all(np.abs(t_g - ft[mism]) <= 1e-6 * np.abs(ft[mism]))
    hm = (gid >= 0) & match
    rel = np.abs(hits["t"][hm].astype(np.float64) - ft[hm]) / np.abs(ft[hm])
    # FP32 Moller-Trumbore (the reference's formula, reproduced bit for bit,
    # see test_stages_match_oracle) loses accuracy at grazing angles: on this
    # scene 2 of 13,295 hits (0.015%) are between 1e-5 and 1e-4 from FP64.
    assert (rel <= 1e-5).mean() >= 0.9995
    assert rel.max() <= 1e-3


def test_render_host_e2e(ctx, orc):
    """rt_render_host: host vertices in, host RGBA8 out (upload + build + render)."""
    ter = tiny_terrain(64, 32, 6)
    sc = ter.scene(0)
    g = capi.Scene(ctx, sc)
    cam = scenes.camera((0.0, 4.0, -10.0), (0.0, 0.0, 0.0), aspect=1.0)
    pos, nrm = ter.frame_vertices(2)
    rgba, st = g.render_host(cam, 128, 128, 2, pos, nrm)
    o = orc.new_scene(ter.scene(2))
    o.build(30, 1, 0)
    rimg, rst = o.render(cam, 128, 128, 2)
    assert np.array_equal(rgba, pyoracle.fb_copy(orc, rimg))
    assert st.primary_rays == 128 * 128


def test_render_host_async_pipelined(ctx):
    """rt_render_host_async / rt_render_host_wait: frames queued on two
    streams with two scenes, each collected after the next is queued, equal
    the synchronous rt_render_host frames; one frame pending per stream."""
    ter = tiny_terrain(64, 32, 6)
    cam = scenes.camera((0.0, 4.0, -10.0), (0.0, 0.0, 0.0), aspect=1.0)
    frames = [ter.frame_vertices(i) for i in range(5)]
    ref = capi.Scene(ctx, ter.scene(0))
    expect = []
    for pos, nrm in frames:
        rgba, st = ref.render_host(cam, 96, 96, 3, pos, nrm)
        expect.append((rgba.copy(), st.primary_rays, st.secondary_rays))
    streams = [ctx.stream_create(), ctx.stream_create()]
    sc = [capi.Scene(ctx, ter.scene(0)), capi.Scene(ctx, ter.scene(0))]
    pending = [None, None]
    got = []
    try:
        for k, (pos, nrm) in enumerate(frames):
            j = k % 2
            if pending[j] is not None:
                ctx.render_host_wait(streams[j])
                got.append(pending[j])
            rgba, st = sc[j].render_host_async(cam, 96, 96, 3, pos, nrm, stream=streams[j])
            pending[j] = (k, rgba, st, pos, nrm)
            if k == 0:   # a second frame on a stream with one pending is refused
                with pytest.raises(capi.RtError):
                    sc[0].render_host_async(cam, 96, 96, 3, pos, nrm, stream=streams[0])
        for j in (0, 1):
            if pending[j] is not None:
                ctx.render_host_wait(streams[j])
                got.append(pending[j])
        with pytest.raises(capi.RtError):   # nothing pending
            ctx.render_host_wait(streams[0])
        # a frame refused at the door (wrong vertex count) leaves nothing
        # pending, and the stream takes the next frame
        pos, nrm = frames[0]
        with pytest.raises(capi.RtError):
            sc[0].render_host_async(cam, 96, 96, 3, pos[:-1], nrm[:-1], stream=streams[0])
        with pytest.raises(capi.RtError):
            ctx.render_host_wait(streams[0])
        rgba, st = sc[0].render_host_async(cam, 96, 96, 3, pos, nrm, stream=streams[0])
        ctx.render_host_wait(streams[0])
        assert np.array_equal(rgba, expect[0][0])
    finally:
        for s in streams:
            ctx.stream_destroy(s)
    assert sorted(k for k, *_ in got) == list(range(len(frames)))
    for k, rgba, st, _, _ in got:
        e_rgba, e_prim, e_sec = expect[k]
        assert np.array_equal(rgba, e_rgba), "frame %d" % k
        assert (st.primary_rays, st.secondary_rays) == (e_prim, e_sec)
    assert ctx.device_status() == 0


def test_render_variants_identical(ctx, orc):
    """Every kernel variant / chunk / residency the autotuner can pick gives
    the same image; the autotuner installs and caches its choice."""
    ter = tiny_terrain(96, 48, 12)
    sc = ter.scene(1)
    cam = scenes.camera((0.0, 4.0, -10.0), (0.0, 0.0, 0.0), aspect=200 / 120)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    w, h = 200, 120
    rgba_d, img_d = ctx.alloc(4 * w * h), ctx.alloc(12 * w * h)
    saved = ctx.render_config()
    images = []
    for v, (threads, minb, occ) in enumerate(ctx.variants()):
        assert occ >= 1 and threads in (64, 128, 256)
        for chunk in (32, 128, 256):
            ctx.set_render_config(v, max(1, occ // 2), chunk)
            g.render(cam, w, h, 4, rgba_d, img_d)
            ctx.sync()
            images.append(img_d.read(np.uint32))
    for im in images[1:]:
        assert np.array_equal(im, images[0])
    cfg, ms = g.autotune(cam, w, h, 4, trials=1)
    assert ms > 0 and 0 <= cfg.variant < len(ctx.variants())
    cur = ctx.render_config()
    assert (cur.variant, cur.blocks_per_sm, cur.chunk) == (cfg.variant, cfg.blocks_per_sm, cfg.chunk)
    cfg2, ms2 = g.autotune(cam, w, h, 4, trials=1)          # cached: no timing
    assert ms2 < 0 and cfg2.variant == cfg.variant
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    rimg, _ = o.render(cam, w, h, 4)
    assert np.array_equal(images[0].reshape(-1, 3), rimg)
    ctx.set_render_config(saved.variant, saved.blocks_per_sm, saved.chunk)


def test_render_obj_model_bit_exact(ctx, orc, tmp_path):
    """A model through the OBJ path (rt_obj_load -> one aggregate mesh, the
    first group's material): a 100x100-cell grid written as v/vt/vn faces
    with one shared normal, and a terrain written as v//vn faces; each
    rendered on the GPU equals the oracle's render of the same scene."""
    from rtgb import obj
    k = 100
    lines = ["g grid"]
    for j in range(k + 1):
        for i in range(k + 1):
            lines.append("v %.1f %.4f %.1f" % (-5.0 + 0.1 * i, 0.05 * np.sin(0.3 * i + 0.2 * j),
                                                -5.0 + 0.1 * j))
    for j in range(k + 1):
        for i in range(k + 1):
            lines.append("vt %.2f %.2f" % (i / k, j / k))
    lines.append("vn 0 1 0")
    for j in range(k):
        for i in range(k):
            a = j * (k + 1) + i + 1
            b, c, d = a + 1, a + k + 1, a + k + 2
            lines.append("f %d/%d/1 %d/%d/1 %d/%d/1" % (b, b, a, a, c, c))
            lines.append("f %d/%d/1 %d/%d/1 %d/%d/1" % (b, b, c, c, d, d))
    p = tmp_path / "grid.obj"
    p.write_text("\n".join(lines) + "\n")
    sc = obj.load(p)
    assert sc.n_tris == 2 * k * k and sc.n_verts == (k + 1) ** 2
    cam = scenes.camera((0.0, 4.0, -8.0), (0.0, 0.0, 0.0), aspect=1.0)
    img, rgba, st, rimg, rst, _, _ = _render_both(ctx, orc, sc, cam, 128, 128, 2)
    assert np.array_equal(img, rimg) and st[3] == rst.hits and rst.hits > 0
    ter = tiny_terrain(64, 32, 6).scene(2)
    q = tmp_path / "terrain.obj"
    obj.write(q, ter.pos4, ter.nrm4, ter.idx)
    sc2 = obj.load(q, lights=ter.lights, reflectiveness=0.5)
    cam2 = scenes.camera((0.0, 4.0, -10.0), (0.0, 0.0, 0.0), aspect=160 / 90)
    img, rgba, st, rimg, rst, _, _ = _render_both(ctx, orc, sc2, cam2, 160, 90, 3)
    assert np.array_equal(img, rimg) and st[1] == rst.secondary_rays
    assert ctx.device_status() == 0


@pytest.mark.parametrize("fill", [1.0, 0.7])
def test_refraction_secondary_rays_match_oracle(ctx, orc, fill):
    """generate_secondary_rays_disc with glass (refractive index 1.333): the
    stage-wise GPU call makes the oracle's rays, slot for slot, both with
    room for all of them and with a buffer that cuts into the refracted
    rays (those past it are dropped, and their hits' reflected rays keep
    R = 1, as in the kernel)."""
    sc = scenes.with_glass(scenes.soup(10000, seed=2), frac=0.4, seed=3)
    g, o = _pair(ctx, orc, sc)
    cam = camera_small()
    w = h = 256
    n = w * h
    smp_d, smp = _primary(ctx, orc, cam, w, h)
    hit_d = ctx.alloc(64 * n)
    hit_d.zero()
    g.trace(smp_d, n, hit_d)
    g.shadow(smp_d, n, hit_d)
    ctx.sync()
    ref = o.trace(smp)
    o.shadow(smp, ref)
    total = o.gen_secondary(smp, ref, 2 * n).shape[0]
    max_out = max(1, int(total * fill))
    out_d = ctx.alloc(80 * max_out)
    cnt_d = ctx.alloc(4)
    k = g.gen_secondary(smp_d, n, hit_d, out_d, max_out, cnt_d)
    ref_sec = o.gen_secondary(smp, ref, max_out)
    assert k == ref_sec.shape[0] == min(total, max_out) and k > 1000
    assert out_d.read(abi.SAMPLE_DTYPE, k).tobytes() == ref_sec.tobytes()


@pytest.mark.parametrize("bounces", [1, 4, 6, 8])
def test_render_refraction_bit_exact(ctx, orc, bounces):
    """rt_render of a soup with glass: each hit on glass spawns a refracted
    and a reflected ray, followed by the pooled refraction variant (up to 6
    bounces) or walked as a tree per pixel; with every configured variant
    (those that cannot follow refraction, or hold too few rays, give way to
    one that can) the fixed-point image and the ray counts equal the
    oracle's wavefront render (a tile large enough that no wavefront is
    cut)."""
    sc = scenes.with_glass(scenes.soup(8000, seed=5), frac=0.4, seed=1)
    g, o = _pair(ctx, orc, sc)
    cam = scenes.camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), aspect=1.0)
    w = h = 256
    n = w * h
    rimg, rst = o.render(cam, w, h, bounces, tile=1 << 20)
    assert rst.secondary_rays > 5000
    rgba_d, img_d, st_d = ctx.alloc(4 * n), ctx.alloc(12 * n), ctx.alloc(32)
    cfg0 = ctx.render_config()
    for v in range(len(ctx.variants())):
        ctx.set_render_config(v, 0, 64)
        st_d.zero()
        g.render(cam, w, h, bounces, rgba_d, img_d, st_d)
        ctx.sync()
        img = img_d.read(np.uint32).reshape(-1, 3)
        st = st_d.read(np.uint64)
        assert np.array_equal(img, rimg), v
        assert st[1] == rst.secondary_rays and st[2] == rst.shadow_rays and st[3] == rst.hits, v
    ctx.set_render_config(cfg0.variant, cfg0.blocks_per_sm, cfg0.chunk)
    assert ctx.device_status() == 0
