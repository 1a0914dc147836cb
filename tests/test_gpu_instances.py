"""Multi-root (instanced) scenes on the GPU against the oracle's restatement
of trace_multi / shadow_trace_multi and the render loop (pinned against the
reference's kernels in test_oracle_pin.py)."""
import numpy as np
import pytest

from helpers import tiny_terrain
from rtgb import abi, capi, scenes
from test_oracle_pin import _instances

pytestmark = pytest.mark.gpu


def _setup(ctx, orc):
    meshes = [scenes.soup(3000, seed=4), tiny_terrain(32, 16, 2).scene(0)]
    gs, os_ = [], []
    for sc in meshes:
        g = capi.Scene(ctx, sc)
        g.build(30, 1)
        o = orc.new_scene(sc)
        o.build(30, 1, 0)
        gs.append(g)
        os_.append(o)
    return gs, os_


@pytest.mark.parametrize("light", ["point", "dir", "spot"])
def test_instances_render_bit_exact(ctx, orc, light):
    gs, os_ = _setup(ctx, orc)
    inst, T, Ti = _instances()
    L = {"point": dict(type=abi.RT_POINT_L, pos=(0.0, 4.0, -3.0), color=(1.0, 1.0, 1.0)),
         "dir": dict(type=abi.RT_DIR_L, dir=(0.3, -1.0, 0.4), color=(1.0, 1.0, 1.0)),
         "spot": dict(type=abi.RT_SPOT_L, pos=(0.0, 4.0, -3.0), dir=(0.0, -0.8, 0.6),
                      angle=0.8, color=(1.0, 1.0, 1.0))}[light]
    lights = abi.make_lights((0.1, 0.1, 0.1), [L])
    I = capi.Instances(ctx, gs, inst, T, Ti, lights)
    om = orc.multi([o.h for o in os_], inst, T, Ti, lights)
    cam = scenes.camera((0.0, 1.5, -6.0), (0.0, 0.0, 0.5), aspect=1.0)
    w = h = 200
    n = w * h
    rgba_d, img_d, st_d = ctx.alloc(4 * n), ctx.alloc(12 * n), ctx.alloc(32)
    st_d.zero()
    I.render(cam, w, h, 3, rgba_d, img_d, st_d)
    ctx.sync()
    img = img_d.read(np.uint32).reshape(-1, 3)
    st = st_d.read(np.uint64)
    rimg, rst = orc.multi_render(om, cam, w, h, 3)
    assert np.array_equal(img, rimg)
    assert st[1] == rst.secondary_rays and st[3] == rst.hits and rst.hits > 5000
    # new transforms (update_bvh_roots): swap the instances' matrices; and
    # rebuild one mesh, which moves its sorted buffers
    I.set_transforms(T[::-1], Ti[::-1])
    gs[0].build(30, 1)
    orc.multi_free(om)
    om = orc.multi([o.h for o in os_], inst, T[::-1].copy(), Ti[::-1].copy(), lights)
    I.render(cam, w, h, 2, rgba_d, img_d)
    ctx.sync()
    rimg, _ = orc.multi_render(om, cam, w, h, 2)
    assert np.array_equal(img_d.read(np.uint32).reshape(-1, 3), rimg)
    orc.multi_free(om)
    I.close()
    assert ctx.device_status() == 0


def test_instances_reject_unbuilt_and_deep_glass(ctx):
    sc = scenes.soup(500, seed=1)
    g = capi.Scene(ctx, sc)
    inst, T, Ti = [0], np.eye(4, dtype=np.float32)[None], np.eye(4, dtype=np.float32)[None]
    with pytest.raises(capi.RtError):
        capi.Instances(ctx, [g], inst, T, Ti, sc.lights)          # not built
    glass = capi.Scene(ctx, scenes.with_glass(sc, 0.5))
    glass.build(30, 1)
    I = capi.Instances(ctx, [glass], inst, T, Ti, sc.lights)
    rgba = ctx.alloc(4 * 32 * 32)
    with pytest.raises(capi.RtError):                                 # glass: up to 6 bounces
        I.render(scenes.camera((0, 0, -4), (0, 0, 0)), 32, 32, 7, rgba)
    I.close()


@pytest.mark.parametrize("bounces", [2, 4, 6])
def test_instances_glass_bit_exact(ctx, orc, bounces):
    """Instances of meshes with glass: reflected and refracted rays of the
    moved, unnormalised normals, against the oracle's multi-root render
    (pinned against the reference's kernels with glass)."""
    meshes = [scenes.with_glass(scenes.soup(3000, seed=4), frac=0.5, seed=2),
              scenes.with_glass(tiny_terrain(32, 16, 2).scene(0), frac=0.5, seed=3)]
    gs, os_ = [], []
    for sc in meshes:
        g = capi.Scene(ctx, sc)
        g.build(30, 1)
        o = orc.new_scene(sc)
        o.build(30, 1, 0)
        gs.append(g)
        os_.append(o)
    inst, T, Ti = _instances()
    lights = abi.make_lights((0.1, 0.1, 0.1), [dict(type=abi.RT_POINT_L, pos=(0.0, 4.0, -3.0),
                                                    color=(1.0, 1.0, 1.0))])
    I = capi.Instances(ctx, gs, inst, T, Ti, lights)
    om = orc.multi([o.h for o in os_], inst, T, Ti, lights)
    cam = scenes.camera((0.0, 1.5, -6.0), (0.0, 0.0, 0.5), aspect=1.0)
    w = h = 160
    rgba_d, img_d, st_d = ctx.alloc(4 * w * h), ctx.alloc(12 * w * h), ctx.alloc(32)
    st_d.zero()
    I.render(cam, w, h, bounces, rgba_d, img_d, st_d)
    ctx.sync()
    rimg, rst = orc.multi_render(om, cam, w, h, bounces, tile=1 << 20)
    st = st_d.read(np.uint64)
    assert np.array_equal(img_d.read(np.uint32).reshape(-1, 3), rimg)
    assert st[1] == rst.secondary_rays > 3000 and st[3] == rst.hits
    orc.multi_free(om)
    I.close()
    assert ctx.device_status() == 0


def test_instances_many_roots_and_ties(ctx, orc):
    """40 roots (two groups of the near-to-far visit), five of them exact
    copies of earlier roots, so that equal world t must go to the lower
    index as in the reference's loop."""
    meshes = [scenes.soup(2000, seed=11), tiny_terrain(24, 12, 1).scene(0)]
    gs, os_ = [], []
    for sc in meshes:
        g = capi.Scene(ctx, sc)
        g.build(30, 1)
        o = orc.new_scene(sc)
        o.build(30, 1, 0)
        gs.append(g)
        os_.append(o)
    rng = np.random.default_rng(3)
    inst, T, Ti = [], [], []
    for k in range(35):
        s = float(rng.uniform(0.3, 1.0))
        m, mi = scenes.transform(float(rng.uniform(0, 360)), (s, s, s),
                                 (float(rng.uniform(-5, 5)), float(rng.uniform(-1, 2)),
                                  float(rng.uniform(-2, 6))))
        inst.append(int(k % 7 == 0)), T.append(m), Ti.append(mi)
    for k in (3, 8, 14, 20, 33):              # duplicates: ties in world t
        inst.append(inst[k]), T.append(T[k]), Ti.append(Ti[k])
    order = rng.permutation(40)               # copies before and after their originals
    inst = [inst[k] for k in order]
    T, Ti = np.array(T)[order], np.array(Ti)[order]
    lights = abi.make_lights((0.1, 0.1, 0.1), [dict(type=abi.RT_POINT_L, pos=(0.0, 5.0, -4.0),
                                                    color=(1.0, 1.0, 1.0))])
    I = capi.Instances(ctx, gs, inst, T, Ti, lights)
    om = orc.multi([o.h for o in os_], inst, T, Ti, lights)
    cam = scenes.camera((0.0, 2.0, -9.0), (0.0, 0.0, 1.0), aspect=1.0)
    w = h = 160
    rgba_d, img_d, st_d = ctx.alloc(4 * w * h), ctx.alloc(12 * w * h), ctx.alloc(32)
    st_d.zero()
    I.render(cam, w, h, 3, rgba_d, img_d, st_d)
    ctx.sync()
    rimg, rst = orc.multi_render(om, cam, w, h, 3)
    st = st_d.read(np.uint64)
    assert np.array_equal(img_d.read(np.uint32).reshape(-1, 3), rimg)
    assert st[1] == rst.secondary_rays and st[3] == rst.hits and rst.hits > 3000
    orc.multi_free(om)
    I.close()
    assert ctx.device_status() == 0
