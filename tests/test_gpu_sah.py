"""The library's CPU SAH BVH (rt_bvh_build_sah) against the oracle's
restatement of the reference's BVH::construct (pinned in test_oracle_pin.py):
the same tree, the same triangle order, and the same frame from every
render path that traverses it."""
import numpy as np
import pytest

from helpers import tiny_terrain
from rtgb import capi, scenes

pytestmark = pytest.mark.gpu


def _negative_soup():
    sc = scenes.soup(2500, seed=8)
    pos = sc.pos4.copy()
    pos[:, :3] -= np.float32(5.0)
    return scenes.Scene(pos, sc.nrm4, sc.idx, sc.mats, sc.mat_map, sc.lights)


CASES = {"soup": lambda: scenes.soup(4000, seed=2),
         "terrain": lambda: tiny_terrain(48, 24, 3).scene(0),
         "negative": _negative_soup,
         "soup200k": lambda: scenes.soup(200_000, seed=5)}


@pytest.mark.parametrize("kind", list(CASES))
def test_sah_tree_and_frame(ctx, orc, kind):
    sc = CASES[kind]()
    g = capi.Scene(ctx, sc)
    g.build_sah()
    o = orc.new_scene(sc)
    o.build_sah()
    gc, oc = g.canon(), o.canon()
    assert gc.shape == oc.shape and gc.tobytes() == oc.tobytes()
    gi, gm = g.read_sorted_buffers()
    oi, om = o.buffers()
    assert np.array_equal(gi, oi) and np.array_equal(gm, om)
    if kind == "negative":
        cam = scenes.camera((-5.0, -4.0, -9.0), (-5.0, -5.0, -5.0))
    elif kind == "terrain":
        cam = scenes.camera((0.0, 3.0, -6.0), (0.0, 0.0, 0.5))
    else:
        cam = scenes.camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0))
    w = h = 192
    rimg, rst = o.render(cam, w, h, 3, tile=1 << 20)
    assert rst.hits > 1000
    rgba, img, st = ctx.alloc(4 * w * h), ctx.alloc(12 * w * h), ctx.alloc(32)
    cfg0 = ctx.render_config()
    for variant in range(len(ctx.variants())):
        ctx.set_render_config(variant, 0, 64)
        st.zero()
        g.render(cam, w, h, 3, rgba, img, st)
        ctx.sync()
        assert np.array_equal(img.read(np.uint32).reshape(-1, 3), rimg), variant
        s = st.read(np.uint64)
        assert s[1] == rst.secondary_rays and s[3] == rst.hits
    ctx.set_render_config(cfg0.variant, cfg0.blocks_per_sm, cfg0.chunk)
    with pytest.raises(capi.RtError):
        g.refit()                                   # an SAH tree is rebuilt, not refit
    g.build(30, 1)                                  # the LBVH again, from the SAH order
    g.refit()
    assert ctx.device_status() == 0


def _deep_scene():
    """240 tiny triangles at x = 2^k, k = -120..119: the SAH peels about five
    off per level (those within a factor 32 of the farthest), so the tree is
    44 levels deep."""
    c = (2.0 ** np.arange(-120, 120)).astype(np.float32)
    n = c.shape[0]
    pos = np.zeros((3 * n, 4), np.float32)
    pos[:, 0] = np.repeat(c, 3)
    pos[1::3, 1] = 1e-3
    pos[2::3, 2] = 1e-3
    nrm = np.zeros_like(pos)
    nrm[:, 0] = 1.0
    base = scenes.soup(n, seed=1)
    return scenes.Scene(pos, nrm, np.arange(3 * n, dtype=np.uint32).reshape(-1, 3), base.mats,
                        base.mat_map, base.lights)


def test_sah_too_deep_is_refused(ctx, orc):
    """A tree deeper than the traversal's 32-entry stack (the reference's
    kernel would write past its stack) is refused by both builders; the
    scene keeps no tree."""
    sc = _deep_scene()
    o = orc.new_scene(sc)
    with pytest.raises(ValueError):
        o.build_sah()
    g = capi.Scene(ctx, sc)
    with pytest.raises(capi.RtError):
        g.build_sah()
    g.build(30, 1)                 # the LBVH of the same scene is fine
    assert ctx.device_status() == 0
