"""GPU parity at the stress scale: the 17.7M-triangle terrain (4096x2048-cell
fBm field + 1,000 mirror spheres), one LBVH build and one whole 3840x2160
pose at depth 6 with 3 point lights, against the oracle."""
import numpy as np
import pytest

import pyoracle
from helpers import assert_canon_equal, tree_invariants
from rtgb import capi, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stress(ctx, orc):
    wl = scenes.workload_stress()
    sc = wl["terrain"].scene(0)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    yield wl, sc, g, o
    g.close()


def test_stress_tree(stress):
    """The whole tree: keys, permutation and the canonical tree (ranges, leaf
    flags, depths, AABBs) of 17,737,216 triangles, equal to the oracle's."""
    wl, sc, g, o = stress
    gk, gp, _, _ = g.sort_arrays()
    ok, op, _, _ = o.sort_arrays()
    assert np.array_equal(gk, ok) and np.array_equal(gp, op)
    gc = g.canon()
    assert_canon_equal(gc, o.canon())
    tree_invariants(gc, sc.n_tris)
    leaf = gc["leaf"] == 1
    assert int((gc["end"] - gc["start"])[leaf].max()) > 3     # equal-key leaves


@pytest.mark.parametrize("pose", [0, 3])
def test_stress_pose_full_frame(ctx, orc, stress, pose):
    """A pose rendered in full (8,294,400 primary samples, up to 6 bounces,
    3 lights; pose 3 has the most reflection rays of the 8): the fixed-point
    image, the RGBA8 frame and the four ray counters equal the oracle's."""
    wl, sc, g, o = stress
    w, h, b = wl["width"], wl["height"], wl["max_bounces"]
    cam = wl["cameras"][pose]
    n = w * h
    rgba_d, img_d = ctx.alloc(4 * n), ctx.alloc(12 * n)
    st_d = ctx.alloc(32)
    st_d.zero()
    g.render(cam, w, h, b, rgba_d, img_d, st_d)
    ctx.sync()
    assert ctx.device_status() == 0
    img = img_d.read(np.uint32).reshape(-1, 3)
    rgba = rgba_d.read(np.uint8).reshape(-1, 4)
    st = st_d.read(np.uint64)
    rimg, rst = o.render(cam, w, h, b)
    assert np.array_equal(img, rimg)
    assert np.array_equal(rgba, pyoracle.fb_copy(orc, rimg))
    assert (st[0], st[1], st[2], st[3]) == (rst.primary_rays, rst.secondary_rays,
                                            rst.shadow_rays, rst.hits)
    assert rst.secondary_rays > 1_000_000
