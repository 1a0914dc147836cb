"""Unit tests of the oracle: Morton known answers (bvh-builder.cl:181-252),
the reference's leaf rule (find_middle, bvh-builder.cl:484-552) against an
independent pure-Python split, and the bitonic network's properties."""
import numpy as np
import pytest

import pyoracle
from rtgb import abi, scenes

_p = pyoracle._p


def _point_scene(points):
    """One degenerate triangle per point (AABB = the point)."""
    pts = np.asarray(points, np.float32)
    n = pts.shape[0]
    pos = np.zeros((3 * n, 4), np.float32)
    pos[:, :3] = np.repeat(pts, 3, axis=0)
    nrm = np.zeros_like(pos)
    nrm[:, 1] = 1
    base = scenes.soup(n, seed=0)
    return scenes.Scene(pos, nrm, np.arange(3 * n, dtype=np.uint32).reshape(-1, 3), base.mats,
                        base.mat_map, base.lights)


def _keys(orc, sc, depth):
    s = orc.new_scene(sc)
    k = np.zeros(sc.n_tris, np.uint32)
    assert orc.morton_keys(s.h, depth, _p(k), None, None) == 0
    return k


def test_morton_known_answers(orc):
    # scene AABB [0,1]^3; (0.5, 0.25, 0.75) -> cells (512, 256, 768) at 10 bits/axis;
    # MSB -> LSB order x9 z9 y9 x8 z8 y8 ...: bits 29 (x9), 28 (z9), 25 (z8), 24 (y8)
    k = _keys(orc, _point_scene([(0, 0, 0), (1, 1, 1), (0.5, 0.25, 0.75)]), 30)
    assert k[0] == 0
    assert k[1] == 0            # slice 1.0 * 1024 = 1024: no in-range bit set (the 2^k quirk)
    assert k[2] == (1 << 29) | (1 << 28) | (1 << 25) | (1 << 24)


def test_morton_degenerate_axis(orc):
    # y extent 0: (c - lo) * (1 / 0) = 0 * inf = NaN -> fmin/fmax -> 1.0 -> cell 0
    pts = [(0, 0.3, 0), (1, 0.3, 1), (0.5, 0.3, 0.5)]
    k = _keys(orc, _point_scene(pts), 30)
    ybits = sum(1 << b for b in range(0, 30, 3))
    assert (k & ybits == 0).all()
    assert k[2] == (1 << 29) | (1 << 28)


def _py_morton(c, depth):
    """Independent restatement: bit i takes axis (offset + 1 + i) % 3, source
    bit (i + offset) / 3 (bvh-builder.cl:231-249)."""
    offset = (3 - depth % 3) if depth % 3 else 0
    code = 0
    for i in range(depth):
        axis = (offset + 1 + i) % 3
        code |= ((int(c[axis]) >> ((i + offset) // 3)) & 1) << i
    return code


@pytest.mark.parametrize("depth", [1, 2, 7, 10, 16, 29, 30, 31, 32])
def test_morton_interleave_any_depth(orc, depth):
    rng = np.random.default_rng(depth)
    bits = -(-depth // 3)
    cells = rng.integers(0, 1 << bits, size=(200, 3))
    # points on the exact cell lattice of [0, 2^bits] (corners fix the AABB)
    pts = np.concatenate([[(0, 0, 0), (1 << bits, 1 << bits, 1 << bits)], cells]).astype(np.float32)
    k = _keys(orc, _point_scene(pts), depth)
    for i, c in enumerate(cells):
        assert k[i + 2] == _py_morton(c, depth)


def _py_tree(keys, depth, min_leaf):
    """Pure-Python top-down split of find_middle / set_children."""
    out = []

    def rec(s, e, level, d):
        first, last = s, e - 1
        bit = depth - 1 - level
        me = len(out)
        out.append(None)
        leaf = ((last - first - 1) & 0xFFFFFFFF) <= min_leaf or bit < 0
        if not leaf:
            while ((keys[first] >> bit) & 1) or not ((keys[last] >> bit) & 1):
                level += 1
                bit = depth - 1 - level
                if bit < 0:
                    leaf = True
                    break
        if leaf:
            out[me] = (s, e, 1, d)
            return
        while first + 1 < last:
            mid = (first + last) // 2
            if (keys[mid] >> bit) & 1:
                last = mid
            else:
                first = mid
        out[me] = (s, e, 0, d)
        rec(s, last, level + 1, d + 1)
        rec(last, e, level + 1, d + 1)

    rec(0, len(keys), 0, 0)
    return np.array(out, np.uint32)


@pytest.mark.parametrize("seed,n,vals,depth,min_leaf", [
    (0, 1, 8, 30, 1), (1, 2, 8, 30, 1), (2, 3, 8, 30, 1), (3, 4, 1 << 30, 30, 1),
    (4, 50, 4, 30, 1), (5, 300, 64, 12, 1), (6, 300, 1 << 30, 30, 3), (7, 257, 16, 30, 8),
    (8, 1000, 1 << 20, 21, 1), (9, 64, 1, 30, 1)])
def test_leaf_rule_vs_python(orc, seed, n, vals, depth, min_leaf):
    rng = np.random.default_rng(seed)
    keys = np.sort(rng.integers(0, vals, size=n).astype(np.uint32) & np.uint32((1 << depth) - 1
                                                                                if depth < 32
                                                                                else 0xFFFFFFFF))
    got = orc.emit_keys(keys, depth, min_leaf)
    ref = _py_tree([int(x) for x in keys], depth, min_leaf)
    assert np.array_equal(np.stack([got["start"], got["end"], got["leaf"], got["depth"]], 1), ref)


def test_leaf_rule_cases(orc):
    # a single triangle: count - 2 wraps (unsigned) so the bit loop decides: leaf
    assert orc.emit_keys([5]).shape[0] == 1
    # 2 and 3 triangles (count <= min_leaf + 2): leaves even with distinct keys
    assert orc.emit_keys([1, 2]).shape[0] == 1
    assert orc.emit_keys([1, 2, 3]).shape[0] == 1
    # 4 distinct keys split; equal keys never do, however many
    assert orc.emit_keys([1, 2, 3, 4]).shape[0] == 3
    assert orc.emit_keys([7] * 100).shape[0] == 1


def test_bitonic_sorts_and_is_unstable(orc):
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 8, size=1024).astype(np.uint32)
    p = np.zeros(1024, np.uint32)
    assert orc.sort_bitonic(_p(keys), 1024, _p(p)) == 0
    assert (np.diff(keys[p].astype(np.int64)) >= 0).all()
    assert np.array_equal(np.sort(p), np.arange(1024))
    stable = np.argsort(keys, kind="stable")
    assert not np.array_equal(p, stable)     # same key runs, different order
    for v in range(8):
        assert set(p[keys[p] == v]) == set(stable[keys[stable] == v])


def test_oracle_sah_refuses_deep_trees(orc):
    """The oracle's SAH build refuses a tree deeper than the traversal's
    32-entry stack (240 tiny triangles at x = 2^k, k = -120..119: 44 levels)."""
    c = (2.0 ** np.arange(-120, 120)).astype(np.float32)
    n = c.shape[0]
    pos = np.zeros((3 * n, 4), np.float32)
    pos[:, 0] = np.repeat(c, 3)
    pos[1::3, 1] = 1e-3
    pos[2::3, 2] = 1e-3
    base = scenes.soup(n, seed=1)
    sc = scenes.Scene(pos, pos.copy(), np.arange(3 * n, dtype=np.uint32).reshape(-1, 3),
                      base.mats, base.mat_map, base.lights)
    s = orc.new_scene(sc)
    with pytest.raises(ValueError):
        s.build_sah()
    s2 = orc.new_scene(scenes.soup(3000, seed=3))
    s2.build_sah()
    c2 = s2.canon()
    assert c2["depth"].max() <= 32 and c2[c2["leaf"] == 1]["end"].max() == 3000


def test_oracle_traversal_counts(orc):
    """Traversal work counts: every ray that hits tested a triangle, shadow
    rays number hits x lights, and a ray that misses the scene's box enters
    no node."""
    from helpers import tiny_terrain
    sc = tiny_terrain(32, 16, 3).scene(0)
    s = orc.new_scene(sc)
    s.build(30, 1, 0)
    cam = scenes.camera((0.0, 3.0, -6.0), (0.0, 0.0, 0.5), aspect=1.0)
    smp = pyoracle.gen_primary(orc, cam, 64, 64)
    c = s.traversal_counts(smp)
    hits = int(s.trace(smp)["hit"].sum())
    assert hits > 500 and c["shadow_rays"] == hits * sc.lights.count
    assert c["tris"] >= hits and c["nodes"] >= hits and c["shadow_nodes"] > 0
    # the shadow rays of lights behind the surface are not traced (and the
    # field's hits facing the lights are)
    assert 0 < c["shadow_traced"] < c["shadow_rays"]
    # level rays 50 units above the field, looking away from it
    away = pyoracle.gen_primary(orc, scenes.camera((0.0, 50.0, 0.0), (100.0, 50.0, 0.0)), 8, 8)
    assert s.traversal_counts(away) == {"nodes": 0, "tris": 0, "shadow_nodes": 0,
                                        "shadow_tris": 0, "shadow_rays": 0, "shadow_traced": 0}


@pytest.mark.parametrize("kind", ["soup", "terrain"])
def test_skipped_shadow_rays_do_not_change_the_image(orc, kind):
    """The fused renders do not trace the shadow ray of a light whose two
    shading terms are zero (behind the surface, or a surface without diffuse
    colour and shininess).  On the oracle: flipping exactly those shadow
    bits, for every hit, gives the same fixed-point image; and the rule
    applies often enough to matter (back faces and the soup's mirrors)."""
    from helpers import tiny_terrain
    if kind == "soup":
        sc = scenes.soup(6000, seed=12)
        sc.lights = abi.make_lights((0.1,) * 3, [
            dict(type=abi.RT_POINT_L, pos=(0.0, 4.0, -2.0)),
            dict(type=abi.RT_DIR_L, dir=(0.3, -0.9, 0.3)),
            dict(type=abi.RT_SPOT_L, pos=(2.0, 3.0, -3.0), dir=(-0.4, -0.6, 0.6), angle=0.5)])
        cam = scenes.camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0))
    else:
        sc = tiny_terrain(64, 32, 6).scene(2)
        cam = scenes.camera((0.0, 4.0, -10.0), (0.0, 0.0, 0.0))
    s = orc.new_scene(sc)
    s.build(30, 1, 0)
    smp = pyoracle.gen_primary(orc, cam, 160, 160)
    hits = s.trace(smp)
    s.shadow(smp, hits)
    vm = s.vanishing_lights(smp, hits)
    assert int((vm != 0).sum()) > 200
    img = np.zeros((160 * 160, 3), np.uint32)
    s.shade(smp, hits, img)
    flipped = hits.copy()
    flipped["shadow_hit"] = (flipped["shadow_hit"].astype(np.uint32) ^ vm).astype(
        flipped["shadow_hit"].dtype)
    img2 = np.zeros_like(img)
    s.shade(smp, flipped, img2)
    assert np.array_equal(img, img2)
    # control: flipping every light's bit does change the image
    every = hits.copy()
    every["shadow_hit"] = (every["shadow_hit"].astype(np.uint32) ^
                           np.uint32((1 << sc.lights.count) - 1)).astype(every["shadow_hit"].dtype)
    img3 = np.zeros_like(img)
    s.shade(smp, every, img3)
    assert not np.array_equal(img, img3)
