"""Shared helpers for the parity tests (scenes and comparisons)."""
import numpy as np

from rtgb import abi, scenes


def tiny_terrain(nx=64, nz=32, spheres=4, seed=5):
    return scenes.Terrain(nx, nz, n_spheres=spheres, seed=seed)


def assert_canon_equal(a, b):
    """Canonical range trees equal: ranges, leaf flags, depths, AABBs (==)."""
    assert a.shape == b.shape, "node count %d vs %d" % (a.shape[0], b.shape[0])
    for f in ("start", "end", "leaf", "depth"):
        bad = np.nonzero(a[f] != b[f])[0]
        assert bad.size == 0, "field %s differs at nodes %s" % (f, bad[:5])
    for f in ("lo", "hi"):
        assert np.array_equal(a[f][:, :3], b[f][:, :3]), "%s differs" % f


def tree_invariants(canon, n):
    """Every triangle in exactly one leaf; children partition parents."""
    leaves = canon[canon["leaf"] == 1]
    cover = np.zeros(n, np.int32)
    for s, e in zip(leaves["start"], leaves["end"]):
        cover[s:e] += 1
    assert (cover == 1).all()
    assert canon[0]["start"] == 0 and canon[0]["end"] == n


def camera_small():
    return scenes.camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), fov_deg=60.0, aspect=1.0)


def single_light(kind="point"):
    if kind == "point":
        return abi.make_lights((0.1,) * 3, [dict(type=abi.RT_POINT_L, pos=(0.0, 4.0, -2.0))])
    if kind == "spot":
        return abi.make_lights((0.1,) * 3, [dict(type=abi.RT_SPOT_L, pos=(0.0, 4.0, -2.0),
                                                 dir=(0.0, -0.894427, 0.447214), angle=0.7)])
    return abi.make_lights((0.1,) * 3, [dict(type=abi.RT_DIR_L, dir=(0.3, -0.9, 0.3))])
