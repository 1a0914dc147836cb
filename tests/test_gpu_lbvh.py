"""GPU parity of the LBVH build against the oracle (bit-exact)."""
import numpy as np
import pytest

from helpers import assert_canon_equal, tiny_terrain, tree_invariants
from rtgb import abi, capi, scenes

pytestmark = pytest.mark.gpu


def _both(ctx, orc, sc, depth=30, min_leaf=1):
    g = capi.Scene(ctx, sc)
    g.build(depth, min_leaf)
    o = orc.new_scene(sc)
    o.build(depth, min_leaf, 0)
    return g, o


def _compare(g, o, n):
    gk, gp, gs, go = g.sort_arrays()
    ok, op, os_, oo = o.sort_arrays()
    assert np.array_equal(gk, ok), "Morton keys differ"
    assert np.array_equal(gs, os_), "sorted keys differ"
    assert np.array_equal(gp, op), "permutation differs (both sorts are stable)"
    assert np.array_equal(go, oo)
    gi, gm = g.read_sorted_buffers()
    oi, om = o.buffers()
    assert np.array_equal(gi, oi) and np.array_equal(gm, om), "permuted index/material buffers"
    gc, oc = g.canon(), o.canon()
    assert_canon_equal(gc, oc)
    tree_invariants(gc, n)


@pytest.mark.parametrize("seed", [0, 1])
def test_soup_10k(ctx, orc, seed):
    sc = scenes.soup(10000, seed=seed)
    g, o = _both(ctx, orc, sc)
    _compare(g, o, sc.n_tris)
    assert ctx.device_status() == 0


@pytest.mark.parametrize("depth,min_leaf", [(30, 1), (30, 4), (10, 1), (16, 2), (32, 1), (1, 1),
                                            (8, 256)])
def test_terrain_duplicates(ctx, orc, depth, min_leaf):
    """Heightfield + spheres: many equal Morton keys, large leaves."""
    sc = tiny_terrain().scene(0)
    g, o = _both(ctx, orc, sc, depth, min_leaf)
    _compare(g, o, sc.n_tris)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 17, 2047, 2048, 2049, 4095, 4096, 4097, 8193])
def test_small_and_ragged_sizes(ctx, orc, n):
    sc = scenes.soup(n, seed=n)
    g, o = _both(ctx, orc, sc)
    _compare(g, o, n)


def test_all_equal_keys(ctx, orc):
    """Every triangle has the same centroid: the root is one leaf."""
    rng = np.random.default_rng(3)
    n = 300
    base = rng.normal(size=(3, 3)).astype(np.float32)
    v = np.tile(base[None], (n, 1, 1))
    v[:, 0, 0] += np.float32(0.0)
    pos = np.zeros((3 * n, 4), np.float32)
    pos[:, :3] = v.reshape(-1, 3)
    nrm = np.zeros_like(pos)
    nrm[:, 1] = 1
    sc0 = scenes.soup(n, seed=1)
    sc = scenes.Scene(pos, nrm, sc0.idx, sc0.mats, sc0.mat_map, sc0.lights)
    g, o = _both(ctx, orc, sc)
    _compare(g, o, n)
    c = g.canon()
    assert c.shape[0] == 1 and c[0]["leaf"] == 1 and c[0]["end"] == n


def test_flat_axis(ctx, orc):
    """A scene flat in y (hi == lo): NaN slices map to Morton cell 0."""
    sc = scenes.soup(5000, seed=7)
    sc.pos4[:, 1] = 0.25
    g, o = _both(ctx, orc, sc)
    _compare(g, o, sc.n_tris)


def test_rebuild_composes_permutation(ctx, orc):
    """A second build starts from the previously sorted order (in-place
    permutation of the index buffer and material map, as the reference)."""
    sc = tiny_terrain(48, 24, 3).scene(0)
    g, o = _both(ctx, orc, sc)
    ter = tiny_terrain(48, 24, 3)
    pos, nrm = ter.frame_vertices(5)
    g.update_vertices(pos, nrm)
    g.build(30, 1)
    orc.set_positions(o.h, pos.ctypes.data, nrm.ctypes.data)
    o.build(30, 1, 0)
    _compare(g, o, sc.n_tris)


def test_refit_matches_oracle(ctx, orc):
    ter = tiny_terrain(64, 32, 4)
    sc = ter.scene(0)
    g, o = _both(ctx, orc, sc)
    pos, nrm = ter.frame_vertices(9)
    g.update_vertices(pos, nrm)
    g.refit()
    orc.set_positions(o.h, pos.ctypes.data, nrm.ctypes.data)
    orc.refit(o.h)
    assert_canon_equal(g.canon(), o.canon())


def test_build_full_mid_scale_properties(ctx, orc):
    """1,240,000-triangle terrain: properties at full size, exact keys."""
    w = scenes.workload_mid()
    sc = w["terrain"].scene(0)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    keys, perm, sk, orig = g.sort_arrays()
    o = orc.new_scene(sc)
    ok = np.zeros(sc.n_tris, np.uint32)
    orc.morton_keys(o.h, 30, ok.ctypes.data, None, None)
    assert np.array_equal(keys, ok)
    assert (np.diff(sk.astype(np.int64)) >= 0).all()
    assert np.array_equal(np.sort(perm), np.arange(sc.n_tris, dtype=np.uint32))
    assert np.array_equal(keys[perm], sk)
    # stability: equal keys keep ascending original ids
    same = sk[1:] == sk[:-1]
    assert (perm[1:][same] > perm[:-1][same]).all()
    c = g.canon()
    tree_invariants(c, sc.n_tris)
    assert ctx.device_status() == 0


@pytest.mark.parametrize("frame", [0, 11])
def test_mid_scale_animated_frames_equal_oracle(ctx, orc, frame):
    """The 1,240,576-triangle terrain at animation frames 0 and 11, rebuilt
    from the previous frame's sorted order as the per-frame loop does: the
    whole tree equals the oracle's.  Frame 11 has blocks of the emit whose
    leftover runs outnumber a warp and all reach outside the block."""
    ter = scenes.workload_mid()["terrain"]
    g = capi.Scene(ctx, ter.scene(0))
    g.build(30, 1)
    pos, nrm = ter.frame_vertices(frame)
    g.update_vertices(pos, nrm)
    g.build(30, 1)
    assert ctx.device_status() == 0
    sc = scenes.Scene(pos, nrm, ter.idx, ter.mats, ter.mat_map, ter.lights)
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    assert np.array_equal(g.sort_arrays()[2], o.sort_arrays()[2])
    gc = g.canon()
    assert_canon_equal(gc, o.canon())
    tree_invariants(gc, sc.n_tris)


def test_calls_on_one_scene_ordered_across_streams(ctx):
    """Calls on one scene run in call order whatever streams they name: a
    build of the 1,240,576-triangle terrain on the context's stream, two more
    issued at once on two other streams, then a render on a third, give the
    tree and image of the same calls on one stream."""
    wl = scenes.workload_mid()
    sc = wl["terrain"].scene(0)
    w, h, nb, cam = 480, 270, 3, wl["camera"]
    ref = capi.Scene(ctx, sc)
    for _ in range(3):
        ref.build(30, 1)
    want = ctx.alloc(4 * w * h)
    ref.render(cam, w, h, nb, want)
    ctx.sync()
    streams = [ctx.stream_create() for _ in range(3)]
    try:
        g = capi.Scene(ctx, sc)
        g.build(30, 1)
        g.build(30, 1, stream=streams[0])
        g.build(30, 1, stream=streams[1])
        got = ctx.alloc(4 * w * h)
        g.render(cam, w, h, nb, got, stream=streams[2])
        assert_canon_equal(g.canon(), ref.canon())
        ctx.sync(streams[2])
        assert np.array_equal(got.read(np.uint8), want.read(np.uint8))
        assert np.array_equal(g.sort_arrays()[2], ref.sort_arrays()[2])
    finally:
        for s in streams:
            ctx.stream_destroy(s)
    assert ctx.device_status() == 0


def test_invalid_inputs_rejected(ctx):
    sc = scenes.soup(100, seed=1)
    bad = scenes.Scene(sc.pos4, sc.nrm4, sc.idx.copy(), sc.mats, sc.mat_map, sc.lights)
    bad.idx[5, 1] = sc.n_verts + 10
    with pytest.raises(capi.RtError) as e:
        capi.Scene(ctx, bad)
    assert e.value.code == -2
    mats = sc.mats.copy()
    mats["texture"][0] = 2
    with pytest.raises(capi.RtError):   # textured materials are not rendered
        capi.Scene(ctx, scenes.Scene(sc.pos4, sc.nrm4, sc.idx, mats, sc.mat_map, sc.lights))
    g = capi.Scene(ctx, sc)
    with pytest.raises(capi.RtError) as e:
        g.build(33, 1)
    assert e.value.code == -2
    g2 = capi.Scene(ctx, sc)
    with pytest.raises(capi.RtError) as e:
        g2.canon()
    assert e.value.code == -6
