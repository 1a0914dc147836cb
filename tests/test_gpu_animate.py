"""Device-side animation (mangle, src/kernel/mangler.cl:12-32) and the
refit-only frame it feeds (renderer.cpp:53-70 with bvh_refit_only)."""
import numpy as np
import pytest

from helpers import assert_canon_equal, tiny_terrain, tree_invariants
from rtgb import capi, scenes

pytestmark = pytest.mark.gpu

# CUDA's sinf / cosf against the host's: a few ulp of values within [-1, 1]
# (positions are scaled by the wave height 0.2)
TOL = 2e-6


@pytest.mark.parametrize("arg", [1.0, 40.0])
def test_mangle_matches_oracle(ctx, orc, arg):
    ter = tiny_terrain(96, 48, 6)
    sc = ter.scene(0)
    g = capi.Scene(ctx, sc)
    g.mangle(arg, arg - 1.0, 0.2)
    gp, gn = g.read_vertices(sc.n_verts)
    op, on = orc.mangle(sc.pos4, sc.nrm4, arg, arg - 1.0, 0.2)
    # untouched components are exactly the inputs
    for c in (0, 2, 3):
        assert np.array_equal(gp[:, c], sc.pos4[:, c])
    assert np.array_equal(gn[:, 1], sc.nrm4[:, 1])
    assert np.abs(gp[:, 1] - op[:, 1]).max() <= TOL
    assert np.abs(gn[:, [0, 2]] - on[:, [0, 2]]).max() <= TOL
    assert np.mean(gp[:, 1] == op[:, 1]) > 0.5   # most are bit-identical


def test_refit_after_mangle_equals_oracle(ctx, orc):
    """Build, animate on the device, refit: the tree (topology of the build,
    boxes of the new positions) equals the oracle's refit of the same
    positions, bit for bit."""
    ter = tiny_terrain(128, 64, 8)
    sc = ter.scene(0)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    for f in (1.0, 2.0, 3.0):
        g.mangle(f, f - 1.0, 0.2)
        g.refit()
        gp, gn = g.read_vertices(sc.n_verts)
        orc.set_positions(o.h, gp.ctypes.data, gn.ctypes.data)
        orc.refit(o.h)
    gc = g.canon()
    assert_canon_equal(gc, o.canon())
    tree_invariants(gc, sc.n_tris)
    assert ctx.device_status() == 0


def test_mangle_refit_render_frame_mid_scale(ctx, orc):
    """The 1,240,576-triangle terrain animated by mangle and refit: the tree
    after refit equals the oracle's refit of the device positions."""
    ter = scenes.workload_mid()["terrain"]
    sc = ter.scene(0)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    g.mangle(5.0, 4.0, 0.2)
    g.refit()
    gp, gn = g.read_vertices(sc.n_verts)
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    orc.set_positions(o.h, gp.ctypes.data, gn.ctypes.data)
    orc.refit(o.h)
    assert_canon_equal(g.canon(), o.canon())
    assert ctx.device_status() == 0
