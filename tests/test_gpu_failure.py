"""Failure detection on the GPU without a fault: a device-side bounded wait
made to run out.  One radix-pass tile is launched without its predecessor,
so the predecessor's look-back word is a flag that nothing sets; the wait
gives up after its limit, the kernel reports RT_DEV_TIMEOUT and returns, the
host maps it to RT_ERR_TIMEOUT, and the context keeps working."""
import numpy as np
import pytest

import pyoracle
from rtgb import abi, capi, scenes

pytestmark = pytest.mark.gpu


def test_lookback_wait_times_out_and_context_survives(ctx, orc):
    assert ctx.device_status() == 0
    rc = ctx.selftest_wait_timeout()
    assert rc == abi.RT_ERR_TIMEOUT
    assert b"timed out" in ctx.lib.rt_last_error()
    bits = ctx.device_status()          # reads and clears
    assert bits & abi.RT_DEV_TIMEOUT
    assert ctx.device_status() == 0
    # the same context renders correctly afterwards
    sc = scenes.soup(3000, seed=21)
    cam = scenes.camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0))
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    w = h = 128
    rgba_d, img_d = ctx.alloc(4 * w * h), ctx.alloc(12 * w * h)
    g.render(cam, w, h, 3, rgba_d, img_d)
    ctx.sync()
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    rimg, _ = o.render(cam, w, h, 3)
    assert np.array_equal(img_d.read(np.uint32).reshape(-1, 3), rimg)
    assert ctx.device_status() == 0
    g.close()


def test_timeout_on_a_second_stream(ctx):
    """The same on a stream of the caller's: the status is the context's."""
    s = ctx.stream_create()
    try:
        assert ctx.selftest_wait_timeout(s) == abi.RT_ERR_TIMEOUT
        assert ctx.device_status() & abi.RT_DEV_TIMEOUT
        assert ctx.device_status() == 0
    finally:
        ctx.stream_destroy(s)
