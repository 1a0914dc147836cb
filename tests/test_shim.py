"""The drop-in C++ classes (include/rt/*.hpp over librt_shim.so): a C++
program drives one frame stage by stage through BVHBuilder,
PrimaryRayGenerator, Tracer, RayShader, SecondaryRayGenerator and
FrameBuffer, in the reference renderer's tile and bounce loop
(tests/shim_frame.cpp); its image equals rt_render's and the oracle's."""
import os
import subprocess

import numpy as np
import pytest

import pyoracle
from helpers import tiny_terrain
from rtgb import build as rb
from rtgb import capi, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "tesina-rt_gb300")


def _program(tmp):
    """Builds the libraries (if stale) and the C++ frame program."""
    rb.build()
    exe = os.path.join(str(tmp), "shim_frame")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-Werror",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "shim_frame.cpp"),
           "-L", PKG, "-lrt_shim", "-lrt_cuda", "-Wl,-rpath," + PKG, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_headers_compile_and_link(tmp_path):
    """The headers compile warning-free and every class method the program
    calls resolves in librt_shim.so / librt_cuda.so."""
    assert os.path.exists(_program(tmp_path))


def _write_scene(d, sc, cam, w, h, bounces, tile, depth=30, min_leaf=1):
    sc.pos4.astype(np.float32).tofile(os.path.join(d, "pos4.bin"))
    sc.nrm4.astype(np.float32).tofile(os.path.join(d, "nrm4.bin"))
    sc.idx.astype(np.uint32).tofile(os.path.join(d, "idx.bin"))
    sc.mats.tofile(os.path.join(d, "mats.bin"))
    sc.mat_map.astype(np.uint32).tofile(os.path.join(d, "map.bin"))
    with open(os.path.join(d, "lights.bin"), "wb") as f:
        f.write(bytes(sc.lights))
    with open(os.path.join(d, "camera.bin"), "wb") as f:
        f.write(bytes(cam))
    np.array([w, h, bounces, tile, depth, min_leaf], np.int32).tofile(os.path.join(d, "params.bin"))


CASES = {
    "soup10k_512x512_d3": lambda: (scenes.workload_small()["scene"],
                                   scenes.workload_small()["camera"], 512, 512, 3, 65536),
    "terrain_2lights_d4": lambda: (tiny_terrain(96, 48, 12).scene(3),
                                   scenes.camera((0.0, 4.0, -10.0), (0.0, 0.0, 0.0),
                                                 aspect=320 / 180), 320, 180, 4, 20000),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_shim_frame_equals_render(ctx, orc, tmp_path, name):
    sc, cam, w, h, bounces, tile = CASES[name]()
    exe = _program(tmp_path)
    _write_scene(str(tmp_path), sc, cam, w, h, bounces, tile)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    n = w * h
    img = np.fromfile(os.path.join(tmp_path, "image.bin"), np.uint32).reshape(-1, 3)
    rgba = np.fromfile(os.path.join(tmp_path, "rgba.bin"), np.uint8).reshape(-1, 4)
    total, secondary = np.fromfile(os.path.join(tmp_path, "stats.bin"), np.uint64)
    # the same frame through rt_render (one fused launch)
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    rgba_d, img_d = ctx.alloc(4 * n), ctx.alloc(12 * n)
    st_d = ctx.alloc(32)
    st_d.zero()
    g.render(cam, w, h, bounces, rgba_d, img_d, st_d)
    ctx.sync()
    st = st_d.read(np.uint64)
    assert np.array_equal(img, img_d.read(np.uint32).reshape(-1, 3))
    assert np.array_equal(rgba, rgba_d.read(np.uint8).reshape(-1, 4))
    assert total == st[0] + st[1] and secondary == st[1] > 0
    # and the oracle
    o = orc.new_scene(sc)
    o.build(30, 1, 0)
    rimg, rst = o.render(cam, w, h, bounces)
    assert np.array_equal(img, rimg)
    assert np.array_equal(rgba, pyoracle.fb_copy(orc, rimg))
    assert secondary == rst.secondary_rays
    g.close()
