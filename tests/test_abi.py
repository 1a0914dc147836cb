"""The C ABI: the library builds, loads without a GPU and exports every
entry point that include/rt_cuda.h declares; struct layouts agree with the
Python mirrors."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from rtgb import abi, capi
from rtgb import build as rb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rt_cuda.h")


def _declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"RT_API\s+[\w\s\*]+?\b(rt_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    rb.build()
    return capi.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 35
    for n in names:
        assert hasattr(lib, n), n
        assert n in capi.SIGNATURES, n


def test_init_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.rt_init(C.byref(h), 0) == -3
    assert b"no CUDA device" in lib.rt_last_error()


def test_camera_set_is_host_only(lib):
    cam = abi.Camera()
    f3 = C.c_float * 3
    assert lib.rt_camera_set(C.byref(cam), f3(0, 0, -4), f3(0, 0, 1), f3(0, 1, 0),
                             C.c_float(1.0471976), C.c_float(1.0), 0) == 0
    assert abs(cam.right[0] - 0.57735) < 1e-4 and abs(cam.up[1] - 0.57735) < 1e-4
    assert lib.rt_camera_set(C.byref(cam), f3(0, 0, 0), f3(0, 0, 0), f3(0, 1, 0),
                             C.c_float(1.0), C.c_float(1.0), 0) == -2


def test_struct_layouts(tmp_path):
    prog = tmp_path / "layout.c"
    prog.write_text('''
#include <stdio.h>
#include <stddef.h>
#include "rt_cuda.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(rt_sample), sizeof(rt_hit),
         sizeof(rt_material), sizeof(rt_canon_node), sizeof(rt_lights), sizeof(rt_camera),
         offsetof(rt_hit, uv), offsetof(rt_hit, hit_point));
  printf("%zu %zu %zu\\n", sizeof(rt_scene_desc), offsetof(rt_scene_desc, lights),
         sizeof(rt_render_stats));
  return 0; }
''')
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)])
    a, b = subprocess.check_output([str(exe)], text=True).splitlines()
    vals = [int(x) for x in a.split()]
    assert vals[:6] == [abi.SAMPLE_DTYPE.itemsize, abi.HIT_DTYPE.itemsize,
                        abi.MATERIAL_DTYPE.itemsize, abi.CANON_DTYPE.itemsize,
                        C.sizeof(abi.Lights), C.sizeof(abi.Camera)]
    assert vals[6] == abi.HIT_DTYPE.fields["uv"][1]
    assert vals[7] == abi.HIT_DTYPE.fields["hit_point"][1]
    d = [int(x) for x in b.split()]
    assert d == [C.sizeof(abi.SceneDesc), abi.SceneDesc.lights.offset, C.sizeof(abi.RenderStats)]
