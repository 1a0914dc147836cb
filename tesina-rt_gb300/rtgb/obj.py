"""Wavefront OBJ scenes through the library's reader (rt_obj_load).

load() mirrors Scene::load_obj_file_as_aggregate + Scene::add_object
(src/rt/scene.cpp:441-468): the model becomes one aggregate mesh whose
object takes the material of its first group (Kd as diffuse, Ns / 1000 as
shininess, no reflection); write() emits a scene as OBJ text (positions,
normals, v//vn faces) for models the tests and the bench make themselves.
"""
import ctypes as C

import numpy as np

from rtgb import abi, capi

GROUP_DTYPE = np.dtype([("first_triangle", np.uint32), ("triangle_count", np.uint32),
                        ("diffuse", np.float32, 3), ("shininess", np.float32),
                        ("alpha", np.float32)])


def read(path):
    """(pos4 [V, 4], nrm4 [V, 4], idx [N, 3], groups) as the reader returns them."""
    lib = capi.load()
    h = C.c_void_p()
    capi.check(lib, lib.rt_obj_load(str(path).encode(), C.byref(h)))
    try:
        V, N, G = C.c_uint32(), C.c_uint32(), C.c_uint32()
        capi.check(lib, lib.rt_obj_info(h, C.byref(V), C.byref(N), C.byref(G)))
        pos = np.zeros((V.value, 4), np.float32)
        nrm = np.zeros((V.value, 4), np.float32)
        idx = np.zeros((N.value, 3), np.uint32)
        groups = np.zeros(G.value, GROUP_DTYPE)
        capi.check(lib, lib.rt_obj_copy(h, pos.ctypes.data, nrm.ctypes.data, idx.ctypes.data,
                                         groups.ctypes.data))
    finally:
        lib.rt_obj_free(h)
    return pos, nrm, idx, groups


def load(path, lights=None, reflectiveness=0.0):
    """A host Scene of the model, one material (its first group's)."""
    from rtgb import scenes
    pos, nrm, idx, groups = read(path)
    mats = np.zeros(1, dtype=abi.MATERIAL_DTYPE)
    mats["texture"] = -1
    mats["diffuse"][0, :3] = groups["diffuse"][0]
    mats["shininess"][0] = groups["shininess"][0]
    mats["reflectiveness"][0] = reflectiveness
    if lights is None:
        lights = abi.make_lights((0.1, 0.1, 0.1),
                                 [dict(type=abi.RT_POINT_L, pos=(0.0, 4.0, -2.0),
                                       color=(1.0, 1.0, 1.0))])
    return scenes.Scene(pos, nrm, idx, mats, np.zeros(idx.shape[0], np.uint32), lights)


def write(path, pos4, nrm4, idx):
    """OBJ text of a mesh: v and vn per vertex, faces as v//vn (1-based)."""
    with open(path, "w") as f:
        f.write("# written by rtgb.obj\n")
        np.savetxt(f, pos4[:, :3], fmt="v %.9g %.9g %.9g")
        np.savetxt(f, nrm4[:, :3], fmt="vn %.9g %.9g %.9g")
        i = idx.astype(np.int64) + 1
        np.savetxt(f, np.stack([i[:, 0], i[:, 0], i[:, 1], i[:, 1], i[:, 2], i[:, 2]], 1),
                   fmt="f %d//%d %d//%d %d//%d")
