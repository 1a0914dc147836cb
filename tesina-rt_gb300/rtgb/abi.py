"""ctypes / numpy mirrors of the structs in include/rt_cuda.h."""
import ctypes as C

import numpy as np

RT_MAX_LIGHTS = 8
RT_SPOT_L, RT_DIR_L, RT_POINT_L = 0, 1, 2
RT_OK, RT_ERR_TIMEOUT, RT_ERR_OVERFLOW = 0, -5, -7          # rt_status
RT_DEV_TIMEOUT, RT_DEV_OVERFLOW, RT_DEV_BADINDEX = 0x1, 0x2, 0x4   # device status bits


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("radius", C.c_float), ("angle", C.c_float),
                ("_pad0", C.c_float), ("pos", C.c_float * 4), ("dir", C.c_float * 4),
                ("color", C.c_float * 4)]


class Lights(C.Structure):
    _fields_ = [("ambient", C.c_float * 4), ("count", C.c_int32), ("_pad", C.c_int32 * 3),
                ("light", Light * RT_MAX_LIGHTS)]


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 4), ("dir", C.c_float * 4), ("right", C.c_float * 4),
                ("up", C.c_float * 4)]


class SceneDesc(C.Structure):
    _fields_ = [("h_vertices", C.c_void_p), ("vertex_count", C.c_uint32),
                ("vertex_stride", C.c_uint32), ("position_offset", C.c_uint32),
                ("normal_offset", C.c_uint32), ("h_normals", C.c_void_p),
                ("h_indices", C.c_void_p), ("triangle_count", C.c_uint32),
                ("material_count", C.c_uint32), ("h_materials", C.c_void_p),
                ("h_material_map", C.c_void_p), ("lights", Lights)]


class BvhCfg(C.Structure):
    _fields_ = [("depth", C.c_int32), ("min_leaf_size", C.c_int32)]


class RenderConfig(C.Structure):
    _fields_ = [("variant", C.c_int32), ("blocks_per_sm", C.c_int32), ("chunk", C.c_int32),
                ("stack_depth", C.c_int32)]

    def __repr__(self):
        return "RenderConfig(variant=%d, blocks_per_sm=%d, chunk=%d)" % (
            self.variant, self.blocks_per_sm, self.chunk)


class BatchView(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("cam", Camera), ("width", C.c_int32),
                ("height", C.c_int32), ("max_bounces", C.c_int32), ("rgba_offset", C.c_uint32)]


RT_REQ_RENDER, RT_REQ_UPLOAD = 0, 1


class ServerCfg(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("fb_arena_bytes", C.c_uint64),
                ("max_batch_views", C.c_int32), ("max_inflight", C.c_int32),
                ("max_scenes", C.c_int32), ("reserved", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("type", C.c_int32), ("max_bounces", C.c_int32), ("width", C.c_int32),
                ("height", C.c_int32), ("scene_id", C.c_uint64), ("cam", Camera),
                ("upload", C.c_void_p)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_views", C.c_int32), ("scene_id", C.c_uint64),
                ("submit_ms", C.c_double), ("start_ms", C.c_double), ("done_ms", C.c_double),
                ("rays", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("rejected", C.c_uint64), ("evicted", C.c_uint64),
                ("batches", C.c_uint64), ("rays", C.c_uint64), ("resident_scenes", C.c_uint64),
                ("resident_bytes", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_batch_views", C.c_double), ("first_submit_ms", C.c_double),
                ("last_done_ms", C.c_double)]


class RenderStats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("secondary_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("hits", C.c_uint64)]


MATERIAL_DTYPE = np.dtype([("diffuse", "<f4", 4), ("shininess", "<f4"),
                           ("reflectiveness", "<f4"), ("refractive_index", "<f4"),
                           ("texture", "<i4")])
assert MATERIAL_DTYPE.itemsize == 32

SAMPLE_DTYPE = np.dtype([("ori", "<f4", 4), ("dir", "<f4", 4), ("inv_dir", "<f4", 4),
                         ("tmin", "<f4"), ("tmax", "<f4"), ("_pad", "<f4", 2),
                         ("pixel", "<i4"), ("contribution", "<f4"), ("_pad2", "<i4", 2)])
assert SAMPLE_DTYPE.itemsize == 80

HIT_DTYPE = np.dtype([("hit", "u1"), ("shadow_hit", "u1"), ("inverse_n", "u1"),
                      ("reserved", "u1"), ("t", "<f4"), ("id", "<i4"), ("_pad0", "<f4"),
                      ("uv", "<f4", 2), ("_pad1", "<f4", 2), ("n", "<f4", 4),
                      ("hit_point", "<f4", 4)])
assert HIT_DTYPE.itemsize == 64

CANON_DTYPE = np.dtype([("start", "<u4"), ("end", "<u4"), ("leaf", "<u4"), ("depth", "<u4"),
                        ("lo", "<f4", 4), ("hi", "<f4", 4)])
assert CANON_DTYPE.itemsize == 48

PIXEL_SAMPLE_DTYPE = np.dtype([("ox", "<f4"), ("oy", "<f4"), ("contribution", "<f4")])

assert C.sizeof(Light) == 64
assert C.sizeof(Lights) == 32 + 64 * RT_MAX_LIGHTS
assert C.sizeof(Camera) == 64


def make_lights(ambient, lights):
    """lights: list of dicts {type, pos, dir, color, angle, radius}."""
    L = Lights()
    L.ambient[:3] = [float(a) for a in ambient]
    L.count = len(lights)
    assert 1 <= len(lights) <= RT_MAX_LIGHTS
    for i, d in enumerate(lights):
        li = L.light[i]
        li.type = int(d.get("type", RT_POINT_L))
        li.radius = float(d.get("radius", 0.0))
        li.angle = float(d.get("angle", 0.0))
        li.pos[:3] = [float(v) for v in d.get("pos", (0, 0, 0))]
        li.dir[:3] = [float(v) for v in d.get("dir", (0, 0, 1))]
        li.color[:3] = [float(v) for v in d.get("color", (1, 1, 1))]
    return L


def ptr(a):
    """Host pointer of a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)
