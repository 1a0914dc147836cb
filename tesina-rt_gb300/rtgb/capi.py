"""ctypes binding of librt_cuda.so (include/rt_cuda.h) and thin Python helpers.

Every call goes through the C ABI; there is no Python or CPU implementation
of any compute entry point.  ``load()`` raises if the library is missing, and
compute calls raise ``RtError`` when the library reports a failure (for
example RT_ERR_CUDA when no GPU is present).
"""
import ctypes as C
import os

import numpy as np

from . import abi

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "librt_cuda.so")

P, I32, U32, SZ, F = C.c_void_p, C.c_int32, C.c_uint32, C.c_size_t, C.c_float

# name -> (restype, argtypes); the list of every exported entry point
SIGNATURES = {
    "rt_last_error": (C.c_char_p, []),
    "rt_camera_set": (I32, [P, P, P, P, F, F, I32]),
    "rt_init": (I32, [C.POINTER(P), I32]),
    "rt_shutdown": (I32, [P]),
    "rt_device_status": (I32, [P, C.POINTER(U32)]),
    "rt_selftest_wait_timeout": (I32, [P, P]),
    "rt_stream_create": (I32, [P, C.POINTER(P)]),
    "rt_stream_destroy": (I32, [P, P]),
    "rt_stream_sync": (I32, [P, P]),
    "rt_buf_alloc": (I32, [P, SZ, C.POINTER(P)]),
    "rt_buf_free": (I32, [P, P]),
    "rt_buf_write": (I32, [P, P, P, SZ, P]),
    "rt_buf_read": (I32, [P, P, P, SZ, P]),
    "rt_buf_copy": (I32, [P, P, P, SZ, P]),
    "rt_buf_zero": (I32, [P, P, SZ, P]),
    "rt_scene_create": (I32, [P, C.POINTER(P)]),
    "rt_scene_destroy": (I32, [P, P]),
    "rt_scene_upload": (I32, [P, P, P, P]),
    "rt_scene_update_vertices": (I32, [P, P, P, P, U32, P]),
    "rt_scene_update_vertices_device": (I32, [P, P, P, P, U32, P]),
    "rt_scene_set_lights": (I32, [P, P, P]),
    "rt_scene_buffers": (I32, [P, P, P, P, P, P, P]),
    "rt_scene_read_sort": (I32, [P, P, P, P, P]),
    "rt_scene_read_orig": (I32, [P, P, P]),
    "rt_bvh_build_lbvh": (I32, [P, P, P, P]),
    "rt_bvh_refit_lbvh": (I32, [P, P, P]),
    "rt_bvh_build_sah": (I32, [P, P, P]),
    "rt_scene_mangle": (I32, [P, P, F, F, F, P]),
    "rt_obj_load": (I32, [C.c_char_p, C.POINTER(P)]),
    "rt_obj_info": (I32, [P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]),
    "rt_obj_copy": (I32, [P, P, P, P, P]),
    "rt_obj_free": (I32, [P]),
    "rt_instances_create": (I32, [P, P, I32, P, P, P, I32, P, C.POINTER(P)]),
    "rt_instances_set_transforms": (I32, [P, P, P, P]),
    "rt_instances_render": (I32, [P, P, P, I32, I32, I32, P, P, P, P]),
    "rt_instances_destroy": (I32, [P, P]),
    "rt_bvh_export": (I32, [P, P, P, U32, C.POINTER(U32)]),
    "rt_bvh_last_time_ms": (I32, [P, P, C.POINTER(F)]),
    "rt_gen_primary": (I32, [P, P, I32, I32, I32, I32, P, SZ, SZ, P, P]),
    "rt_trace": (I32, [P, P, P, I32, P, I32, P]),
    "rt_shadow_trace": (I32, [P, P, P, I32, P, I32, P]),
    "rt_shade": (I32, [P, P, P, P, I32, P, I32, P]),
    "rt_gen_secondary": (I32, [P, P, P, I32, P, P, I32, P, P, P]),
    "rt_fb_clear": (I32, [P, P, SZ, P]),
    "rt_fb_copy": (I32, [P, P, P, SZ, P]),
    "rt_render": (I32, [P, P, P, I32, I32, I32, P, P, P, P]),
    "rt_render_host": (I32, [P, P, P, P, U32, P, P, I32, I32, I32, P, P, P]),
    "rt_render_host_async": (I32, [P, P, P, P, U32, P, P, I32, I32, I32, P, P, P]),
    "rt_render_host_wait": (I32, [P, P]),
    "rt_sort_pairs_noalloc": (I32, [P, P, P, P, P, U32, I32, P]),
    "rt_render_variants": (I32, [C.POINTER(I32)]),
    "rt_render_variant_info": (I32, [P, I32, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)]),
    "rt_render_variant_pooled": (I32, [I32, C.POINTER(I32)]),
    "rt_set_render_config": (I32, [P, P]),
    "rt_get_render_config": (I32, [P, P]),
    "rt_autotune_render": (I32, [P, P, P, I32, I32, I32, I32, P, C.POINTER(F)]),
    "rt_batch_create": (I32, [P, C.POINTER(P)]),
    "rt_batch_destroy": (I32, [P, P]),
    "rt_batch_set": (I32, [P, P, P, I32, P]),
    "rt_batch_build": (I32, [P, P, P]),
    "rt_batch_render": (I32, [P, P, P, P, P]),
    "rt_batch_capture": (I32, [P, P, P, P]),
    "rt_batch_replay": (I32, [P, P, P]),
    "rt_batch_info": (I32, [P, P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]),
    "rt_batch_profile": (I32, [P, P, I32]),
    "rt_batch_stage_times": (I32, [P, P, P]),
    "rt_server_create": (I32, [P, P, C.POINTER(P)]),
    "rt_server_destroy": (I32, [P]),
    "rt_server_add_scene": (I32, [P, P, C.POINTER(C.c_uint64)]),
    "rt_server_submit": (I32, [P, P, C.POINTER(C.c_uint64)]),
    "rt_server_upload": (I32, [P, P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "rt_server_result": (I32, [P, C.c_uint64, P, P]),
    "rt_server_get_stats": (I32, [P, P]),
    "rt_server_reset_stats": (I32, [P]),
}


class RtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rt error %d: %s" % (code, msg))
        self.code = code


_LIB = None


def load(path=None):
    """Load librt_cuda.so (fails loudly if it has not been built)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("librt_cuda.so not built (%s): run __graft_entry__.build()" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(lib, code):
    if code != 0:
        raise RtError(code, lib.rt_last_error().decode(errors="replace"))
    return code


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


class Context:
    """An rt_ctx on one GPU."""

    def __init__(self, device=0):
        self.lib = load()
        h = P()
        check(self.lib, self.lib.rt_init(C.byref(h), device))
        self.h = h

    def close(self):
        if self.h:
            self.lib.rt_shutdown(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # device buffers ------------------------------------------------------
    def alloc(self, nbytes):
        d = P()
        check(self.lib, self.lib.rt_buf_alloc(self.h, nbytes, C.byref(d)))
        return DeviceBuffer(self, d, nbytes)

    def to_device(self, arr, stream=None):
        arr = np.ascontiguousarray(arr)
        b = self.alloc(arr.nbytes)
        check(self.lib, self.lib.rt_buf_write(self.h, b.ptr, _p(arr), arr.nbytes, stream))
        return b

    def sync(self, stream=None):
        check(self.lib, self.lib.rt_stream_sync(self.h, stream))

    def render_host_wait(self, stream=None, raise_on_error=True):
        """Waits for the frame rt_render_host_async queued on `stream`."""
        r = self.lib.rt_render_host_wait(self.h, stream)
        if raise_on_error:
            check(self.lib, r)
        return r

    def stream_create(self):
        """A new non-blocking stream of the context (rt_stream handle)."""
        s = P()
        check(self.lib, self.lib.rt_stream_create(self.h, C.byref(s)))
        return s

    def stream_destroy(self, s):
        check(self.lib, self.lib.rt_stream_destroy(self.h, s))

    def device_status(self):
        bits = U32(0)
        check(self.lib, self.lib.rt_device_status(self.h, C.byref(bits)))
        return bits.value

    def selftest_wait_timeout(self, stream=None):
        """rt_selftest_wait_timeout: the raw status (RT_ERR_TIMEOUT when the
        device wait gave up, as it should)."""
        return self.lib.rt_selftest_wait_timeout(self.h, stream)

    # stage-wise pipeline ---------------------------------------------------
    def gen_primary(self, cam, w, h, out_buf, count=None, offset=0, quad=32, stream=None):
        count = w * h if count is None else count
        check(self.lib, self.lib.rt_gen_primary(self.h, C.byref(cam), w, h, quad, 1, None, count,
                                                offset, out_buf.ptr, stream))

    def render_config(self):
        cfg = abi.RenderConfig()
        check(self.lib, self.lib.rt_get_render_config(self.h, C.byref(cfg)))
        return cfg

    def set_render_config(self, variant, blocks_per_sm=0, chunk=32):
        cfg = abi.RenderConfig(variant, blocks_per_sm, chunk, 32)
        check(self.lib, self.lib.rt_set_render_config(self.h, C.byref(cfg)))

    def variants(self):
        n = I32(0)
        check(self.lib, self.lib.rt_render_variants(C.byref(n)))
        out = []
        for v in range(n.value):
            t, m, o = I32(0), I32(0), I32(0)
            check(self.lib, self.lib.rt_render_variant_info(self.h, v, C.byref(t), C.byref(m),
                                                            C.byref(o)))
            out.append((t.value, m.value, o.value))
        return out

    def variant_pooled(self, v):
        p = I32(0)
        check(self.lib, self.lib.rt_render_variant_pooled(v, C.byref(p)))
        return bool(p.value)

    def fb_copy(self, img_buf, rgba_buf, pixels, stream=None):
        check(self.lib, self.lib.rt_fb_copy(self.h, img_buf.ptr, rgba_buf.ptr, pixels, stream))


class DeviceBuffer:
    def __init__(self, ctx, ptr, nbytes):
        self.ctx, self.ptr, self.nbytes = ctx, ptr, nbytes

    def read(self, dtype, count=None, stream=None):
        dtype = np.dtype(dtype)
        count = self.nbytes // dtype.itemsize if count is None else count
        out = np.empty(count, dtype)
        check(self.ctx.lib, self.ctx.lib.rt_buf_read(self.ctx.h, _p(out), self.ptr,
                                                     out.nbytes, stream))
        return out

    def write(self, arr, stream=None):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        check(self.ctx.lib, self.ctx.lib.rt_buf_write(self.ctx.h, self.ptr, _p(arr), arr.nbytes,
                                                      stream))

    def zero(self, stream=None):
        check(self.ctx.lib, self.ctx.lib.rt_buf_zero(self.ctx.h, self.ptr, self.nbytes, stream))

    def free(self):
        if self.ptr:
            self.ctx.lib.rt_buf_free(self.ctx.h, self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            if self.ctx.h:
                self.free()
        except Exception:
            pass


def scene_desc(sc):
    d = abi.SceneDesc()
    d.h_vertices = _p(sc.pos4)
    d.vertex_count = sc.n_verts
    d.vertex_stride = 16
    d.position_offset = 0
    d.normal_offset = 0
    d.h_normals = _p(sc.nrm4)
    d.h_indices = _p(sc.idx)
    d.triangle_count = sc.n_tris
    d.material_count = sc.mats.shape[0]
    d.h_materials = _p(sc.mats)
    d.h_material_map = _p(sc.mat_map)
    d.lights = sc.lights
    return d


class Scene:
    """An rt_scene: upload, LBVH build, render, parity read-outs."""

    def __init__(self, ctx, sc=None, stream=None):
        self.ctx, self.lib = ctx, ctx.lib
        h = P()
        check(self.lib, self.lib.rt_scene_create(ctx.h, C.byref(h)))
        self.h = h
        self.n = 0
        if sc is not None:
            self.upload(sc, stream)

    def upload(self, sc, stream=None):
        self._keep = sc
        d = scene_desc(sc)
        check(self.lib, self.lib.rt_scene_upload(self.ctx.h, self.h, C.byref(d), stream))
        self.n = sc.n_tris

    def update_vertices(self, pos4, nrm4=None, stream=None):
        check(self.lib, self.lib.rt_scene_update_vertices(self.ctx.h, self.h, _p(pos4), _p(nrm4),
                                                          pos4.shape[0], stream))

    def build(self, depth=30, min_leaf=1, stream=None):
        cfg = abi.BvhCfg(depth, min_leaf)
        check(self.lib, self.lib.rt_bvh_build_lbvh(self.ctx.h, self.h, C.byref(cfg), stream))

    def refit(self, stream=None):
        check(self.lib, self.lib.rt_bvh_refit_lbvh(self.ctx.h, self.h, stream))

    def build_sah(self, stream=None):
        """The reference's CPU SAH BVH, on the host, then on the device."""
        check(self.lib, self.lib.rt_bvh_build_sah(self.ctx.h, self.h, stream))

    def mangle(self, arg, last_arg=-1000.0, height=0.2, stream=None):
        """Device-side vertex animation (mangler.cl); follow with refit() or build()."""
        check(self.lib, self.lib.rt_scene_mangle(self.ctx.h, self.h, arg, last_arg, height,
                                                 stream))

    def last_build_ms(self):
        ms = F(0)
        check(self.lib, self.lib.rt_bvh_last_time_ms(self.ctx.h, self.h, C.byref(ms)))
        return ms.value

    def sort_arrays(self):
        n = self.n
        keys, perm, sk, orig = (np.zeros(n, np.uint32) for _ in range(4))
        check(self.lib, self.lib.rt_scene_read_sort(self.ctx.h, self.h, _p(keys), _p(perm), _p(sk)))
        check(self.lib, self.lib.rt_scene_read_orig(self.ctx.h, self.h, _p(orig)))
        return keys, perm, sk, orig

    def canon(self):
        cnt = U32(0)
        check(self.lib, self.lib.rt_bvh_export(self.ctx.h, self.h, None, 0, C.byref(cnt)))
        out = np.zeros(cnt.value, abi.CANON_DTYPE)
        check(self.lib, self.lib.rt_bvh_export(self.ctx.h, self.h, _p(out), cnt.value, C.byref(cnt)))
        return out

    def buffers(self):
        idx, mp, pos, nrm = P(), P(), P(), P()
        n = U32(0)
        check(self.lib, self.lib.rt_scene_buffers(self.ctx.h, self.h, C.byref(idx), C.byref(mp),
                                                  C.byref(pos), C.byref(nrm), C.byref(n)))
        return idx, mp, pos, nrm, n.value

    def read_sorted_buffers(self):
        idx, mp, _, _, n = self.buffers()
        a = np.zeros((n, 3), np.uint32)
        m = np.zeros(n, np.uint32)
        check(self.lib, self.lib.rt_buf_read(self.ctx.h, _p(a), idx, a.nbytes, None))
        check(self.lib, self.lib.rt_buf_read(self.ctx.h, _p(m), mp, m.nbytes, None))
        return a, m

    def read_vertices(self, n_verts):
        """Device positions and normals (float32 [V, 4] each)."""
        _, _, pos, nrm, _ = self.buffers()
        p = np.zeros((n_verts, 4), np.float32)
        q = np.zeros((n_verts, 4), np.float32)
        check(self.lib, self.lib.rt_buf_read(self.ctx.h, _p(p), pos, p.nbytes, None))
        check(self.lib, self.lib.rt_buf_read(self.ctx.h, _p(q), nrm, q.nbytes, None))
        return p, q

    # stage-wise --------------------------------------------------------------
    def trace(self, smp_buf, n, hit_buf, stream=None):
        check(self.lib, self.lib.rt_trace(self.ctx.h, self.h, smp_buf.ptr, n, hit_buf.ptr, 0, stream))

    def shadow(self, smp_buf, n, hit_buf, stream=None):
        check(self.lib, self.lib.rt_shadow_trace(self.ctx.h, self.h, smp_buf.ptr, n, hit_buf.ptr, 0,
                                                 stream))

    def shade(self, smp_buf, hit_buf, n, img_buf, primary=1, stream=None):
        check(self.lib, self.lib.rt_shade(self.ctx.h, self.h, smp_buf.ptr, hit_buf.ptr, n,
                                          img_buf.ptr, primary, stream))

    def gen_secondary(self, in_buf, n, hit_buf, out_buf, max_out, count_buf, stream=None):
        hc = I32(0)
        check(self.lib, self.lib.rt_gen_secondary(self.ctx.h, self.h, in_buf.ptr, n, hit_buf.ptr,
                                                  out_buf.ptr, max_out, count_buf.ptr,
                                                  C.byref(hc), stream))
        return hc.value

    # fused ----------------------------------------------------------------
    def render(self, cam, w, h, max_bounces, rgba_buf, img_buf=None, stats_buf=None, stream=None):
        check(self.lib, self.lib.rt_render(self.ctx.h, self.h, C.byref(cam), w, h, max_bounces,
                                           rgba_buf.ptr, img_buf.ptr if img_buf else None,
                                           stats_buf.ptr if stats_buf else None, stream))

    def render_host(self, cam, w, h, max_bounces, pos4=None, nrm4=None, depth=30, min_leaf=1,
                    rgba=None, stream=None):
        if rgba is None:
            rgba = np.zeros((h * w, 4), np.uint8)
        st = abi.RenderStats()
        cfg = abi.BvhCfg(depth, min_leaf)
        V = pos4.shape[0] if pos4 is not None else 0
        check(self.lib, self.lib.rt_render_host(self.ctx.h, self.h, _p(pos4), _p(nrm4), V,
                                                C.byref(cfg), C.byref(cam), w, h, max_bounces,
                                                _p(rgba), C.byref(st), stream))
        return rgba, st

    def render_host_async(self, cam, w, h, max_bounces, pos4=None, nrm4=None, depth=30,
                          min_leaf=1, rgba=None, stats=None, stream=None):
        """Queues a render_host frame on `stream` and returns (rgba, stats) at
        once; both are filled by Context.render_host_wait(stream), and they,
        pos4 and nrm4 must stay alive until then."""
        if rgba is None:
            rgba = np.zeros((h * w, 4), np.uint8)
        if stats is None:
            stats = abi.RenderStats()
        cfg = abi.BvhCfg(depth, min_leaf)
        V = pos4.shape[0] if pos4 is not None else 0
        check(self.lib, self.lib.rt_render_host_async(self.ctx.h, self.h, _p(pos4), _p(nrm4), V,
                                                      C.byref(cfg), C.byref(cam), w, h,
                                                      max_bounces, _p(rgba), C.byref(stats),
                                                      stream))
        return rgba, stats

    def autotune(self, cam, w, h, max_bounces, trials=2):
        cfg = abi.RenderConfig()
        ms = F(0)
        check(self.lib, self.lib.rt_autotune_render(self.ctx.h, self.h, C.byref(cam), w, h,
                                                    max_bounces, trials, C.byref(cfg),
                                                    C.byref(ms)))
        return cfg, ms.value

    def close(self):
        if self.h:
            self.lib.rt_scene_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            if self.ctx.h:
                self.close()
        except Exception:
            pass


class Batch:
    """An rt_batch: views of uploaded scenes, built and rendered together."""

    def __init__(self, ctx):
        self.ctx, self.lib = ctx, ctx.lib
        h = P()
        check(self.lib, self.lib.rt_batch_create(ctx.h, C.byref(h)))
        self.h = h

    def set(self, items, depth=30, min_leaf=1):
        """items: list of (Scene, Camera, width, height, max_bounces)."""
        n = len(items)
        arr = (abi.BatchView * n)()
        off = 0
        self.offsets = []
        for k, (sc, cam, w, h, b) in enumerate(items):
            arr[k].scene = sc.h
            arr[k].cam = cam
            arr[k].width, arr[k].height, arr[k].max_bounces = w, h, b
            arr[k].rgba_offset = off
            self.offsets.append((off, w, h))
            off += w * h
        self.pixels = off
        self._items = items
        cfg = abi.BvhCfg(depth, min_leaf)
        check(self.lib, self.lib.rt_batch_set(self.ctx.h, self.h, arr, n, C.byref(cfg)))

    def build(self, stream=None):
        check(self.lib, self.lib.rt_batch_build(self.ctx.h, self.h, stream))

    def render(self, rgba_buf, stats_buf=None, stream=None):
        check(self.lib, self.lib.rt_batch_render(self.ctx.h, self.h, rgba_buf.ptr,
                                                 stats_buf.ptr if stats_buf else None, stream))

    def capture(self, rgba_buf, stats_buf=None):
        check(self.lib, self.lib.rt_batch_capture(self.ctx.h, self.h, rgba_buf.ptr,
                                                  stats_buf.ptr if stats_buf else None))

    def replay(self, stream=None):
        check(self.lib, self.lib.rt_batch_replay(self.ctx.h, self.h, stream))

    def profile(self, enable=True):
        check(self.lib, self.lib.rt_batch_profile(self.ctx.h, self.h, int(enable)))

    def stage_times(self):
        ms = (F * 6)()
        check(self.lib, self.lib.rt_batch_stage_times(self.ctx.h, self.h, ms))
        return dict(zip(["init", "bounds", "morton", "sort", "permute", "emit"], list(ms)))

    def info(self):
        a, b, c = U32(0), U32(0), U32(0)
        check(self.lib, self.lib.rt_batch_info(self.ctx.h, self.h, C.byref(a), C.byref(b),
                                               C.byref(c)))
        return a.value, b.value, c.value

    def close(self):
        if self.h:
            self.lib.rt_batch_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            if self.ctx.h:
                self.close()
        except Exception:
            pass


class Server:
    """An rt_server: resident scenes, admission, continuous batching."""

    def __init__(self, ctx, budget=120 << 30, arena=2 << 30, max_views=256, max_inflight=2,
                 max_scenes=0):
        self.ctx, self.lib = ctx, ctx.lib
        cfg = abi.ServerCfg(budget, arena, max_views, max_inflight, max_scenes, 0)
        h = P()
        check(self.lib, self.lib.rt_server_create(ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._uploads = {}

    def add_scene(self, sc):
        d = scene_desc(sc)
        sid = C.c_uint64(0)
        check(self.lib, self.lib.rt_server_add_scene(self.h, C.byref(d), C.byref(sid)))
        return sid.value

    def submit_render(self, scene_id, cam, w, h, bounces):
        r = abi.Request(abi.RT_REQ_RENDER, bounces, w, h, scene_id, cam, None)
        t = C.c_uint64(0)
        check(self.lib, self.lib.rt_server_submit(self.h, C.byref(r), C.byref(t)))
        return t.value

    def submit_upload(self, sc):
        d = scene_desc(sc)
        r = abi.Request(abi.RT_REQ_UPLOAD, 0, 0, 0, 0, abi.Camera(), C.addressof(d))
        t = C.c_uint64(0)
        check(self.lib, self.lib.rt_server_submit(self.h, C.byref(r), C.byref(t)))
        self._uploads[t.value] = (d, sc)        # host data stays alive until done
        return t.value

    def upload(self, sc):
        """Upload request returning (ticket, scene id); the id is usable at once."""
        d = scene_desc(sc)
        t, sid = C.c_uint64(0), C.c_uint64(0)
        check(self.lib, self.lib.rt_server_upload(self.h, C.byref(d), C.byref(t), C.byref(sid)))
        self._uploads[t.value] = (d, sc)
        return t.value, sid.value

    def result(self, ticket, w=0, h=0, raise_on_error=True):
        rgba = np.zeros((h * w, 4), np.uint8) if w * h else None
        info = abi.RequestInfo()
        r = self.lib.rt_server_result(self.h, ticket, _p(rgba), C.byref(info))
        self._uploads.pop(ticket, None)
        if r and raise_on_error:
            raise RtError(r, self.lib.rt_last_error().decode(errors="replace"))
        return rgba, info

    def stats(self):
        st = abi.ServerStats()
        check(self.lib, self.lib.rt_server_get_stats(self.h, C.byref(st)))
        return st

    def reset_stats(self):
        check(self.lib, self.lib.rt_server_reset_stats(self.h))

    def close(self):
        if self.h:
            self.lib.rt_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Instances:
    """Multi-root scene: instances of built Scenes under 4x4 transforms."""

    def __init__(self, ctx, scenes_, inst_scene, tr, tr_inv, lights):
        self.ctx, self.lib = ctx, ctx.lib
        self._scenes = list(scenes_)   # kept alive with the instance set
        arr = (P * len(self._scenes))(*[s.h for s in self._scenes])
        self._ins = np.ascontiguousarray(inst_scene, np.int32)
        t = np.ascontiguousarray(tr, np.float32)
        ti = np.ascontiguousarray(tr_inv, np.float32)
        self._lights = lights
        h = P()
        check(self.lib, self.lib.rt_instances_create(ctx.h, C.cast(arr, P), len(self._scenes),
                                                     _p(self._ins), _p(t), _p(ti),
                                                     self._ins.shape[0], C.byref(lights),
                                                     C.byref(h)))
        self.h = h

    def set_transforms(self, tr, tr_inv):
        t = np.ascontiguousarray(tr, np.float32)
        ti = np.ascontiguousarray(tr_inv, np.float32)
        check(self.lib, self.lib.rt_instances_set_transforms(self.ctx.h, self.h, _p(t), _p(ti)))

    def render(self, cam, w, h, max_bounces, rgba_buf, img_buf=None, stats_buf=None, stream=None):
        check(self.lib, self.lib.rt_instances_render(self.ctx.h, self.h, C.byref(cam), w, h,
                                                     max_bounces, rgba_buf.ptr,
                                                     img_buf.ptr if img_buf else None,
                                                     stats_buf.ptr if stats_buf else None, stream))

    def close(self):
        if self.h:
            self.lib.rt_instances_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

