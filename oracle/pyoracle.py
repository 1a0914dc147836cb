"""ctypes bindings of the oracle libraries (test infrastructure only).

``Oracle`` wraps liboracle.so (the CPU restatement); ``RefKernels`` wraps
oracle/_ref/libref.so (the reference's own kernels compiled for the CPU),
which exists only where the reference checkout was available at build time.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "tesina-rt_gb300"))
from rtgb import abi  # noqa: E402

P = C.c_void_p
U32, I32, SZ, F = C.c_uint32, C.c_int32, C.c_size_t, C.c_float


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


class _Lib:
    def _bind(self, lib, name, res, args):
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
        return f


class Oracle(_Lib):
    def __init__(self, path=None):
        self.lib = C.CDLL(path or os.path.join(HERE, "liboracle.so"))
        b, L = self._bind, self.lib
        self.scene_new = b(L, "orc_scene_new", P, [P, P, U32, P, U32, P, U32, P, P])
        self.scene_free = b(L, "orc_scene_free", None, [P])
        self.set_positions = b(L, "orc_set_positions", C.c_int, [P, P, P])
        self.morton_keys = b(L, "orc_morton_keys", C.c_int, [P, C.c_int, P, P, P])
        self.sort_bitonic = b(L, "orc_sort_bitonic", C.c_int, [P, U32, P])
        self.build = b(L, "orc_build", C.c_int, [P, C.c_int, C.c_int, C.c_int])
        self.refit = b(L, "orc_refit", C.c_int, [P])
        self.get_sort = b(L, "orc_get_sort", C.c_int, [P, P, P, P, P])
        self.get_buffers = b(L, "orc_get_buffers", C.c_int, [P, P, P])
        self.export = b(L, "orc_export", C.c_int, [P, P, U32, C.POINTER(U32)])
        self.gen_primary = b(L, "orc_gen_primary", C.c_int,
                             [P, I32, I32, I32, I32, P, SZ, SZ, P])
        self.trace = b(L, "orc_trace", C.c_int, [P, P, I32, P, C.c_int])
        self.shadow = b(L, "orc_shadow", C.c_int, [P, P, I32, P, C.c_int])
        self.shade = b(L, "orc_shade", C.c_int, [P, P, P, I32, P, C.c_int])
        self.gen_secondary = b(L, "orc_gen_secondary", C.c_int,
                               [P, P, I32, P, P, I32, C.POINTER(I32)])
        self.fb_copy = b(L, "orc_fb_copy", C.c_int, [P, P, SZ])
        self.render = b(L, "orc_render", C.c_int,
                        [P, P, I32, I32, I32, SZ, SZ, SZ, P, P, C.c_int])
        self.fp64_closest = b(L, "orc_fp64_closest", C.c_int, [P, P, I32, P, P, C.c_int])
        self.fp64_t_of = b(L, "orc_fp64_t_of", C.c_int, [P, P, I32, P, P])
        self.emit_keys_raw = b(L, "orc_emit_keys", C.c_int, [P, U32, C.c_int, C.c_int, P, U32,
                                                              C.POINTER(U32)])
        self.mangle_raw = b(L, "orc_mangle", C.c_int, [P, P, U32, F, F, F])
        self.multi_new_raw = b(L, "orc_multi_new", P, [P, I32, P, P, P, I32, P])
        self.multi_free = b(L, "orc_multi_free", None, [P])
        self.multi_trace_raw = b(L, "orc_multi_trace", C.c_int, [P, P, I32, P, C.c_int])
        self.multi_shadow_raw = b(L, "orc_multi_shadow", C.c_int, [P, P, I32, P, C.c_int])
        self.multi_render_raw = b(L, "orc_multi_render", C.c_int,
                                  [P, P, I32, I32, I32, SZ, P, P, C.c_int])
        self.build_sah_raw = b(L, "orc_build_sah", C.c_int, [P])
        self.traversal_counts_raw = b(L, "orc_traversal_counts", C.c_int, [P, P, I32, C.c_int, P])
        self.vanishing_raw = b(L, "orc_vanishing_lights", C.c_int, [P, P, P, I32, P])
        self.sah_nodes_raw = b(L, "orc_sah_nodes", C.c_int, [P, P, P, P, P, P, P, C.POINTER(U32)])

    def multi(self, scene_handles, inst_scene, tr, trinv, lights):
        """Multi-root scene over built oracle scenes; tr / trinv: float32 [n, 4, 4]."""
        arr = (P * len(scene_handles))(*scene_handles)
        ins = np.ascontiguousarray(inst_scene, np.int32)
        t = np.ascontiguousarray(tr, np.float32)
        ti = np.ascontiguousarray(trinv, np.float32)
        h = self.multi_new_raw(C.cast(arr, P), len(scene_handles), _p(ins), _p(t), _p(ti),
                               ins.shape[0], C.byref(lights))
        if not h:
            raise RuntimeError("oracle multi-root scene rejected")
        return h

    def multi_trace(self, h, samples, threads=0):
        hits = np.zeros(samples.shape[0], abi.HIT_DTYPE)
        self.multi_trace_raw(h, _p(samples), samples.shape[0], _p(hits), threads or os.cpu_count())
        return hits

    def multi_shadow(self, h, samples, hits, threads=0):
        self.multi_shadow_raw(h, _p(samples), samples.shape[0], _p(hits), threads or os.cpu_count())

    def multi_render(self, h, cam, w, hh, max_bounces, tile=1 << 20, threads=0):
        image = np.zeros((hh * w, 3), np.uint32)
        st = abi.RenderStats()
        self.multi_render_raw(h, C.byref(cam), w, hh, max_bounces, tile, _p(image), C.byref(st),
                              threads or os.cpu_count())
        return image, st

    def mangle(self, pos4, nrm4, arg, last_arg=-1000.0, height=0.2):
        """mangle on copies of float32 [V, 4] positions / normals."""
        p, n = np.array(pos4, np.float32, copy=True), np.array(nrm4, np.float32, copy=True)
        self.mangle_raw(_p(p), _p(n), p.shape[0], arg, last_arg, height)
        return p, n

    def emit_keys(self, sorted_keys, depth=30, min_leaf=1):
        k = np.ascontiguousarray(sorted_keys, np.uint32)
        cnt = U32(0)
        if self.emit_keys_raw(_p(k), k.shape[0], depth, min_leaf, None, 0, C.byref(cnt)):
            raise RuntimeError("emit failed")
        out = np.zeros(cnt.value, abi.CANON_DTYPE)
        self.emit_keys_raw(_p(k), k.shape[0], depth, min_leaf, _p(out), cnt.value, C.byref(cnt))
        return out

    def new_scene(self, sc):
        h = self.scene_new(_p(sc.pos4), _p(sc.nrm4), sc.n_verts, _p(sc.idx), sc.n_tris,
                           _p(sc.mats), sc.mats.shape[0], _p(sc.mat_map), C.byref(sc.lights))
        return OracleScene(self, h, sc)


class OracleScene:
    def __init__(self, orc, h, sc):
        self.o, self.h, self.n = orc, h, sc.n_tris
        self.lights = sc.lights

    def __del__(self):
        try:
            self.o.scene_free(self.h)
        except Exception:
            pass

    def build(self, depth=30, min_leaf=1, sort_kind=0):
        r = self.o.build(self.h, depth, min_leaf, sort_kind)
        if r:
            raise RuntimeError("oracle build failed")

    def build_sah(self):
        """The reference's CPU SAH BVH over the current triangle order."""
        r = self.o.build_sah_raw(self.h)
        if r == -2:
            raise ValueError("SAH tree deeper than the traversal's 32-entry stack")
        if r:
            raise RuntimeError("oracle SAH build failed")

    def sah_nodes(self):
        """(lo, hi, a, b, leaf, order) of the SAH tree in the reference's numbering."""
        cnt = U32(0)
        self.o.sah_nodes_raw(self.h, None, None, None, None, None, None, C.byref(cnt))
        m = cnt.value
        lo, hi = np.zeros((m, 3), np.float32), np.zeros((m, 3), np.float32)
        a, b, leaf = (np.zeros(m, np.uint32) for _ in range(3))
        order = np.zeros(self.n, np.uint32)
        if self.o.sah_nodes_raw(self.h, _p(lo), _p(hi), _p(a), _p(b), _p(leaf), _p(order),
                                C.byref(cnt)):
            raise RuntimeError("no SAH tree")
        return lo, hi, a, b, leaf, order

    def traversal_counts(self, samples, threads=0):
        """{nodes, tris} entered / tested by the closest-hit rays of samples
        and by the shadow rays of their hits that the fused renders trace,
        the shadow ray count and the number traced."""
        out = np.zeros(6, np.uint64)
        if self.o.traversal_counts_raw(self.h, _p(samples), samples.shape[0],
                                       threads or os.cpu_count(), _p(out)):
            raise RuntimeError("oracle scene not built")
        return {"nodes": int(out[0]), "tris": int(out[1]), "shadow_nodes": int(out[2]),
                "shadow_tris": int(out[3]), "shadow_rays": int(out[4]),
                "shadow_traced": int(out[5])}

    def vanishing_lights(self, samples, hits):
        """Per hit, the bitmask of lights whose shadow ray the fused renders
        skip (both terms the light would add are zero)."""
        m = np.zeros(samples.shape[0], np.uint32)
        self.o.vanishing_raw(self.h, _p(samples), _p(hits), samples.shape[0], _p(m))
        return m

    def sort_arrays(self):
        n = self.n
        keys, perm, sk, orig = (np.zeros(n, np.uint32) for _ in range(4))
        self.o.get_sort(self.h, _p(keys), _p(perm), _p(sk), _p(orig))
        return keys, perm, sk, orig

    def buffers(self):
        idx = np.zeros((self.n, 3), np.uint32)
        mp = np.zeros(self.n, np.uint32)
        self.o.get_buffers(self.h, _p(idx), _p(mp))
        return idx, mp

    def canon(self):
        cnt = U32(0)
        self.o.export(self.h, None, 0, C.byref(cnt))
        out = np.zeros(cnt.value, abi.CANON_DTYPE)
        self.o.export(self.h, _p(out), cnt.value, C.byref(cnt))
        return out

    def trace(self, samples, threads=0):
        hits = np.zeros(samples.shape[0], abi.HIT_DTYPE)
        self.o.trace(self.h, _p(samples), samples.shape[0], _p(hits), threads or os.cpu_count())
        return hits

    def shadow(self, samples, hits, threads=0):
        self.o.shadow(self.h, _p(samples), samples.shape[0], _p(hits), threads or os.cpu_count())
        return hits

    def shade(self, samples, hits, image, threads=0):
        self.o.shade(self.h, _p(samples), _p(hits), samples.shape[0], _p(image),
                     threads or os.cpu_count())
        return image

    def gen_secondary(self, samples, hits, max_out=None):
        n = samples.shape[0]
        max_out = n if max_out is None else max_out
        out = np.zeros(max_out, abi.SAMPLE_DTYPE)
        cnt = I32(0)
        self.o.gen_secondary(self.h, _p(samples), n, _p(hits), _p(out), max_out, C.byref(cnt))
        return out[:cnt.value]

    def render(self, cam, w, h, max_bounces, offset=0, count=None, tile=1 << 18, threads=0,
               image=None):
        count = w * h if count is None else count
        if image is None:
            image = np.zeros((h * w, 3), np.uint32)
        st = abi.RenderStats()
        r = self.o.render(self.h, C.byref(cam), w, h, max_bounces, offset, count, tile,
                          _p(image), C.byref(st), threads or os.cpu_count())
        if r:
            raise RuntimeError("oracle render failed")
        return image, st

    def fp64_closest(self, samples, threads=0):
        n = samples.shape[0]
        ids = np.zeros(n, np.int32)
        ts = np.zeros(n, np.float64)
        self.o.fp64_closest(self.h, _p(samples), n, _p(ids), _p(ts), threads)
        return ids, ts

    def fp64_t_of(self, samples, tri_orig):
        n = samples.shape[0]
        ts = np.zeros(n, np.float64)
        tri = np.ascontiguousarray(tri_orig, np.int32)
        self.o.fp64_t_of(self.h, _p(samples), n, _p(tri), _p(ts))
        return ts


def gen_primary(orc, cam, w, h, count=None, offset=0, quad=32):
    count = w * h if count is None else count
    out = np.zeros(count, abi.SAMPLE_DTYPE)
    orc.gen_primary(C.byref(cam), w, h, quad, 1, None, count, offset, _p(out))
    return out


def fb_copy(orc, image):
    px = image.shape[0]
    rgba = np.zeros((px, 4), np.uint8)
    orc.fb_copy(_p(image), _p(rgba), px)
    return rgba


class RefKernels(_Lib):
    """The reference's kernels compiled for the CPU plus the restated host loops."""

    PATH = os.path.join(HERE, "_ref", "libref.so")

    @classmethod
    def available(cls):
        return os.path.exists(cls.PATH)

    def __init__(self):
        self.lib = C.CDLL(self.PATH)
        b, L = self._bind, self.lib
        self.scene_new = b(L, "refd_scene_new", P, [P, P, U32, P, U32, P, U32, P, P])
        self.scene_free = b(L, "refd_scene_free", None, [P])
        self.morton = b(L, "refd_morton", C.c_int, [P, C.c_int, P, P, P])
        self.bitonic = b(L, "refd_bitonic", C.c_int, [P, U32, P])
        self.apply_perm = b(L, "refd_apply_perm", C.c_int, [P, P])
        self.get_buffers = b(L, "refd_get_buffers", C.c_int, [P, P, P])
        self.set_tree = b(L, "refd_set_tree", C.c_int, [P, P, U32])
        self.build_lbvh_raw = b(L, "refd_build_lbvh", C.c_int,
                                [P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, P])
        self.canon_raw = b(L, "refd_canon", C.c_int, [P, P, U32, C.POINTER(U32)])
        self.get_tree = b(L, "refd_get_tree", C.c_int, [P, P])
        self.gen_primary = b(L, "refd_gen_primary", C.c_int,
                             [P, I32, I32, I32, I32, P, SZ, SZ, P])
        self.trace = b(L, "refd_trace", C.c_int, [P, P, I32, P, C.c_int])
        self.shadow = b(L, "refd_shadow", C.c_int, [P, P, I32, P, C.c_int])
        self.shade = b(L, "refd_shade", C.c_int, [P, P, P, I32, P, C.c_int, C.c_int])
        self.gen_secondary = b(L, "refd_gen_secondary", C.c_int,
                               [P, P, I32, P, P, I32, C.POINTER(I32)])
        self.render = b(L, "refd_render", C.c_int,
                        [P, P, I32, I32, I32, SZ, SZ, SZ, P, P, C.c_int])
        self.mangle_raw = b(L, "refk_mangle", None, [P, P, U32, F, F, F])
        self.multi_new_raw = b(L, "refd_multi_new", P, [P, I32, P, P, P, I32, P])
        self.multi_free = b(L, "refd_multi_free", None, [P])
        self.multi_trace_raw = b(L, "refd_multi_trace", C.c_int, [P, P, I32, P, C.c_int])
        self.multi_shadow_raw = b(L, "refd_multi_shadow", C.c_int, [P, P, I32, P, C.c_int])
        self.multi_render_raw = b(L, "refd_multi_render", C.c_int,
                                  [P, P, I32, I32, I32, SZ, P, P, C.c_int])
        self.obj_load_raw = b(L, "refo_load", P, [C.c_char_p])
        self.obj_sizes = b(L, "refo_sizes", None, [P, C.POINTER(U32), C.POINTER(U32),
                                                    C.POINTER(U32)])
        self.obj_copy = b(L, "refo_copy", None, [P, P, P, P, P, P, P, P])
        self.obj_free = b(L, "refo_free", None, [P])
        self.sah_build_raw = b(L, "refs_build", P, [P, U32, P, U32, C.POINTER(U32)])
        self.sah_copy = b(L, "refs_copy", None, [P, P, P, P, P, P, P])
        self.sah_free = b(L, "refs_free", None, [P])

    multi = Oracle.multi
    multi_trace = Oracle.multi_trace
    multi_shadow = Oracle.multi_shadow
    multi_render = Oracle.multi_render

    def build_lbvh(self, rh, n, depth=30, min_leaf=1, group_size=16, compute_units=2):
        """BVHBuilder::build_lbvh over the reference's own kernels (process_task
        and max_local_bbox as emulated work-groups of group_size work-items,
        up to compute_units groups at once).  Returns (keys, perm, glo, ghi);
        the tree stays in the scene handle, in the reference's numbering."""
        keys, perm = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        glo, ghi = np.zeros(3, np.float32), np.zeros(3, np.float32)
        if self.build_lbvh_raw(rh, depth, min_leaf, group_size, compute_units, _p(keys),
                               _p(perm), _p(glo), _p(ghi)):
            raise RuntimeError("reference build_lbvh failed")
        return keys, perm, glo, ghi

    def canon(self, rh):
        """The canonical range tree (pre-order, left first) of the scene's tree."""
        cnt = U32(0)
        if self.canon_raw(rh, None, 0, C.byref(cnt)):
            raise RuntimeError("malformed reference tree")
        out = np.zeros(cnt.value, abi.CANON_DTYPE)
        self.canon_raw(rh, _p(out), cnt.value, C.byref(cnt))
        return out

    def sah_build(self, pos4, idx):
        """BVH::construct of the reference over (pos4, idx): (lo, hi, a, b,
        leaf, order) in its numbering."""
        pos4 = np.ascontiguousarray(pos4, np.float32)
        idx = np.ascontiguousarray(idx, np.uint32)
        cnt = U32(0)
        h = self.sah_build_raw(_p(pos4), pos4.shape[0], _p(idx), idx.shape[0], C.byref(cnt))
        m = cnt.value
        lo, hi = np.zeros((m, 3), np.float32), np.zeros((m, 3), np.float32)
        a, b, leaf = (np.zeros(m, np.uint32) for _ in range(3))
        order = np.zeros(idx.shape[0], np.uint32)
        self.sah_copy(h, _p(lo), _p(hi), _p(a), _p(b), _p(leaf), _p(order))
        self.sah_free(h)
        return lo, hi, a, b, leaf, order

    def obj_load(self, path):
        """The reference's OBJ import: (pos4, nrm4, idx, group starts / ends
        in index-buffer units, diffuse [G, 3], shininess [G])."""
        h = self.obj_load_raw(str(path).encode())
        if not h:
            raise RuntimeError("reference OBJ import failed: %s" % path)
        try:
            V, N, G = U32(), U32(), U32()
            self.obj_sizes(h, C.byref(V), C.byref(N), C.byref(G))
            pos = np.zeros((V.value, 4), np.float32)
            nrm = np.zeros((V.value, 4), np.float32)
            idx = np.zeros((N.value, 3), np.uint32)
            gs = np.zeros(G.value, np.uint32)
            ge = np.zeros(G.value, np.uint32)
            gd = np.zeros((G.value, 3), np.float32)
            gsh = np.zeros(G.value, np.float32)
            self.obj_copy(h, _p(pos), _p(nrm), _p(idx), _p(gs), _p(ge), _p(gd), _p(gsh))
        finally:
            self.obj_free(h)
        return pos, nrm, idx, gs, ge, gd, gsh

    def mangle(self, pos4, nrm4, arg, last_arg=-1000.0, height=0.2):
        p, n = np.array(pos4, np.float32, copy=True), np.array(nrm4, np.float32, copy=True)
        self.mangle_raw(_p(p), _p(n), p.shape[0], arg, last_arg, height)
        return p, n

    def new_scene(self, sc):
        h = self.scene_new(_p(sc.pos4), _p(sc.nrm4), sc.n_verts, _p(sc.idx), sc.n_tris,
                           _p(sc.mats), sc.mats.shape[0], _p(sc.mat_map), C.byref(sc.lights))
        if not h:
            raise RuntimeError("reference scene rejected")
        return h
