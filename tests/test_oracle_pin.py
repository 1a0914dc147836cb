"""Live pin of the oracle against the reference's kernels compiled for the
CPU (oracle/_ref, built where the reference checkout exists)."""
import ctypes as C

import numpy as np
import pytest

import pyoracle
from helpers import camera_small, single_light, tiny_terrain
from rtgb import abi, scenes

pytestmark = pytest.mark.skipif(not pyoracle.RefKernels.available(),
                                reason="reference kernels not built (no reference checkout)")
_p = pyoracle._p


@pytest.fixture(scope="module")
def ref():
    return pyoracle.RefKernels()


def _pair(orc, ref, sc):
    s = orc.new_scene(sc)
    s.build(30, 1, 1)
    rh = ref.new_scene(sc)
    return s, rh


@pytest.mark.parametrize("light", ["point", "spot", "dir"])
def test_pin_soup_10k(orc, ref, light):
    sc = scenes.soup(10000, seed=1)
    sc.lights = single_light(light)
    s, rh = _pair(orc, ref, sc)
    n = sc.n_tris
    kr = np.zeros(n, np.uint32)
    assert ref.morton(rh, 30, _p(kr), None, None) == 0
    keys, perm, _, _ = s.sort_arrays()
    assert np.array_equal(kr, keys)
    pr = np.zeros(n, np.uint32)
    assert ref.bitonic(_p(kr), n, _p(pr)) == 0
    assert np.array_equal(pr, perm)
    ref.apply_perm(rh, _p(pr))
    ir, mr = np.zeros((n, 3), np.uint32), np.zeros(n, np.uint32)
    ref.get_buffers(rh, _p(ir), _p(mr))
    io, mo = s.buffers()
    assert np.array_equal(ir, io) and np.array_equal(mr, mo)
    canon = s.canon()
    assert ref.set_tree(rh, _p(canon), canon.shape[0]) == 0
    tr = canon.copy()
    ref.get_tree(rh, _p(tr))
    assert np.array_equal(tr["lo"], canon["lo"]) and np.array_equal(tr["hi"], canon["hi"])
    cam = camera_small()
    w = h = 256
    so = pyoracle.gen_primary(orc, cam, w, h)
    sr = np.zeros(w * h, abi.SAMPLE_DTYPE)
    ref.gen_primary(C.byref(cam), w, h, 32, 1, None, w * h, 0, _p(sr))
    assert so.tobytes() == sr.tobytes()
    ho = s.trace(so)
    s.shadow(so, ho)
    hr = np.zeros(w * h, abi.HIT_DTYPE)
    ref.trace(rh, _p(sr), w * h, _p(hr), 4)
    ref.shadow(rh, _p(sr), w * h, _p(hr), 4)
    m = ho["hit"] == 1
    assert np.array_equal(ho["hit"], hr["hit"])
    for f in ("id", "t", "inverse_n", "shadow_hit"):
        assert np.array_equal(ho[f][m], hr[f][m]), f
    for f in ("n", "hit_point"):
        assert np.array_equal(ho[f][m], hr[f][m]), f
    io_, ir_ = np.zeros((w * h, 3), np.uint32), np.zeros((w * h, 3), np.uint32)
    s.shade(so, ho, io_)
    ref.shade(rh, _p(sr), _p(hr), w * h, _p(ir_), 1, 4)
    assert np.array_equal(io_, ir_)
    s2 = s.gen_secondary(so, ho)
    out = np.zeros(w * h, abi.SAMPLE_DTYPE)
    cnt = C.c_int32(0)
    ref.gen_secondary(rh, _p(sr), w * h, _p(hr), _p(out), w * h, C.byref(cnt))
    assert cnt.value == s2.shape[0] and s2.tobytes() == out[:cnt.value].tobytes()
    ref.scene_free(rh)


def test_pin_full_render_small_workload(orc, ref):
    """The 512x512, depth-3 soup rendered end to end by the reference's own
    kernels (one point light, expressed as a cone-less spot light) and by the
    oracle: identical fixed-point images."""
    wl = scenes.workload_small()
    sc = wl["scene"]
    s, rh = _pair(orc, ref, sc)
    keys, perm, _, _ = s.sort_arrays()
    ref.apply_perm(rh, _p(perm))
    canon = s.canon()
    ref.set_tree(rh, _p(canon), canon.shape[0])
    img_o, st_o = s.render(wl["camera"], 512, 512, 3)
    img_r = np.zeros((512 * 512, 3), np.uint32)
    st_r = abi.RenderStats()
    ref.render(rh, C.byref(wl["camera"]), 512, 512, 3, 0, 512 * 512, 1 << 18, _p(img_r),
               C.byref(st_r), 8)
    assert np.array_equal(img_o, img_r)
    assert st_o.secondary_rays == st_r.secondary_rays
    ref.scene_free(rh)


def _ref_vs_oracle_tree(orc, ref, sc, depth, min_leaf, group_size=16, compute_units=2):
    """BVHBuilder::build_lbvh run over the reference's own kernels (the emit
    and the global AABB reduction as emulated work-groups) against the
    oracle's build: keys, permutation, sorted buffers and the canonical tree
    (ranges, leaf flags, depths, AABBs) byte for byte."""
    rh = ref.new_scene(sc)
    keys, perm, glo, ghi = ref.build_lbvh(rh, sc.n_tris, depth, min_leaf, group_size,
                                          compute_units)
    s = orc.new_scene(sc)
    s.build(depth, min_leaf, 1)
    ok, op, _, _ = s.sort_arrays()
    assert np.array_equal(keys, ok), "Morton keys"
    assert np.array_equal(perm, op), "bitonic permutation"
    ir, mr = np.zeros((sc.n_tris, 3), np.uint32), np.zeros(sc.n_tris, np.uint32)
    ref.get_buffers(rh, _p(ir), _p(mr))
    io, mo = s.buffers()
    assert np.array_equal(ir, io) and np.array_equal(mr, mo)
    # the max_local_bbox reduction equals the order-free min / max
    tri = sc.pos4[sc.idx.astype(np.int64)][:, :, :3]
    assert np.array_equal(glo, tri.min(axis=(0, 1))) and np.array_equal(ghi, tri.max(axis=(0, 1)))
    rc, oc = ref.canon(rh), s.canon()
    assert rc.shape == oc.shape, "node count %d vs %d" % (rc.shape[0], oc.shape[0])
    assert rc.tobytes() == oc.tobytes()
    return rh, s, rc


def test_pin_emit_soup_10k(orc, ref):
    """The 10k soup: the reference's process_task tree is the oracle's."""
    rh, _, rc = _ref_vs_oracle_tree(orc, ref, scenes.soup(10000, seed=1), 30, 1)
    assert int(rc["leaf"].sum()) > 2000
    ref.scene_free(rh)


@pytest.mark.parametrize("min_leaf", [1, 4, 256])
@pytest.mark.parametrize("depth", [1, 10, 16, 30, 32])
def test_pin_emit_terrain_duplicates(orc, ref, depth, min_leaf):
    """The duplicate-heavy terrain (shared grid vertices, flat cells, so many
    equal keys) over the depth and minimum-leaf range: large leaves of equal
    keys, the bit-exhausted leaf rule and the last launched level."""
    rh, _, _ = _ref_vs_oracle_tree(orc, ref, tiny_terrain().scene(1), depth, min_leaf)
    ref.scene_free(rh)


@pytest.mark.parametrize("n", [17, 2047, 4097])
def test_pin_emit_sizes(orc, ref, n):
    rh, _, _ = _ref_vs_oracle_tree(orc, ref, scenes.soup(n, seed=n), 30, 1)
    ref.scene_free(rh)


@pytest.mark.parametrize("group_size,compute_units", [(2, 1), (8, 4), (64, 3)])
def test_pin_emit_launch_shapes(orc, ref, group_size, compute_units):
    """Work-group size and group count change the reference's node numbering,
    not its range tree."""
    rh, _, _ = _ref_vs_oracle_tree(orc, ref, tiny_terrain(48, 24, 2, seed=9).scene(3), 30, 1,
                                   group_size, compute_units)
    ref.scene_free(rh)


def test_pin_render_over_reference_tree(orc, ref):
    """The 512x512, depth-3 soup rendered by the reference's kernels over the
    tree its own builder emitted (reference node numbering, boxes from its
    refit kernels) equals the oracle's render."""
    wl = scenes.workload_small()
    rh, s, _ = _ref_vs_oracle_tree(orc, ref, wl["scene"], 30, 1)
    img_o, st_o = s.render(wl["camera"], 512, 512, 3)
    img_r = np.zeros((512 * 512, 3), np.uint32)
    st_r = abi.RenderStats()
    ref.render(rh, C.byref(wl["camera"]), 512, 512, 3, 0, 512 * 512, 1 << 18, _p(img_r),
               C.byref(st_r), 8)
    assert np.array_equal(img_o, img_r)
    assert st_o.secondary_rays == st_r.secondary_rays > 0
    ref.scene_free(rh)


@pytest.mark.parametrize("depth", [30, 10, 1])
def test_pin_terrain_duplicates(orc, ref, depth):
    """Equal keys: the oracle's bitonic restatement reproduces the reference's
    (unstable) tie order exactly."""
    sc = tiny_terrain().scene(1)
    s = orc.new_scene(sc)
    s.build(depth, 1, 1)
    rh = ref.new_scene(sc)
    kr = np.zeros(sc.n_tris, np.uint32)
    ref.morton(rh, depth, _p(kr), None, None)
    pr = np.zeros(sc.n_tris, np.uint32)
    assert ref.bitonic(_p(kr), sc.n_tris, _p(pr)) == 0
    keys, perm, _, _ = s.sort_arrays()
    assert np.array_equal(kr, keys) and np.array_equal(pr, perm)
    ref.scene_free(rh)


@pytest.mark.parametrize("n", [1, 2, 4, 8, 16, 17, 31, 33, 1000])
def test_pin_bitonic_sizes(orc, ref, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 64, size=n).astype(np.uint32)    # many duplicates
    pr, po = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    rr = ref.bitonic(_p(keys), n, _p(pr))
    ro = orc.sort_bitonic(_p(keys), n, _p(po))
    assert rr == ro == 0
    assert np.array_equal(pr, po)
    assert (np.diff(keys[pr].astype(np.int64)) >= 0).all()


@pytest.mark.parametrize("n", [3, 5, 6, 7, 9, 12, 15])
def test_pin_bitonic_aborts_like_reference(orc, ref, n):
    """Non-power-of-two N < 16 make the reference launch zero work-items and
    exit(1) (bvh-builder.cpp:403-406); both report it as -1."""
    keys = np.arange(n, dtype=np.uint32)[::-1].copy()
    p = np.zeros(n, np.uint32)
    assert ref.bitonic(_p(keys), n, _p(p)) == -1
    assert orc.sort_bitonic(_p(keys), n, _p(p)) == -1


@pytest.mark.parametrize("arg", [1.0, 17.0, 250.0])
def test_pin_mangle(orc, ref, arg):
    """mangle (mangler.cl:12-32): the oracle's restatement equals the
    reference kernel compiled for the CPU, bit for bit, on a terrain's
    vertices (positions, and the normals' x and z it rewrites)."""
    ter = tiny_terrain(64, 32, 4)
    sc = ter.scene(0)
    po, no = orc.mangle(sc.pos4, sc.nrm4, arg, arg - 1.0, 0.2)
    pr, nr = ref.mangle(sc.pos4, sc.nrm4, arg, arg - 1.0, 0.2)
    assert np.array_equal(po.view(np.uint32), pr.view(np.uint32))
    assert np.array_equal(no.view(np.uint32), nr.view(np.uint32))
    assert not np.array_equal(po, sc.pos4)


OBJ_MODELS = ["floor", "teapot-low_res", "teapot2", "teapot", "grid100", "frame_boat1",
              "frame_water1"]


@pytest.mark.parametrize("name", OBJ_MODELS)
def test_pin_obj_models(ref, name):
    """The library's OBJ reader against the reference's own import compiled
    for the CPU, on every model the reference ships: vertices, normals
    (read or generated), triangles and material groups, bit for bit."""
    import os
    import build as ob
    from rtgb import obj
    path = os.path.join(ob.REFERENCE_ROOT, "models", "obj", name + ".obj")
    if not os.path.exists(path):
        pytest.skip("model not present")
    rp, rn, ri, gs, ge, gd, gsh = ref.obj_load(path)
    op, on, oi, groups = obj.read(path)
    assert np.array_equal(op.view(np.uint32), rp.view(np.uint32))
    assert np.array_equal(on.view(np.uint32), rn.view(np.uint32))
    assert np.array_equal(oi, ri)
    assert np.array_equal(groups["first_triangle"] * 3, gs)
    # the reference's end_index is its start (in index-buffer units) plus a
    # triangle count (obj-loader.cpp:1380-1381)
    assert np.array_equal(groups["first_triangle"] * 3 + groups["triangle_count"], ge)
    assert np.array_equal(groups["diffuse"], gd)
    assert np.array_equal(groups["shininess"], gsh)


@pytest.mark.parametrize("frac", [0.3, 1.0])
def test_pin_refraction_render(orc, ref, frac):
    """Refraction (secondary-ray-generator.cl:220-256): a soup with glass
    triangles (refractive index 1.333) rendered end to end by the
    reference's kernels and by the oracle, depth 4; the secondary rays of the
    first bounce compared ray by ray, and the images, bit for bit."""
    sc = scenes.with_glass(scenes.soup(6000, seed=9), frac=frac, seed=2)
    s, rh = _pair(orc, ref, sc)
    keys, perm, _, _ = s.sort_arrays()
    ref.apply_perm(rh, _p(perm))
    canon = s.canon()
    ref.set_tree(rh, _p(canon), canon.shape[0])
    cam = scenes.camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), aspect=1.0)
    w = h = 200
    img_o, st_o = s.render(cam, w, h, 4)
    img_r = np.zeros((w * h, 3), np.uint32)
    st_r = abi.RenderStats()
    ref.render(rh, C.byref(cam), w, h, 4, 0, w * h, 1 << 18, _p(img_r), C.byref(st_r), 8)
    assert st_o.secondary_rays == st_r.secondary_rays > 2000
    assert np.array_equal(img_o, img_r)
    ref.scene_free(rh)


def _instances():
    """Two meshes, four instances: identity, a translation, a rotation with
    uniform scale, a non-uniform scale (row-major 4x4, inverse in float64)."""
    def tr(rot_deg=0.0, scale=(1, 1, 1), t=(0, 0, 0)):
        a = np.radians(rot_deg)
        r = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
        m = np.eye(4)
        m[:3, :3] = r @ np.diag(scale)
        m[:3, 3] = t
        return m
    ms = [tr(), tr(t=(2.0, 0.0, 0.0)), tr(30.0, (0.7, 0.7, 0.7), (-1.5, 0.3, 1.0)),
          tr(0.0, (1.0, 0.5, 1.2), (0.0, -1.0, 2.0))]
    T = np.array(ms, np.float32)
    Ti = np.array([np.linalg.inv(m) for m in ms], np.float32)
    return [0, 1, 1, 0], T, Ti


@pytest.mark.parametrize("glass", [False, True])
def test_pin_multi_root(orc, ref, glass):
    """trace_multi / shadow_trace_multi (trace-bvh.cl:420-463,
    shadow-trace-bvh.cl:317-373) and the render over several roots: the
    oracle against the reference's kernels on the same trees, bit for bit;
    with glass, the refracted rays of the moved, unnormalised normals too."""
    meshes = [scenes.soup(3000, seed=4), tiny_terrain(32, 16, 2).scene(0)]
    if glass:
        meshes = [scenes.with_glass(meshes[0], frac=0.5, seed=2),
                  scenes.with_glass(meshes[1], frac=0.5, seed=3)]
    o_h, r_h = [], []
    for sc in meshes:
        s, rh = _pair(orc, ref, sc)
        keys, perm, _, _ = s.sort_arrays()
        ref.apply_perm(rh, _p(perm))
        canon = s.canon()
        ref.set_tree(rh, _p(canon), canon.shape[0])
        o_h.append(s)
        r_h.append(rh)
    inst, T, Ti = _instances()
    lights = abi.make_lights((0.1, 0.1, 0.1), [dict(type=abi.RT_POINT_L, pos=(0.0, 4.0, -3.0),
                                                   color=(1.0, 1.0, 1.0))])
    om = orc.multi([s.h for s in o_h], inst, T, Ti, lights)
    rm = ref.multi(r_h, inst, T, Ti, lights)
    cam = scenes.camera((0.0, 1.5, -6.0), (0.0, 0.0, 0.5), aspect=1.0)
    w = h = 160
    import pyoracle as po
    smp = po.gen_primary(orc, cam, w, h)
    ho = orc.multi_trace(om, smp)
    hr = ref.multi_trace(rm, smp)
    m = ho["hit"] == 1
    assert np.array_equal(ho["hit"], hr["hit"]) and m.sum() > 2000
    for f in ("id", "t", "inverse_n"):
        assert np.array_equal(ho[f][m], hr[f][m]), f
    for f in ("n", "hit_point"):
        assert np.array_equal(ho[f][m][:, :3].view(np.uint32), hr[f][m][:, :3].view(np.uint32)), f
    orc.multi_shadow(om, smp, ho)
    ref.multi_shadow(rm, smp, hr)
    assert np.array_equal(ho["shadow_hit"][m], hr["shadow_hit"][m])
    img_o, st_o = orc.multi_render(om, cam, w, h, 3, tile=1 << 20)
    img_r, st_r = ref.multi_render(rm, cam, w, h, 3, tile=1 << 20)
    assert np.array_equal(img_o, img_r) and st_o.secondary_rays == st_r.secondary_rays > 0
    orc.multi_free(om)
    ref.multi_free(rm)
    for rh in r_h:
        ref.scene_free(rh)


def _canon_of_numbered(lo, hi, a, b, leaf):
    """A tree in the reference's numbering (root 0; children or leaf range in
    a, b) as canonical pre-order nodes, interior ranges from their subtrees."""
    out = []

    def walk(k, depth):
        me = len(out)
        out.append(None)
        if leaf[k]:
            s, e = int(a[k]), int(b[k])
        else:
            s, _ = walk(int(a[k]), depth + 1)
            _, e = walk(int(b[k]), depth + 1)
        out[me] = (s, e, int(leaf[k]), depth, lo[k], hi[k])
        return s, e

    walk(0, 0)
    c = np.zeros(len(out), abi.CANON_DTYPE)
    for i, (s, e, lf, d, l, h) in enumerate(out):
        c[i]["start"], c[i]["end"], c[i]["leaf"], c[i]["depth"] = s, e, lf, d
        c[i]["lo"][:3], c[i]["hi"][:3] = l, h
    return c


def _negative_soup():
    sc = scenes.soup(2500, seed=8)
    pos = sc.pos4.copy()
    pos[:, :3] -= np.float32(5.0)       # every coordinate negative
    return scenes.Scene(pos, sc.nrm4, sc.idx, sc.mats, sc.mat_map, sc.lights)


@pytest.mark.parametrize("kind", ["soup", "terrain", "negative"])
def test_pin_sah(orc, ref, kind):
    """BVH::construct (bvh.cpp:92-141) against the oracle's restatement: the
    same nodes in the same numbering, the same triangle order; and the
    reference's trace / shadow / shade kernels over the reference's SAH tree
    against the oracle's render over its own, pixel for pixel.  The negative
    scene makes the empty-bucket boxes' FLT_MIN maximum count."""
    sc = {"soup": lambda: scenes.soup(4000, seed=2),
          "terrain": lambda: tiny_terrain(48, 24, 3).scene(0),
          "negative": _negative_soup}[kind]()
    sc.lights = single_light("point")          # the reference's kernels hold one light
    rlo, rhi, ra, rb, rleaf, rorder = ref.sah_build(sc.pos4, sc.idx)
    s = orc.new_scene(sc)
    s.build_sah()
    olo, ohi, oa, ob, oleaf, oorder = s.sah_nodes()
    assert np.array_equal(rorder, oorder)
    assert np.array_equal(rleaf, oleaf)
    assert np.array_equal(ra, oa) and np.array_equal(rb, ob)
    assert rlo.tobytes() == olo.tobytes() and rhi.tobytes() == ohi.tobytes()
    assert int(rleaf.sum()) > sc.n_tris // 3
    canon = _canon_of_numbered(rlo, rhi, ra, rb, rleaf)
    assert s.canon().tobytes() == canon.tobytes()
    rh = ref.new_scene(sc)
    ref.apply_perm(rh, _p(rorder))
    assert ref.set_tree(rh, _p(canon), canon.shape[0]) == 0
    cam = camera_small() if kind != "negative" else scenes.camera((-5.0, -4.0, -9.0),
                                                                  (-5.0, -5.0, -5.0))
    w = h = 160
    img_r = np.zeros((w * h, 3), np.uint32)
    st_r = abi.RenderStats()
    assert ref.render(rh, C.byref(cam), w, h, 3, 0, w * h, 1 << 20, _p(img_r), C.byref(st_r),
                      4) == 0
    img_o, st_o = s.render(cam, w, h, 3, tile=1 << 20)
    assert st_o.hits > 1000
    assert np.array_equal(img_o, img_r)
    assert st_o.secondary_rays == st_r.secondary_rays   # ref_driver.cpp counts no hits
    ref.scene_free(rh)
