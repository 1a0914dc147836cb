"""OBJ input (rt_obj_load): the loader's rules on small files written here."""
import numpy as np
import pytest

from rtgb import capi, obj, scenes


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_quads_fan_negative_indices_and_sharing(tmp_path):
    p = _write(tmp_path, "q.obj", """
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vt 1 0
f 1/1 2/2 3/1 4/1
f -1/-1 -2/-1 -3/-1
""")
    pos, nrm, idx, groups = obj.read(p)
    # the quad as a fan (0, 1, 2), (0, 2, 3) over corners (v0,vt0) (v1,vt1)
    # (v2,vt0) (v3,vt0); negative indices resolve to k + count - 1: -1 -> v2,
    # -2 -> v1, -3 -> v0, texture -1 -> vt0.  (v2,vt0) and (v0,vt0) share
    # vertices 2 and 0; (v1,vt0) differs from (v1,vt1) and becomes vertex 4.
    assert idx.tolist() == [[0, 1, 2], [0, 2, 3], [2, 4, 0]]
    assert pos[:, :3].tolist() == [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [1, 0, 0]]
    assert groups.shape[0] == 1 and groups["triangle_count"][0] == 3
    # -4 resolves to -1: rejected (the loader would read before its array)
    bad = _write(tmp_path, "q2.obj", "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf -4 -3 -2\n")
    with pytest.raises(capi.RtError):
        obj.read(bad)


def test_materials_groups_and_generated_normals(tmp_path):
    _write(tmp_path, "m.mtl", """
newmtl red
Kd 0.9 0.1 0.1
Ns 500
newmtl glass
Kd 0.2 0.2 0.2
d 0.5
""")
    p = _write(tmp_path, "m.obj", """
usemtl red
mtllib m.mtl
v 0 0 0
v 1 0 0
v 0 1 0
v 0 0 1
f 1 2 3
f 1 3 4
usemtl glass
f 1 4 2
usemtl nosuch
f 2 4 3
""")
    pos, nrm, idx, g = obj.read(p)
    # groups: runs of one material, highest alpha first (glass has 0.5)
    assert g["first_triangle"].tolist() == [0, 3, 2]
    assert g["triangle_count"].tolist() == [2, 1, 1]
    assert np.allclose(g["diffuse"][0], [0.9, 0.1, 0.1]) and g["shininess"][0] == np.float32(0.5)
    assert g["alpha"][2] == np.float32(0.5)
    # no vn: normals from the faces (sum of unnormalised cross products)
    acc = np.zeros((pos.shape[0], 3), np.float32)
    for a, b, c in idx:
        e1 = pos[b, :3] - pos[a, :3]
        e2 = pos[c, :3] - pos[a, :3]
        n = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                      e1[0] * e2[1] - e1[1] * e2[0]], np.float32)
        acc[[a, b, c]] += n
    inv = (np.float32(1) / np.sqrt((acc * acc).sum(1))).astype(np.float32)
    assert np.array_equal(nrm[:, :3], (acc * inv[:, None]).astype(np.float32))


def test_write_read_round_trip(tmp_path):
    sc = scenes.soup(300, seed=4)
    p = tmp_path / "soup.obj"
    obj.write(p, sc.pos4, sc.nrm4, sc.idx)
    pos, nrm, idx, g = obj.read(p)
    # corners that share a position index and record collapse; a soup has
    # distinct vertices per triangle, so the mesh comes back as written
    assert np.array_equal(pos, sc.pos4) and np.array_equal(nrm[:, :3], sc.nrm4[:, :3])
    assert np.array_equal(idx, sc.idx) and g.shape[0] == 1


@pytest.mark.parametrize("text,what", [("v 0 0 0\n", "no faces"),
                                       ("v 0 0 0\nv 1 0 0\nf 1 2 3\n", "out of range")])
def test_bad_files_rejected(tmp_path, text, what):
    p = _write(tmp_path, "bad.obj", text)
    with pytest.raises(capi.RtError) as e:
        obj.read(p)
    assert e.value.code == -2
    with pytest.raises(capi.RtError):
        obj.read(tmp_path / "missing.obj")
