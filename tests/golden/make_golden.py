"""Generate golden vectors from the reference's own kernels compiled for the
CPU (oracle/_ref/libref.so, built by oracle/build.py from the reference
checkout).  The vectors pin the oracle where the reference is not available.

Run from the repository root:  python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tesina-rt_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build as ob            # noqa: E402
import pyoracle               # noqa: E402
from rtgb import abi, scenes  # noqa: E402

_p = pyoracle._p


def cases():
    """(name, scene, camera, width, height, bounces) — small, varied inputs."""
    out = []
    sc = scenes.soup(2000, seed=101)
    out.append(("soup2k_point", sc, scenes.camera((0, 0, -4), (0, 0, 0)), 64, 64, 3))
    sc = scenes.soup(1500, seed=102)
    sc.lights = abi.make_lights((0.1,) * 3, [dict(type=abi.RT_SPOT_L, pos=(0.0, 4.0, -2.0),
                                                  dir=(0.0, -0.894427, 0.447214), angle=0.7)])
    out.append(("soup1500_spot", sc, scenes.camera((0, 0, -4), (0, 0, 0)), 48, 40, 2))
    sc = scenes.soup(1000, seed=103)
    sc.lights = abi.make_lights((0.2,) * 3, [dict(type=abi.RT_DIR_L, dir=(0.3, -0.9, 0.3))])
    out.append(("soup1k_dir", sc, scenes.camera((0, 0.5, -4), (0, 0, 0)), 40, 48, 1))
    ter = scenes.Terrain(32, 16, n_spheres=3, seed=104,
                         lights=[dict(type=abi.RT_POINT_L, pos=(0.0, 6.0, -3.0))])
    out.append(("terrain1k_point", ter.scene(2), scenes.camera((0, 4, -10), (0, 0, 0)), 64, 36, 4))
    return out


def golden_for(R, name, sc, cam, w, h, bounces):
    n = sc.n_tris
    rh = R.new_scene(sc)
    # BVHBuilder::build_lbvh over the reference's own kernels: Morton keys,
    # bitonic permutation, the process_task tree (emulated work-groups) and
    # its refit boxes, all from the reference
    keys, perm, _, _ = R.build_lbvh(rh, n, 30, 1)
    tree = R.canon(rh)
    smp = np.zeros(w * h, abi.SAMPLE_DTYPE)
    R.gen_primary(C.byref(cam), w, h, 32, 1, None, w * h, 0, _p(smp))
    hits = np.zeros(w * h, abi.HIT_DTYPE)
    R.trace(rh, _p(smp), w * h, _p(hits), 1)
    R.shadow(rh, _p(smp), w * h, _p(hits), 1)
    img = np.zeros((w * h, 3), np.uint32)
    st = abi.RenderStats()
    R.render(rh, C.byref(cam), w, h, bounces, 0, w * h, 1 << 18, _p(img), C.byref(st), 1)
    R.scene_free(rh)
    m = hits["hit"] == 1
    return dict(keys=keys, perm=perm, ranges=np.stack([tree["start"], tree["end"], tree["leaf"],
                                                       tree["depth"]], 1),
                lo=tree["lo"][:, :3], hi=tree["hi"][:, :3], dirs=smp["dir"][:, :3],
                hit=hits["hit"], hit_id=hits["id"][m], hit_t=hits["t"][m],
                hit_n=hits["n"][m][:, :3], shadow=hits["shadow_hit"][m], image=img,
                secondary=np.array([st.secondary_rays], np.uint64))


def main():
    ob.build_oracle()
    if not ob.build_ref():
        raise SystemExit("the reference checkout is needed to generate golden vectors")
    R = pyoracle.RefKernels()
    for name, sc, cam, w, h, b in cases():
        g = golden_for(R, name, sc, cam, w, h, b)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **g)
        print(name, {k: v.shape for k, v in g.items()})


if __name__ == "__main__":
    main()
