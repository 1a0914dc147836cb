"""The oracle against golden vectors produced by the reference's own kernels
compiled for the CPU (tests/golden/make_golden.py).  Bit-exact."""
import ctypes as C
import os

import numpy as np
import pytest

import pyoracle
from golden.make_golden import cases

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {c[0]: c for c in cases()}


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(orc, name):
    _, sc, cam, w, h, bounces = CASES[name]
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    s = orc.new_scene(sc)
    s.build(30, 1, 1)                      # the reference's bitonic order
    keys, perm, _, _ = s.sort_arrays()
    assert np.array_equal(keys, g["keys"]), "Morton keys"
    assert np.array_equal(perm, g["perm"]), "bitonic permutation"
    c = s.canon()
    rng = np.stack([c["start"], c["end"], c["leaf"], c["depth"]], 1)
    assert np.array_equal(rng, g["ranges"])
    assert np.array_equal(c["lo"][:, :3], g["lo"]) and np.array_equal(c["hi"][:, :3], g["hi"])
    smp = pyoracle.gen_primary(orc, cam, w, h)
    assert np.array_equal(smp["dir"][:, :3], g["dirs"])
    hits = s.trace(smp)
    s.shadow(smp, hits)
    m = hits["hit"] == 1
    assert np.array_equal(hits["hit"], g["hit"])
    assert np.array_equal(hits["id"][m], g["hit_id"])
    assert np.array_equal(hits["t"][m], g["hit_t"])
    assert np.array_equal(hits["n"][m][:, :3], g["hit_n"])
    assert np.array_equal(hits["shadow_hit"][m], g["shadow"])
    img, st = s.render(cam, w, h, bounces)
    assert np.array_equal(img, g["image"])
    assert st.secondary_rays == int(g["secondary"][0])
