"""rt_sort_pairs_noalloc: the radix sort for callers that cannot allocate.

A caller whose device memory is already committed to its own pool, or whose
frame loop must not hit cudaMalloc's implicit synchronisation, sorts through
this entry point; its scratch is a fixed array inside the library.  The test
checks it, through the C ABI, against the sort that rt_bvh_build_lbvh runs
on the same Morton keys (bit-exact: integer keys and a stable permutation),
on two calls in a row with different inputs, so that contents the first call
leaves in the shared array cannot leak into the second.  This file sorts
last so that a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from rtgb import capi, scenes

pytestmark = pytest.mark.gpu


def _noalloc_sort(ctx, keys, vals, key_bits=30):
    lib = ctx.lib
    n = keys.shape[0]
    kin, vin = ctx.to_device(keys), ctx.to_device(vals)
    kout, vout = ctx.alloc(4 * n), ctx.alloc(4 * n)
    capi.check(lib, lib.rt_sort_pairs_noalloc(ctx.h, kin.ptr, vin.ptr, kout.ptr, vout.ptr, n,
                                              key_bits, None))
    ctx.sync()
    return kout.read(np.uint32), vout.read(np.uint32)


def _reference_sort(ctx, sc):
    """Keys and stable permutation from the existing LBVH entry point."""
    g = capi.Scene(ctx, sc)
    g.build(30, 1)
    keys, perm, sorted_keys, _ = g.sort_arrays()
    g.close()
    return keys, perm, sorted_keys


def test_noalloc_sort_matches_lbvh_sort_twice(ctx):
    inputs = [scenes.soup(200000, seed=21),
              scenes.Terrain(256, 128, n_spheres=20, seed=9).scene(0)]   # many equal keys
    for sc in inputs:
        keys, perm, sorted_keys = _reference_sort(ctx, sc)
        iota = np.arange(keys.shape[0], dtype=np.uint32)
        k, v = _noalloc_sort(ctx, keys, iota)
        assert np.array_equal(k, sorted_keys)
        assert np.array_equal(v, perm)
    assert ctx.device_status() == 0


def test_noalloc_sort_limits(ctx):
    lib = ctx.lib
    big = (1 << 20) + 1
    p = C.c_void_p(1)
    r = lib.rt_sort_pairs_noalloc(ctx.h, p, p, C.c_void_p(2), C.c_void_p(2), big, 30, None)
    assert r == -2
    assert b"RT_NOALLOC_MAX_PAIRS" in lib.rt_last_error()
    # the largest accepted size still sorts correctly (full 32-bit keys)
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 2 ** 32, size=1 << 20, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(1 << 20, dtype=np.uint32)
    k, v = _noalloc_sort(ctx, keys, vals, key_bits=32)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])
