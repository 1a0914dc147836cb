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


@pytest.mark.parametrize("key_bits", [8, 24])
def test_noalloc_sort_odd_pass_counts(ctx, key_bits):
    """One and three 8-bit passes: the first pass writes the outputs and the
    passes route through the scratch temporaries in the other order.  Stable
    order of keys & mask, as numpy's stable argsort."""
    rng = np.random.default_rng(key_bits)
    n = 300_001
    keys = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    k, v = _noalloc_sort(ctx, keys, vals, key_bits=key_bits)
    order = np.argsort(keys & np.uint32((1 << key_bits) - 1), kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])
    assert ctx.device_status() == 0


def test_noalloc_sort_empty_and_overlap(ctx):
    """n = 0 returns RT_OK; an output that overlaps an input, even by one
    pair, or the other output is refused; buffers that only touch sort."""
    lib = ctx.lib
    assert lib.rt_sort_pairs_noalloc(ctx.h, None, None, None, None, 0, 30, None) == 0
    n = 1024
    rng = np.random.default_rng(11)
    data = rng.integers(0, 2 ** 30, size=4 * n, dtype=np.uint64).astype(np.uint32)
    buf = ctx.to_device(data)                  # 4 arrays of n pairs' worth, back to back
    b, q = buf.ptr.value, 4 * n                # q: bytes of one array
    refused = [(b, b + q, b + 2 * q, b + 4),              # values out inside keys in
               (b, b + q, b, b + 3 * q),                  # keys out == keys in
               (b, b + q, b + 2 * q, b + 2 * q + q // 2),  # the two outputs meet
               (b, b + q, b + q - 4, b + 3 * q)]           # keys out starts in values in
    for ki, vi, ko, vo in refused:
        r = lib.rt_sort_pairs_noalloc(ctx.h, C.c_void_p(ki), C.c_void_p(vi), C.c_void_p(ko),
                                      C.c_void_p(vo), n, 30, None)
        assert r == -2 and b"overlaps" in lib.rt_last_error()
    # inputs in arrays 2 and 3, outputs in 0 and 1: adjacent ranges, no overlap
    r = lib.rt_sort_pairs_noalloc(ctx.h, C.c_void_p(b + 2 * q), C.c_void_p(b + 3 * q),
                                  C.c_void_p(b), C.c_void_p(b + q), n, 30, None)
    assert r == 0
    ctx.sync()
    out = buf.read(np.uint32)
    keys, vals = data[2 * n:3 * n], data[3 * n:]
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(out[:n], keys[order]) and np.array_equal(out[n:2 * n], vals[order])
    assert ctx.device_status() == 0
