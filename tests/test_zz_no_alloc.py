"""occ_raster_query_batch_noalloc: queries for callers that must not allocate
device memory (fixed-budget frame loops, engines that forbid cudaMalloc on
their frame thread), staged in one fixed device array instead of per-context
buffers.  Checked through the C ABI against occ_raster_query_batch on calls in
a row (each call reuses the array the previous one left behind), including a
batch that fills the array and an empty batch.  This file is named to run
last."""
import ctypes as C

import numpy as np
import pytest

from rasterizer_gb300 import _lib, api, scenes

from helpers import boxes_occluders, gpu_plain_frame

pytestmark = pytest.mark.gpu

P = C.c_void_p


def _ptr(a):
    return a.ctypes.data_as(P)


def _query_both(lib, r, mins, maxs):
    n = len(mins)
    words = (n + 31) // 32
    ref_v, ref_n = np.zeros(words, np.uint32), np.zeros(words, np.uint32)
    got_v, got_n = np.full(words, 0xDEADBEEF, np.uint32), np.full(words, 0xDEADBEEF, np.uint32)
    assert lib.occ_raster_query_batch(r.handle, n, _ptr(mins), _ptr(maxs), _ptr(ref_v), _ptr(ref_n)) == 0
    assert lib.occ_raster_query_batch_noalloc(r.handle, n, _ptr(mins), _ptr(maxs), _ptr(got_v), _ptr(got_n)) == 0, \
        lib.occ_last_error().decode()
    return (ref_v, ref_n), (got_v, got_n)


def test_noalloc_queries_match_the_allocating_entry_point():
    lib = _lib.lib()
    ctx = api.Context(0)
    r = api.Rasterizer(ctx, 1920, 1080)
    gpu_plain_frame(r, boxes_occluders(), scenes.boxes_camera())
    # calls in a row, different sizes: none may see the previous call's leftovers;
    # 65,536 boxes use every word of the fixed array
    for n, seed in ((4096, 43), (65536, 11), (1000, 7)):
        mins, maxs = scenes.query_boxes(n, seed=seed)
        mins, maxs = np.ascontiguousarray(mins), np.ascontiguousarray(maxs)
        (rv, rn), (gv, gn) = _query_both(lib, r, mins, maxs)
        # the unused high bits of the last word are zero in both results
        assert np.array_equal(gv, rv)
        assert np.array_equal(gn, rn)
        vis = api.unpack_bits(gv, n)
        assert 0 < vis.sum() < n
    # an empty batch succeeds and writes nothing
    mins = np.zeros((1, 4), np.float32)
    bits = np.full(1, 0xDEADBEEF, np.uint32)
    assert lib.occ_raster_query_batch_noalloc(r.handle, 0, _ptr(mins), _ptr(mins), _ptr(bits), _ptr(bits)) == 0
    assert bits[0] == 0xDEADBEEF
    r.close()
    ctx.close()


def test_noalloc_rejects_oversized_batches_and_pending_work():
    lib = _lib.lib()
    ctx = api.Context(0)
    r = api.Rasterizer(ctx, 64, 64)
    n = 65537
    mins = np.zeros((n, 4), np.float32)
    maxs = np.ones((n, 4), np.float32)
    bits = np.zeros((n + 31) // 32, np.uint32)
    assert lib.occ_raster_query_batch_noalloc(r.handle, n, _ptr(mins), _ptr(maxs), _ptr(bits), _ptr(bits)) == -1
    assert b"65536" in lib.occ_last_error()
    r.clear()  # pending work: the call must refuse instead of running it
    assert lib.occ_raster_query_batch_noalloc(r.handle, 1, _ptr(mins), _ptr(maxs), _ptr(bits), _ptr(bits)) == -1
    r.close()
    ctx.close()
