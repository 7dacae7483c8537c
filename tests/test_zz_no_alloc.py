"""occ_raster_query_batch_noalloc: queries for callers that must not allocate
device memory (host callbacks, fixed-budget frame loops), staged in one fixed
device array instead of per-context buffers.  Checked through the C ABI
against occ_raster_query_batch on two calls in a row (the second call reuses
the array the first one left behind).  This file is named to run last."""
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
    # two calls in a row, different sizes: the second must not see the first's leftovers
    for n, seed in ((4096, 43), (1000, 7)):
        mins, maxs = scenes.query_boxes(n, seed=seed)
        mins, maxs = np.ascontiguousarray(mins), np.ascontiguousarray(maxs)
        (rv, rn), (gv, gn) = _query_both(lib, r, mins, maxs)
        # the unused high bits of the last word are zero in both results
        assert np.array_equal(gv, rv)
        assert np.array_equal(gn, rn)
        vis = api.unpack_bits(gv, n)
        assert 0 < vis.sum() < n
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
