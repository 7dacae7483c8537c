"""GPU parity: the CUDA rasteriser against the CPU oracle, bit for bit.

Depth (raw, stale blocks included), hiZ, per-occluder gating flags, visibility
and needs-clipping bits, and readBackDepth must all match exactly.
"""
import numpy as np
import pytest

from rasterizer_gb300 import api, scenes
from oracle.bindings import Oracle

from helpers import boxes_occluders, city_occluders, gpu_plain_frame, mismatch_report, to_baked

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def _compare(r: api.Rasterizer, orc: Oracle, what=("depth", "hiz", "readback")):
    errs = []
    if "depth" in what:
        errs.append(mismatch_report("depth", r.readDepthRaw(), orc.depth()))
    if "hiz" in what:
        errs.append(mismatch_report("hiz", r.readHiZ(), orc.hiz()))
    if "readback" in what:
        errs.append(mismatch_report("readback", r.readBackDepth().ravel(), orc.read_back()))
    errs = [e for e in errs if e]
    assert not errs, "; ".join(errs)


def test_boxes_scene_1080p(ctx):
    """Plain method, single view, 1920x1080, 64 boxes + ground, 4096 queries."""
    occ = boxes_occluders()
    scene = to_baked(occ)
    mvp = scenes.boxes_camera()
    mins, maxs = scenes.query_boxes(4096, seed=43)
    r = api.Rasterizer(ctx, 1920, 1080)
    flags = gpu_plain_frame(r, occ, mvp)
    vis, nc = r.queryVisibilityBatch(mins, maxs)
    orc = Oracle(1920, 1080)
    oflags = orc.frame_plain(scene, mvp)
    ovis, onc = orc.query(mins, maxs)
    assert np.array_equal(flags, oflags)
    _compare(r, orc)
    assert not mismatch_report("visible", vis.astype(np.uint8), ovis)
    assert not mismatch_report("needsClipping", nc.astype(np.uint8), onc)
    assert vis.sum() > 0 and (~vis).sum() > 0


@pytest.mark.parametrize("near_clip", [0, 1])
def test_explicit_variants(ctx, near_clip):
    """rasterize<false> and rasterize<true> forced for every occluder."""
    occ = boxes_occluders()
    scene = to_baked(occ)
    mvp = scenes.view_projection((5.0, 3.0, -40.0), (0.1, -0.15, 1.0))
    r = api.Rasterizer(ctx, 640, 360)
    orc = Oracle(640, 360)
    r.clear()
    orc.clear()
    r.setModelViewProjection(mvp)
    orc.set_mvp(mvp)
    for o, k in zip(occ, range(len(scene))):
        r.rasterize(o, bool(near_clip))
        orc.rasterize(scene.packed[k], scene.packets[k], scene.ref[k, :4], scene.ref[k, 4:], bool(near_clip))
    _compare(r, orc)


def test_city_camera_path(ctx):
    """Dense city, persistent rasterizer across frames of a street-level path
    (stale depth in cleared blocks is part of the compared state)."""
    occ = city_occluders()
    scene = to_baked(occ)
    mvps, _ = scenes.camera_path(300, seed=7)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    r = api.Rasterizer(ctx, 1920, 1080)
    orc = Oracle(1920, 1080)
    near_clipped = 0
    for f in range(0, 300, 20):
        flags = gpu_plain_frame(r, occ, mvps[f])
        oflags = orc.frame_plain(scene, mvps[f])
        assert np.array_equal(flags, oflags), f"frame {f}"
        near_clipped += int(((flags & 3) == 3).sum())
        vis, nc = r.queryVisibilityBatch(mins, maxs)
        ovis, onc = orc.query(mins, maxs)
        assert not mismatch_report(f"frame {f} visible", vis.astype(np.uint8), ovis)
        assert not mismatch_report(f"frame {f} needsClipping", nc.astype(np.uint8), onc)
        _compare(r, orc, ("depth", "hiz"))
    assert near_clipped > 0


@pytest.mark.parametrize("size", [(8, 8), (264, 136), (1032, 520)])
def test_odd_sizes(ctx, size):
    """Views whose block grid is not a multiple of the warp-tile or super-tile."""
    w, h = size
    occ = boxes_occluders()
    scene = to_baked(occ)
    mvp = scenes.view_projection((0.0, 4.0, -30.0), (0.05, -0.1, 1.0), aspect=w / h)
    r = api.Rasterizer(ctx, w, h)
    orc = Oracle(w, h)
    flags = gpu_plain_frame(r, occ, mvp)
    oflags = orc.frame_plain(scene, mvp)
    assert np.array_equal(flags, oflags)
    _compare(r, orc)
    mins, maxs = scenes.query_boxes(2000, seed=9)
    vis, nc = r.queryVisibilityBatch(mins, maxs)
    ovis, onc = orc.query(mins, maxs)
    assert np.array_equal(vis.astype(np.uint8), ovis) and np.array_equal(nc.astype(np.uint8), onc)


def test_stale_state_without_clear(ctx):
    """Seeded depth and hiZ (values 0..65535, including the cleared marker 1)
    and no clear: merging against memory and the hiZ == 1 overwrite rule."""
    rng = np.random.default_rng(5)
    w, h = 320, 200
    occ = boxes_occluders()
    scene = to_baked(occ)
    depth = rng.integers(0, 65536, w * h, dtype=np.uint16)
    hiz = rng.choice(np.array([0, 1, 2, 500, 30000, 65535], np.uint16), (w // 8) * (h // 8) + 8)
    r = api.Rasterizer(ctx, w, h)
    orc = Oracle(w, h)
    r.writeDepthRaw(depth)
    r.writeHiZ(hiz)
    orc.write_depth(depth)
    orc.write_hiz(hiz)
    mvp = scenes.view_projection((0.0, 2.0, -25.0), (0.0, 0.0, 1.0), aspect=w / h)
    r.setModelViewProjection(mvp)
    orc.set_mvp(mvp)
    for k, o in enumerate(occ):
        r.rasterize(o, False)
        orc.rasterize(scene.packed[k], scene.packets[k], scene.ref[k, :4], scene.ref[k, 4:], False)
    _compare(r, orc)
    mins, maxs = scenes.query_boxes(3000, seed=10)
    vis, nc = r.queryVisibilityBatch(mins, maxs)
    ovis, onc = orc.query(mins, maxs)
    assert np.array_equal(vis.astype(np.uint8), ovis) and np.array_equal(nc.astype(np.uint8), onc)


def test_query_only_and_query2d(ctx):
    occ = boxes_occluders()
    scene = to_baked(occ)
    r = api.Rasterizer(ctx, 640, 480)
    orc = Oracle(640, 480)
    mvp = scenes.view_projection((0.0, 1.7, -60.0), (0.0, 0.0, 1.0), aspect=640 / 480)
    gpu_plain_frame(r, occ, mvp)
    orc.frame_plain(scene, mvp)
    rng = np.random.default_rng(3)
    for _ in range(40):
        x0, x1 = sorted(rng.integers(0, 640, 2))
        y0, y1 = sorted(rng.integers(0, 480, 2))
        z = int(rng.integers(0, 65536))
        assert r.query2D(x0, x1, y0, y1, z) == bool(orc.lib.orc_query2d(orc.h, x0, x1, y0, y1, z))


def test_4k_view_full_block_index(ctx):
    """3840x2160 (129,600 blocks): the GPU uses the full 32-bit block index;
    the oracle is run with the same correction of Rasterizer.cpp:1054."""
    occ = boxes_occluders()
    scene = to_baked(occ)
    mvp = scenes.boxes_camera(3840, 2160)
    r = api.Rasterizer(ctx, 3840, 2160)
    orc = Oracle(3840, 2160)
    orc.set_block_index_wrap(False)
    gpu_plain_frame(r, occ, mvp)
    orc.frame_plain(scene, mvp)
    _compare(r, orc, ("depth", "hiz"))


def test_batched_views_match_single_views(ctx):
    """Several views of uneven size in one batch == each view on the oracle."""
    occ = boxes_occluders()
    scene = to_baked(occ)
    sizes = [(1024, 1024), (512, 512), (256, 128), (1920, 1080), (640, 360)]
    views, oracles = [], []
    for i, (w, h) in enumerate(sizes):
        ang = 0.4 * i
        mvp = scenes.view_projection((40 * np.sin(ang), 2.0 + i, -40 * np.cos(ang)),
                                     (-np.sin(ang), -0.05, np.cos(ang)), aspect=w / h)
        mins, maxs = scenes.query_boxes(1000 + 300 * i, seed=100 + i)
        r = api.Rasterizer(ctx, w, h)
        views.append(dict(raster=r, mvp=mvp, clear=True, occluders=occ, flags=np.full(len(occ), 2, np.uint8),
                          mins=mins, maxs=maxs))
        orc = Oracle(w, h)
        orc.frame_plain(scene, mvp)
        oracles.append((orc, orc.query(mins, maxs)))
    res = api.execute_batch(ctx, views)
    for v, (orc, (ovis, onc)) in zip(views, oracles):
        _compare(v["raster"], orc, ("depth", "hiz"))
    for (vis, nc), (orc, (ovis, onc)) in zip(res, oracles):
        assert np.array_equal(vis.astype(np.uint8), ovis) and np.array_equal(nc.astype(np.uint8), onc)


def test_prepared_batch_graph(ctx):
    """CUDA-graph launches with a changing matrix reproduce the oracle."""
    occ = boxes_occluders()
    scene = to_baked(occ)
    mins, maxs = scenes.query_boxes(4096, seed=43)
    r = api.Rasterizer(ctx, 1920, 1080)
    mvps = [scenes.view_projection((x, 1.7, -60.0), (0.0, 0.0, 1.0)) for x in (0.0, 10.0, -20.0)]
    b = api.PreparedBatch(ctx, [dict(raster=r, mvp=mvps[0], clear=True, occluders=occ,
                                     flags=np.full(len(occ), 2, np.uint8), mins=mins, maxs=maxs)])
    orc = Oracle(1920, 1080)
    for m in mvps:
        b.setModelViewProjection(0, m)
        b.launch()
        assert b.check()
        vis, nc = b.results(0)
        orc.frame_plain(scene, m)
        ovis, onc = orc.query(mins, maxs)
        assert np.array_equal(vis.astype(np.uint8), ovis) and np.array_equal(nc.astype(np.uint8), onc)
        _compare(r, orc, ("depth", "hiz"))
    b.close()


def test_multiview_workload_subset(ctx):
    """Views of the 256-view workload (cascades, cube faces, probe views with
    their own occluder subsets and query ranges) in one batch == the oracle,
    view by view."""
    occ = city_occluders()
    scene = to_baked(occ)
    centers = np.stack([o.center for o in occ])
    quads = np.array([o.quads for o in occ])
    pool_min, pool_max = scenes.query_boxes(100_000, seed=44, footprint=300.0, lognormal=(0.0, 1.0),
                                            y_range=(0.0, 20.0))
    specs = scenes.multiview_workload(centers, quads, len(pool_min))
    pick = specs[:2] + specs[64:70] + specs[160:163]
    views = []
    for s in pick:
        r = api.Rasterizer(ctx, s.width, s.height)
        sel = [occ[i] for i in s.occluders]
        views.append(dict(raster=r, mvp=s.mvp, clear=True, occluders=sel, flags=np.full(len(sel), 2, np.uint8),
                          mins=pool_min[s.query_start:s.query_start + s.query_count],
                          maxs=pool_max[s.query_start:s.query_start + s.query_count]))
    res = api.execute_batch(ctx, views)
    for s, v, (vis, nc) in zip(pick, views, res):
        orc = Oracle(s.width, s.height)
        orc.frame_plain(scene, s.mvp, order=s.occluders)
        ovis, onc = orc.query(v["mins"], v["maxs"])
        _compare(v["raster"], orc, ("depth", "hiz"))
        assert np.array_equal(vis.astype(np.uint8), ovis), s.kind
        assert np.array_equal(nc.astype(np.uint8), onc), s.kind


def test_autotuned_launch_shapes_keep_results(ctx):
    """Launch shapes picked by the autotuner (CTAs per SM, tiles per fetch)
    change timing only: the batch still reproduces the oracle."""
    occ = city_occluders()
    scene = to_baked(occ)
    w, h = 960, 544
    mvps, _ = scenes.camera_path(30, seed=29, width=w, height_px=h)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    r = api.Rasterizer(ctx, w, h)
    b = api.PreparedBatch(ctx, [dict(raster=r, mvp=mvps[0], clear=True, occluders=occ,
                                     flags=np.full(len(occ), 2, np.uint8), mins=mins, maxs=maxs)])
    rep = b.autotune(2)
    assert all(v >= 1 for v in rep["tuned"].values())
    orc = Oracle(w, h)
    orc.frame_plain(scene, mvps[0])  # the preparing frame
    for f in (5, 17):
        b.setModelViewProjection(0, mvps[f])
        b.launch()
        assert b.check()
        orc.frame_plain(scene, mvps[f])
        vis, _ = b.results(0)
        ovis, _ = orc.query(mins, maxs)
        assert np.array_equal(vis.astype(np.uint8), ovis)
        _compare(r, orc, ("depth", "hiz"))
    b.close()


@pytest.mark.parametrize("rows,threads,st", [(1, 32, 16), (2, 32, 16), (4, 32, 16), (2, 128, 16), (1, 128, 16),
                                             (2, 32, 8), (2, 128, 8)])
def test_raster_unit_shapes(ctx, rows, threads, st):
    """Raster units of 1, 2 and 4 block rows per warp, and 1- and 2-row units
    per 128-thread CTA, with super-tiles of 16 and 8 blocks (choices of the
    autotuner), give the oracle's frames: two views on persistent rasterizers,
    frames in the reference's clear (stale depth merged and queried), then in
    the zero-depth clear, with win counting on (the other kernel variant)."""
    occ = city_occluders()
    scene = to_baked(occ)
    w, h = 960, 544
    mvps, _ = scenes.camera_path(40, seed=31, width=w, height_px=h)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    rs = [api.Rasterizer(ctx, w, h) for _ in range(2)]
    starts = (0, 11)
    views = [dict(raster=r, mvp=mvps[s], clear=True, occluders=occ, flags=np.full(len(occ), 2, np.uint8),
                  mins=mins, maxs=maxs) for r, s in zip(rs, starts)]
    b = api.PreparedBatch(ctx, views)
    b.setTuning({"raster_unit_rows": rows, "raster_threads_per_unit": threads, "super_tile_blocks": st})
    orcs = [Oracle(w, h) for _ in rs]
    for o, s in zip(orcs, starts):
        o.frame_plain(scene, mvps[s])  # the preparing frame
    for step, (f, zero, wins) in enumerate(((3, False, False), (7, False, True), (19, True, True), (23, True, False))):
        if step == 1 or step == 3:
            b.setSelection(None, 1.0, trackWins=wins)
        b.setZeroDepth(zero)
        for v, o in enumerate(orcs):
            b.setModelViewProjection(v, mvps[f + starts[v]])
            if zero:
                o.write_depth(np.zeros(w * h, np.uint16))
        b.launch()
        assert b.check()
        for v, (r, o) in enumerate(zip(rs, orcs)):
            o.frame_plain(scene, mvps[f + starts[v]])
            vis, nc = b.results(v)
            ovis, onc = o.query(mins, maxs)
            assert np.array_equal(vis.astype(np.uint8), ovis), (rows, f, v)
            assert np.array_equal(nc.astype(np.uint8), onc), (rows, f, v)
            _compare(r, o, ("depth", "hiz"))
    b.close()


def test_large_city_4k_main_view(ctx):
    """The 2M-triangle city's 3840x2160 main view (129,600 blocks, full 32-bit
    block index) with every occluder gated, and 200k boxes, against the oracle."""
    from helpers import large_city_occluders
    occ = large_city_occluders()
    scene = to_baked(occ)
    mvps, _ = scenes.camera_path(3, seed=5, grid=128, width=3840, height_px=2160)
    mins, maxs = scenes.query_boxes(200_000, seed=45, footprint=600.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    r = api.Rasterizer(ctx, 3840, 2160)
    orc = Oracle(3840, 2160)
    orc.set_block_index_wrap(False)
    for f in (0, 2):
        flags = gpu_plain_frame(r, occ, mvps[f])
        oflags = orc.frame_plain(scene, mvps[f])
        assert np.array_equal(flags, oflags)
        _compare(r, orc, ("depth", "hiz"))
        vis, nc = r.queryVisibilityBatch(mins, maxs)
        ovis, onc = orc.query(mins, maxs)
        assert np.array_equal(vis.astype(np.uint8), ovis) and np.array_equal(nc.astype(np.uint8), onc)
        assert (flags & 1).sum() > 100


def test_query_special_values(ctx):
    """Boxes with NaN, infinite, huge, tiny and signed-zero coordinates: the
    x86 NaN and overflow rules of queryVisibility, bit for bit."""
    from helpers import special_boxes
    occ = boxes_occluders()
    scene = to_baked(occ)
    mvp = scenes.view_projection((3.0, 2.0, -50.0), (0.0, -0.05, 1.0), aspect=640 / 360)
    r = api.Rasterizer(ctx, 640, 360)
    orc = Oracle(640, 360)
    gpu_plain_frame(r, occ, mvp)
    orc.frame_plain(scene, mvp)
    mins, maxs = special_boxes(8192, seed=61)
    vis, nc = r.queryVisibilityBatch(mins, maxs)
    ovis, onc = orc.query(mins, maxs)
    assert not mismatch_report("visible", vis.astype(np.uint8), ovis)
    assert not mismatch_report("needsClipping", nc.astype(np.uint8), onc)
    assert vis.sum() > 0 and (~vis).sum() > 0


@pytest.mark.parametrize("form", [255, 1, 2, 4, 8])
def test_query_forms(ctx, form):
    """Both query kernels -- one box per thread, and frustum survivors
    listed per warp over 1-8 rounds of 32 slots -- give the oracle's bits,
    special values (NaN, infinities, huge and signed-zero coordinates) included,
    over views whose slot ranges share CTAs (one view without boxes)."""
    from helpers import special_boxes
    occ = boxes_occluders()
    scene = to_baked(occ)
    sizes = [(640, 360), (320, 200), (512, 512), (64, 64), (256, 128)]
    counts = [5000, 3000, 0, 90, 700]
    views, orcs = [], []
    for i, ((w, h), n) in enumerate(zip(sizes, counts)):
        mvp = scenes.view_projection((3.0 + 4 * i, 2.0, -50.0), (0.0, -0.05, 1.0), aspect=w / h)
        if i == 1:
            mins, maxs = special_boxes(n, seed=61)
        elif n:
            mins, maxs = scenes.query_boxes(n, seed=80 + i)
        else:
            mins = maxs = None
        views.append(dict(raster=api.Rasterizer(ctx, w, h), mvp=mvp, clear=True, occluders=occ,
                          flags=np.full(len(occ), 2, np.uint8), mins=mins, maxs=maxs))
        orc = Oracle(w, h)
        orc.frame_plain(scene, mvp)
        orcs.append(orc)
    b = api.PreparedBatch(ctx, views)  # runs the frame once to prepare
    b.setTuning({"query_rounds": form})
    b.launch()
    assert b.check()
    for v, (view, orc) in enumerate(zip(views, orcs)):
        orc.frame_plain(scene, view["mvp"])  # the same frame again: the launch
        vis, nc = b.results(v)
        if view["mins"] is None:
            assert len(vis) == 0
            continue
        ovis, onc = orc.query(view["mins"], view["maxs"])
        assert not mismatch_report(f"visible view {v}", vis.astype(np.uint8), ovis)
        assert not mismatch_report(f"needsClipping view {v}", nc.astype(np.uint8), onc)
        _compare(view["raster"], orc, ("depth", "hiz"))
    b.close()


def test_read_back_formats(ctx):
    """Every read-back format (the reference's RGBA bytes, float linDepth,
    float depth, packed u16) == the oracle's, after a city frame with stale
    and cleared blocks."""
    occ = city_occluders()
    scene = to_baked(occ)
    w, h = 960, 544
    mvps, _ = scenes.camera_path(10, seed=33, width=w, height_px=h)
    r = api.Rasterizer(ctx, w, h)
    orc = Oracle(w, h)
    for f in (0, 7):
        gpu_plain_frame(r, occ, mvps[f])
        orc.frame_plain(scene, mvps[f])
    assert not mismatch_report("rgba8", r.readBack("rgba8").ravel(), orc.read_back())
    for k in ("linear", "depth", "packed"):
        got, want = r.readBack(k), orc.read_back_values(k)
        assert not mismatch_report(k, got.view(np.uint32 if got.dtype == np.float32 else np.uint16),
                                   want.view(np.uint32 if want.dtype == np.float32 else np.uint16))


def test_bulk_matrices_and_results(ctx):
    """Matrices of many views in one call and every view's bits in one copy
    give what the per-view calls give."""
    occ = boxes_occluders()
    sizes = [(640, 360), (320, 200), (512, 512)]
    views, mvps = [], []
    for i, (w, h) in enumerate(sizes):
        mvps.append(scenes.view_projection((5.0 * i, 2.0, -40.0), (0.0, -0.05, 1.0), aspect=w / h))
        mins, maxs = scenes.query_boxes(700 + 100 * i, seed=70 + i)
        views.append(dict(raster=api.Rasterizer(ctx, w, h), mvp=mvps[-1], clear=True, occluders=occ,
                          flags=np.full(len(occ), 2, np.uint8), mins=mins, maxs=maxs))
    b = api.PreparedBatch(ctx, views)
    moved = [scenes.view_projection((5.0 * i + 3, 2.5, -38.0), (0.05, -0.05, 1.0), aspect=w / h)
             for i, (w, h) in enumerate(sizes)]
    b.setModelViewProjections(np.stack(moved))
    b.launch()
    assert b.check()
    bulk = b.resultsAll(unpack=True)
    single = [b.results(v) for v in range(len(views))]
    for (bv, bn), (sv, sn) in zip(bulk, single):
        assert np.array_equal(bv, sv) and np.array_equal(bn, sn)
    for v, m in enumerate(moved):
        b.setModelViewProjection(v, m)
    b.launch()
    assert b.check()
    for v, (sv, sn) in enumerate(single):
        vv, nn = b.results(v)
        assert np.array_equal(vv, sv) and np.array_equal(nn, sn)
    b.close()


def test_batch_query_boxes_replaced_per_launch(ctx):
    """occ_batch_set_queries: new boxes for every view before a launch (views
    of 64, 50 and 96 boxes: contiguous slot ranges copied together, a padded
    one alone) answer as the oracle does, and occ_batch_results_all_async
    returns the same bits as the synchronous copy."""
    occ = boxes_occluders()
    scene = to_baked(occ)
    w, h = 640, 360
    mvp = scenes.boxes_camera(w, h)
    counts = (64, 50, 96)
    first = [scenes.query_boxes(n, seed=60 + k) for k, n in enumerate(counts)]
    views = [dict(raster=api.Rasterizer(ctx, w, h), mvp=mvp, clear=True, occluders=occ,
                  flags=np.full(len(occ), 2, np.uint8), mins=m, maxs=M) for m, M in first]
    b = api.PreparedBatch(ctx, views)
    orc = Oracle(w, h)
    orc.frame_plain(scene, mvp)
    for rnd in range(2):
        new = [scenes.query_boxes(n, seed=70 + 5 * rnd + k) for k, n in enumerate(counts)]
        b.setQueries(np.concatenate([m for m, _ in new]), np.concatenate([M for _, M in new]))
        b.launch()
        assert b.check()
        res = b.resultsAll(unpack=True)
        words = b.resultWords()
        vis_a, nc_a = np.zeros(words, np.uint32), np.zeros(words, np.uint32)
        b.resultsAllAsync(vis_a, nc_a)
        ctx.synchronize()
        vis_s, nc_s, _ = b.resultsAll()
        assert np.array_equal(vis_a, vis_s) and np.array_equal(nc_a, nc_s)
        for (m, M), (vis, nc) in zip(new, res):
            ovis, onc = orc.query(m, M)
            assert np.array_equal(vis.astype(np.uint8), ovis) and np.array_equal(nc.astype(np.uint8), onc)
    b.close()
    for v in views:
        v["raster"].close()
