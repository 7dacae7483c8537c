"""Whole benchmark configurations against the oracle, every frame or view:
the 300-frame street-level path with all 100k boxes (persistent rasterizer,
stale depth), all 256 views of the multi-view workload in one batch, and the
large workload's 4K main view with its 63 auxiliary views in one batch.  The
oracle runs in spawned worker processes (tests/oracle_pool.py), one task per
view or per stretch of frames; results are compared by digest (raw depth,
hiZ, visibility and needs-clipping bits)."""
import os

import numpy as np
import pytest

from rasterizer_gb300 import api, scenes

from helpers import city_occluders, large_city_occluders, to_baked
import oracle_pool

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CITY = os.path.join(HERE, "golden", "city_occluders.npz")  # the reference's bake of the city


@pytest.fixture(scope="module")
def city_pool():
    p = oracle_pool.pool(CITY)
    yield p
    p.close()
    p.join()


@pytest.fixture(scope="module")
def ctx(city_pool):
    c = api.Context(0)
    yield c
    c.close()


def _gpu(raster, vis, nc):
    return {"depth": oracle_pool.digest(raster.readDepthRaw()), "hiz": oracle_pool.digest(raster.readHiZ()),
            "visible": oracle_pool.digest(vis.astype(np.uint8)),
            "needsClipping": oracle_pool.digest(nc.astype(np.uint8))}


def _diff(got, want):
    return [k for k in want if got[k] != want[k]]


def test_config1_all_frames_all_boxes(ctx, city_pool):
    """Config 1: all 300 frames of the street-level path, all 100k boxes, one
    persistent rasterizer drawn through a prepared batch (occluders gated on
    the GPU).  Each stretch of 25 frames is replayed by a worker from the
    GPU's state before its first frame (stale depth included), so every frame
    is checked against the oracle applied to the state the frame before left."""
    from oracle.bindings import load_baked_scene
    occ = city_occluders()
    assert load_baked_scene(CITY).quads == sum(o.quads for o in occ)
    mvps, _ = scenes.camera_path(300, seed=7)
    mins, maxs = scenes.query_boxes(100_000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    r = api.Rasterizer(ctx, 1920, 1080)
    b = api.PreparedBatch(ctx, [dict(raster=r, mvp=mvps[0], clear=True, occluders=occ,
                                     flags=np.full(len(occ), 2, np.uint8), mins=mins, maxs=maxs)])
    tasks, got = [], []
    span = 25
    for f in range(300):
        if f % span == 0:  # the state this stretch starts from (the preparing launch drew frame 0 once)
            tasks.append({"key": f, "width": 1920, "height": 1080, "frames": [mvps[g] for g in range(f, f + span)],
                          "order": None, "mins": mins, "maxs": maxs, "depth": r.readDepthRaw(), "hiz": r.readHiZ()})
        b.setModelViewProjection(0, mvps[f])
        b.launch()
        assert b.check(), f
        vis, nc = b.results(0)
        got.append(_gpu(r, vis, nc))
    b.close()
    r.close()
    bad = []
    for res in city_pool.imap_unordered(oracle_pool.view_task, tasks):
        for i, want in enumerate(res["frames"]):
            d = _diff(got[res["key"] + i], want)
            if d:
                bad.append((res["key"] + i, d))
    assert not bad, f"frames differing from the oracle: {sorted(bad)[:10]}"


def test_config2_all_256_views(ctx, city_pool):
    """Config 2: every view of the 256-view workload (64 cascades 1024^2, 96
    cube faces 512^2, 96 probe views 256x128..1920x1080, each with its own
    occluder subset in its own order and 10k-100k boxes) in one batch."""
    occ = city_occluders()
    centers = np.stack([o.center for o in occ])
    quads = np.array([o.quads for o in occ])
    pmin, pmax = scenes.query_boxes(100_000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    specs = scenes.multiview_workload(centers, quads, len(pmin))
    assert len(specs) == 256
    views = []
    for s in specs:
        sel = [occ[i] for i in s.occluders]
        views.append(dict(raster=api.Rasterizer(ctx, s.width, s.height), mvp=s.mvp, clear=True, occluders=sel,
                          flags=np.full(len(sel), 2, np.uint8), mins=pmin[s.query_start:s.query_start + s.query_count],
                          maxs=pmax[s.query_start:s.query_start + s.query_count]))
    res = api.execute_batch(ctx, views)
    tasks = [{"key": k, "width": s.width, "height": s.height, "mvp": s.mvp, "order": s.occluders,
              "mins": v["mins"], "maxs": v["maxs"]} for k, (s, v) in enumerate(zip(specs, views))]
    got = [_gpu(v["raster"], vis, nc) for v, (vis, nc) in zip(views, res)]
    for v in views:
        v["raster"].close()
    bad = []
    for r in city_pool.imap_unordered(oracle_pool.view_task, tasks):
        d = _diff(got[r["key"]], r["frames"][0])
        if d:
            bad.append((r["key"], specs[r["key"]].kind, d))
    assert not bad, f"views differing from the oracle: {sorted(bad)[:10]}"


def test_config4_main_view_and_63_auxiliary_views(ctx, tmp_path):
    """Config 4: the 2M-triangle city's 3840x2160 main view (every occluder,
    1M boxes) and its 63 auxiliary views (16 cascades, 24 cube faces, 23
    probes, each with its own subset and boxes) in one batch."""
    from oracle.bindings import save_baked_scene
    occ = large_city_occluders()
    path = str(tmp_path / "city2m.npz")
    save_baked_scene(path, to_baked(occ))
    centers = np.stack([o.center for o in occ])
    quads = np.array([o.quads for o in occ])
    nq = 1_000_000
    pmin, pmax = scenes.query_boxes(nq, seed=45, footprint=600.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    mvps, aux = scenes.large_workload(centers, quads, nq, seed=5, frames=1)
    assert len(aux) == 63
    views = [dict(raster=api.Rasterizer(ctx, 3840, 2160), mvp=mvps[0], clear=True, occluders=occ,
                  flags=np.full(len(occ), 2, np.uint8), mins=pmin, maxs=pmax)]
    for s in aux:
        sel = [occ[i] for i in s.occluders]
        views.append(dict(raster=api.Rasterizer(ctx, s.width, s.height), mvp=s.mvp, clear=True, occluders=sel,
                          flags=np.full(len(sel), 2, np.uint8), mins=pmin[s.query_start:s.query_start + s.query_count],
                          maxs=pmax[s.query_start:s.query_start + s.query_count]))
    res = api.execute_batch(ctx, views)
    got = [_gpu(v["raster"], vis, nc) for v, (vis, nc) in zip(views, res)]
    tasks = [{"key": 0, "width": 3840, "height": 2160, "mvp": mvps[0], "order": None, "mins": pmin, "maxs": pmax}]
    tasks += [{"key": k + 1, "width": s.width, "height": s.height, "mvp": s.mvp, "order": s.occluders,
               "mins": views[k + 1]["mins"], "maxs": views[k + 1]["maxs"]} for k, s in enumerate(aux)]
    for v in views:
        v["raster"].close()
    bad = []
    with oracle_pool.pool(path) as p:
        for r in p.imap_unordered(oracle_pool.view_task, tasks):
            d = _diff(got[r["key"]], r["frames"][0])
            if d:
                bad.append((r["key"], d))
    assert not bad, f"views differing from the oracle: {sorted(bad)[:10]}"
