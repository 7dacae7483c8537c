"""GPU tests of the learned occluder selection: the network's tensor-core
forward and its training kernels against the CPU reference (oracle/mlp.py),
per-occluder pixel wins (the training labels) against the oracle rendering
occluder by occluder, and the selected-subset frame against the oracle drawing
exactly the selected occluders."""
import numpy as np
import pytest

from rasterizer_gb300 import api, scenes
from oracle import mlp as ref
from oracle.bindings import Oracle

from helpers import boxes_occluders, city_occluders, mismatch_report, to_baked

pytestmark = pytest.mark.gpu

GATED = 2


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def _random_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    p = np.zeros(ref.PARAMS, np.float32)
    p[0:1024] = rng.normal(0, np.sqrt(2 / 16) * scale, 1024)
    p[1024:1088] = rng.normal(0, 0.1, 64)
    p[1088:5184] = rng.normal(0, np.sqrt(2 / 64) * scale, 4096)
    p[5184:5248] = rng.normal(0, 0.1, 64)
    p[5248:5312] = rng.normal(0, np.sqrt(1 / 64), 64)
    p[5312] = 0.25
    return p


def _random_features(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, (n, 16)).astype(np.float32)
    x[:, 0] = rng.integers(0, 2, n)
    x[:, 15] = 1.0
    return x


def test_forward_matches_cpu_reference(ctx):
    """bf16 MMA (fp32 accumulation) scores == float64 restatement with the same
    bf16 rounding points, to fp32 accumulation-order tolerance; a row count
    that is not a multiple of the 16-row tile."""
    net = api.OccluderSelector(ctx, seed=1)
    p = _random_params(2)
    net.setParams(p)
    assert np.array_equal(net.params(), p)
    x = _random_features(1000, 3)
    s = net.forward(x)
    r = ref.forward(p, x)
    err = np.abs(s - r)
    # one bf16 ulp of one hidden unit moves a score by about 2^-9 of that unit's term
    assert err.max() <= 2e-3 * max(1.0, np.abs(r).max()), err.max()
    assert np.median(err) <= 1e-5 * max(1.0, np.abs(r).max())


def test_gradients_match_cpu_reference(ctx):
    net = api.OccluderSelector(ctx, seed=1)
    p = _random_params(4)
    net.setParams(p)
    x = _random_features(777, 5)
    t = np.random.default_rng(6).uniform(0, 1, len(x)).astype(np.float32)
    loss, g = net.gradients(x, t)
    rloss, rg = ref.gradients(p, x, t)
    assert abs(loss - rloss) <= 1e-4 * max(1.0, rloss)
    for name, (a, b) in dict(W1=(0, 1024), b1=(1024, 1088), W2=(1088, 5184), b2=(5184, 5248), w3=(5248, 5312),
                             b3=(5312, 5313)).items():
        d = np.linalg.norm(g[a:b] - rg[a:b]) / max(np.linalg.norm(rg[a:b]), 1e-12)
        assert d < 5e-3, (name, d)


def test_listwise_gradients_match_cpu_reference(ctx):
    net = api.OccluderSelector(ctx, seed=1)
    p = _random_params(14)
    net.setParams(p)
    rng = np.random.default_rng(15)
    sizes = rng.integers(1, 60, 40)
    gs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    x = _random_features(int(gs[-1]), 16)
    t = rng.uniform(0, 1, len(x)) ** 3
    for a, b in zip(gs[:-1], gs[1:]):
        t[a:b] /= t[a:b].sum()
    loss, g = net.gradientsListwise(x, t.astype(np.float32), gs)
    rloss, rg = ref.listwise_gradients(p, x, t.astype(np.float32), gs)
    assert abs(loss - rloss) <= 1e-4 * max(1.0, rloss)
    d = np.linalg.norm(g - rg) / np.linalg.norm(rg)
    assert d < 5e-3, d


def test_adam_step_matches_cpu_reference(ctx):
    net = api.OccluderSelector(ctx, seed=7)
    p = net.params()
    x = _random_features(512, 8)
    t = np.random.default_rng(9).uniform(0, 1, len(x)).astype(np.float32)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for step in (1, 2, 3):
        _, g = net.gradients(x, t)  # the train step computes the same gradient
        p_ref, m, v = ref.adam(p, g, m, v, step, 1e-3)
        net.trainStep(x, t, lr=1e-3)
        p = net.params()
        assert np.allclose(p, p_ref, rtol=0, atol=1e-6), np.abs(p - p_ref).max()


def test_training_reduces_loss(ctx):
    """Fit a smooth target of the features: the loss falls by an order of magnitude."""
    net = api.OccluderSelector(ctx, seed=11)
    rng = np.random.default_rng(12)
    x = _random_features(8192, 13)
    t = (0.6 * x[:, 2] * x[:, 0] + 0.3 * np.maximum(x[:, 6] - 0.5, 0) + 0.1 * x[:, 13]).astype(np.float32)
    first = net.trainStep(x[:1024], t[:1024], lr=3e-3)
    for it in range(400):
        i = rng.integers(0, len(x), 1024)
        net.trainStep(x[i], t[i], lr=3e-3)
    final, _ = net.gradients(x, t)
    assert final < first / 10, (first, final)


def _boxes_view(ctx, w=640, h=360, queries=3000):
    occ = boxes_occluders()
    mvp = scenes.view_projection((8.0, 2.5, -45.0), (-0.1, -0.05, 1.0), aspect=w / h)
    mins, maxs = scenes.query_boxes(queries, seed=21)
    r = api.Rasterizer(ctx, w, h)
    return occ, dict(raster=r, mvp=mvp, clear=True, occluders=occ, flags=np.full(len(occ), GATED, np.uint8),
                     mins=mins, maxs=maxs)


@pytest.mark.parametrize("rows,threads", [(1, 32), (2, 32), (4, 32), (2, 128)])
def test_pixel_wins_match_oracle(ctx, rows, threads):
    """Wins (pixels whose final depth an occluder produced) == the oracle drawn
    occluder by occluder, each pixel owned by the last occluder that changed it.
    The oracle starts from zeroed depth, so a nonzero value written into a
    cleared block counts as a change, which is the GPU's rule for cleared
    blocks.  Every raster form (1, 2, 4 block rows per warp; 2 rows per CTA)."""
    occ, view = _boxes_view(ctx)
    scene = to_baked(occ)
    b = api.PreparedBatch(ctx, [view])
    b.setTuning({"raster_unit_rows": rows, "raster_threads_per_unit": threads})
    b.setSelection(None, trackWins=True)
    b.launch()
    assert b.check()
    sel = b.selection(0)
    assert sel["features"][:, 13:15].sum() == 0  # no previous launch
    orc = Oracle(640, 360)
    orc.clear()
    orc.set_mvp(view["mvp"])
    owner = np.full(640 * 360, -1)
    prev = orc.depth().copy()
    for k in range(len(occ)):
        if not sel["candidate"][k]:
            continue
        nc = bool(sel["features"][k, 1])
        orc.rasterize(scene.packed[k], scene.packets[k], scene.ref[k, :4], scene.ref[k, 4:], nc)
        cur = orc.depth()
        owner[cur != prev] = k
        prev = cur.copy()
    expect = np.bincount(owner[owner >= 0], minlength=len(occ)).astype(np.uint32)
    assert not mismatch_report("wins", sel["wins"], expect)
    assert expect.sum() > 0
    # the next launch sees these wins as its previous-frame feature
    b.launch()
    assert b.check()
    sel2 = b.selection(0)
    assert np.array_equal(sel2["wins"], sel["wins"])
    assert np.array_equal(sel2["features"][:, 13] > 0, sel["wins"] > 0)
    assert np.array_equal(sel2["features"][:, 14] > 0, sel["candidate"])  # drawn in the previous launch
    b.close()


def test_full_fraction_equals_plain_frame(ctx):
    """Selecting 100% of the candidates is the plain all-occluder frame."""
    occ, view = _boxes_view(ctx)
    scene = to_baked(occ)
    net = api.OccluderSelector(ctx, seed=3)
    b = api.PreparedBatch(ctx, [view])
    b.setSelection(net, 1.0, trackWins=True)
    b.launch()
    assert b.check()
    sel = b.selection(0)
    assert np.array_equal(sel["selected"], sel["candidate"])
    orc = Oracle(640, 360)
    orc.frame_plain(scene, view["mvp"])
    vis, nc = b.results(0)
    ovis, onc = orc.query(view["mins"], view["maxs"])
    r = view["raster"]
    assert not mismatch_report("depth", r.readDepthRaw(), orc.depth())
    assert not mismatch_report("hiz", r.readHiZ(), orc.hiz())
    assert np.array_equal(vis.astype(np.uint8), ovis) and np.array_equal(nc.astype(np.uint8), onc)
    b.close()


@pytest.mark.parametrize("fraction", [0.05, 0.3, 0.6])
def test_top_k_subset_matches_oracle(ctx, fraction):
    """Top-K of the network's scores, and the frame drawing exactly those
    occluders, bit-exact against the oracle; the subset never culls a box the
    full frame shows (zero false culls)."""
    occ = city_occluders()
    scene = to_baked(occ)
    w, h = 960, 544
    mvps, _ = scenes.camera_path(40, seed=17, width=w, height_px=h)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    net = api.OccluderSelector(ctx, seed=5)
    r = api.Rasterizer(ctx, w, h)
    b = api.PreparedBatch(ctx, [dict(raster=r, mvp=mvps[0], clear=True, occluders=occ,
                                     flags=np.full(len(occ), GATED, np.uint8), mins=mins, maxs=maxs)])
    b.setSelection(net, fraction, trackWins=True)
    b.setZeroDepth(True)  # each frame stands alone, so it compares with a fresh full frame
    orc = Oracle(w, h)
    zeros = np.zeros(w * h, np.uint16)
    for f in (0, 10, 25):
        b.setModelViewProjection(0, mvps[f])
        b.launch()
        assert b.check()
        sel = b.selection(0)
        cand, chosen, score = sel["candidate"], sel["selected"], sel["score"]
        assert not (chosen & ~cand).any()
        ncand = int(cand.sum())
        k = min(max(int(np.ceil(np.float32(fraction) * np.float32(ncand))), 1), ncand)
        assert chosen.sum() == k
        assert np.array_equal(net.forward(sel["features"])[cand], score[cand])
        if k < ncand:
            assert score[chosen].min() >= score[cand & ~chosen].max()
        orc.clear()
        orc.write_depth(zeros)
        orc.set_mvp(mvps[f])
        for i in np.nonzero(chosen)[0]:
            orc.rasterize(scene.packed[i], scene.packets[i], scene.ref[i, :4], scene.ref[i, 4:],
                          bool(sel["features"][i, 1]))
        assert not mismatch_report(f"frame {f} depth", r.readDepthRaw(), orc.depth())
        assert not mismatch_report(f"frame {f} hiz", r.readHiZ(), orc.hiz())
        vis, _ = b.results(0)
        ovis, _ = orc.query(mins, maxs)
        assert np.array_equal(vis.astype(np.uint8), ovis)
        full = Oracle(w, h)
        full.frame_plain(scene, mvps[f])
        fvis, _ = full.query(mins, maxs)
        assert not (~vis & fvis.astype(bool)).any(), "false cull"
    b.close()


def test_trained_selector_gains_over_nearest_first(ctx, tmp_path):
    """A selector trained on the GPU (small recipe) against the reference's
    nearest-first ordering truncated at the same K, on held-out views of the
    256-view workload (K = 35 %) and on held-out street-level 1080p paths at
    the headline's K = 5 %: more occlusion culls kept, none false, and the
    checkpoint round trip reproduces its scores."""
    from rasterizer_gb300 import learned as L
    occ = city_occluders()
    centers = np.stack([o.center for o in occ])
    quads = np.array([o.quads for o in occ])
    mins, maxs = scenes.query_boxes(100_000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    recipe = L.Recipe(street_paths=8, street_frames=60, multiview_seeds=(101, 102), multiview_frames=6,
                      rounds=((0.25, 4, 40, (201,)),), steps0=2000, steps=2000)
    net, report = L.train_selector(ctx, occ, len(mins), recipe, log=None, mins=mins, maxs=maxs)
    assert report["rounds"][-1]["final_loss"] < report["rounds"][0]["final_loss"] * 1.5
    test = L.multiview_tracks(centers, quads, len(mins), frames=3, seed=3)[::2]
    full = L.run_full(ctx, occ, test, mins, maxs)
    a = L.evaluate_learned(ctx, occ, test, mins, maxs, net, 0.35, full)
    b = L.evaluate_heuristic(ctx, occ, test, mins, maxs, "nearest", 0.35, full)
    print("learned", a.as_dict(), "nearest", b.as_dict())
    assert a.false == 0 and b.false == 0
    assert a.full > 100_000
    assert a.retained > b.retained
    assert a.quads_drawn < 0.6 * a.quads_candidates
    street = L.street_tracks(4, 20, seed0=5000, n_occluders=len(occ), queries=len(mins))
    sfull = L.run_full(ctx, occ, street, mins, maxs)
    a = L.evaluate_learned(ctx, occ, street, mins, maxs, net, 0.05, sfull)
    b = L.evaluate_heuristic(ctx, occ, street, mins, maxs, "nearest", 0.05, sfull)
    print("street K=5%: learned", a.as_dict(), "nearest", b.as_dict())
    assert a.false == 0 and a.full > 100_000
    assert a.retained > b.retained
    # checkpoint: weights and Adam state survive a save/load into a fresh network
    x = _random_features(300, 31)
    path = tmp_path / "selector.npz"
    net.save(path)
    other = api.OccluderSelector(ctx, seed=99)
    other.load(path)
    assert np.array_equal(other.forward(x), net.forward(x))
    net.close()
    other.close()


def test_second_pass_matches_oracle(ctx):
    """Top-K pass, then the other candidates still visible against its buffer:
    bit-exact against the oracle drawing the two sets in that order, and no
    false cull against the full frame."""
    occ = city_occluders()
    scene = to_baked(occ)
    w, h = 960, 544
    mvps, _ = scenes.camera_path(30, seed=23, width=w, height_px=h)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    net = api.OccluderSelector(ctx, seed=8)
    r = api.Rasterizer(ctx, w, h)
    b = api.PreparedBatch(ctx, [dict(raster=r, mvp=mvps[0], clear=True, occluders=occ,
                                     flags=np.full(len(occ), GATED, np.uint8), mins=mins, maxs=maxs)])
    b.setSelection(net, 0.1, trackWins=True)
    b.setSecondPass(True)
    b.setZeroDepth(True)
    orc = Oracle(w, h)
    zeros = np.zeros(w * h, np.uint16)
    drawn_second = 0
    for f in (0, 12, 29):
        b.setModelViewProjection(0, mvps[f])
        b.launch()
        assert b.check()
        sel = b.selection(0)
        first = sel["selected"] & ~sel["second_pass"]
        second = sel["second_pass"]
        assert not (second & ~sel["candidate"]).any()
        drawn_second += int(second.sum())
        orc.clear()
        orc.write_depth(zeros)
        orc.set_mvp(mvps[f])
        for group in (first, second):
            for i in np.nonzero(group)[0]:
                orc.rasterize(scene.packed[i], scene.packets[i], scene.ref[i, :4], scene.ref[i, 4:],
                              bool(sel["features"][i, 1]))
        assert not mismatch_report(f"frame {f} depth", r.readDepthRaw(), orc.depth())
        assert not mismatch_report(f"frame {f} hiz", r.readHiZ(), orc.hiz())
        vis, _ = b.results(0)
        ovis, _ = orc.query(mins, maxs)
        assert np.array_equal(vis.astype(np.uint8), ovis)
        full = Oracle(w, h)
        full.frame_plain(scene, mvps[f])
        fvis, _ = full.query(mins, maxs)
        assert not (~vis & fvis.astype(bool)).any(), "false cull"
    assert drawn_second > 0
    b.close()


def test_cull_labels_consistent(ctx):
    """Cull credits: at most 16 samples per culled box, credited only to
    occluders that own pixels (wins > 0), and some credit on this view."""
    occ, view = _boxes_view(ctx)
    b = api.PreparedBatch(ctx, [view])
    b.setSelection(None, trackWins=True)
    b.setZeroDepth(True)
    b.setCullLabels(True)
    for _ in range(2):
        b.launch()
        assert b.check()
        counts = b.cullLabels(0)
        wins = b.selection(0)["wins"]
        vis, _ = b.results(0)
        assert counts.sum() > 0
        assert counts.sum() <= 16 * int((~vis).sum())
        assert not ((counts > 0) & (wins == 0)).any()
    b.close()


@pytest.mark.parametrize("zero", [True, False], ids=["zero-depth", "stale-depth"])
def test_headline_batch_matches_oracle(ctx, zero):
    """The benchmark's headline batch itself: 64 street-level 1920x1080 views
    of the city (the benchmark's seeded paths), the selector's top 5 % of each
    view's candidates, 100k query boxes per view, three consecutive launches
    (each launch's features hold the previous launch's wins and draw flags).
    Every view's depth, hiZ and query bits equal the oracle drawing the
    selected occluders in order on its own persistent rasterizer: in the
    zero-depth clear the headline times (a zeroed buffer each launch), and in
    the reference's clear (stale depth kept and queried)."""
    from rasterizer_gb300 import learned as L
    occ = city_occluders()
    scene = to_baked(occ)
    nq = 100_000
    pmin, pmax = scenes.query_boxes(nq, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    paths = L.street_tracks(64, 64, seed0=7000, n_occluders=len(occ), queries=nq)
    views = L._views(ctx, occ, paths, pmin, pmax)
    net = api.OccluderSelector(ctx, seed=0)
    b = api.PreparedBatch(ctx, views)
    w, h = 1920, 1080
    orcs = [Oracle(w, h) for _ in paths]
    for o, t in zip(orcs, paths):
        o.frame_plain(scene, t.mvps[0])  # the preparing frame (every candidate, the reference's clear)
    b.setSelection(net, 0.05, trackWins=True)
    b.setZeroDepth(zero)
    zeros = np.zeros(w * h, np.uint16)
    drawn = 0
    for f in (1, 2, 3):
        for v, t in enumerate(paths):
            b.setModelViewProjection(v, t.mvps[f])
        b.launch()
        assert b.check()
        res = b.resultsAll(unpack=True)
        for v, (t, o) in enumerate(zip(paths, orcs)):
            s = b.selection(v)
            if zero:
                o.write_depth(zeros)
            o.clear()
            o.set_mvp(t.mvps[f])
            for i in np.nonzero(s["selected"])[0]:
                o.rasterize(scene.packed[i], scene.packets[i], scene.ref[i, :4], scene.ref[i, 4:],
                            bool(s["features"][i, 1]))
            drawn += int(s["selected"].sum())
            r = views[v]["raster"]
            assert not mismatch_report(f"launch {f} view {v} depth", r.readDepthRaw(), o.depth())
            assert not mismatch_report(f"launch {f} view {v} hiz", r.readHiZ(), o.hiz())
            ovis, onc = o.query(pmin, pmax)
            assert np.array_equal(res[v][0].astype(np.uint8), ovis), (f, v)
            assert np.array_equal(res[v][1].astype(np.uint8), onc), (f, v)
    assert drawn > 3 * 64
    b.close()
    net.close()
    for v in views:
        v["raster"].close()
