"""CPU tests of the learned-selection host logic: training targets, the eye
recovered from a view matrix, the cull accounting, the seeded camera tracks
and the selection baselines without the network."""
import numpy as np
import pytest

from rasterizer_gb300 import learned as L
from rasterizer_gb300 import scenes
from oracle import mlp as ref


def test_targets():
    lab = dict(wins=np.array([0, 5, 10, 0, 3, 3, 100]), wh=np.full(7, 100), group=np.array([0, 0, 0, 1, 1, 1, 1]))
    t = L.targets(lab, "log_view")
    assert np.allclose(t, np.log2(1 + lab["wins"]) / np.log2(101))
    r = L.targets(lab, "rank")
    assert r[2] == 1.0 and r[6] == 1.0 and r[0] == 0 and r[3] == 0
    assert 0 < r[1] < 1
    m = L.targets(lab, "log_max")
    assert np.all(m <= 1) and m[0] == 0


def test_eye_of_view_matrix():
    mvps, eyes = scenes.camera_path(20, seed=3)
    for m, e in zip(mvps, eyes):
        got = L._eye_of(np.asarray(m, np.float64).reshape(4, 4))
        assert np.allclose(got, e[:3], atol=2e-3 * max(1.0, np.abs(e[:3]).max()))


def test_cull_stats():
    st = L.CullStats()
    full = dict(culled=np.array([1, 1, 1, 0, 0], bool), visible_empty=np.array([1, 1, 0, 1, 1], bool),
                candidate=np.array([1, 1, 0], bool))
    st.add(np.array([1, 0, 1, 0, 0], bool), full, np.array([1, 0, 0], bool), np.array([10, 20, 30]))
    assert (st.full, st.kept, st.false, st.full_all, st.kept_all) == (2, 1, 0, 3, 2)
    assert (st.candidates, st.drawn, st.quads_candidates, st.quads_drawn) == (2, 1, 30, 10)
    assert st.retained == 0.5


def test_reference_gradient_matches_finite_differences():
    """The CPU reference's gradient (bf16 roundings as identity) against
    central differences of its own forward with the roundings removed."""
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, ref.PARAMS).astype(np.float32)
    x = rng.uniform(0, 1, (40, 16)).astype(np.float32)
    t = rng.uniform(0, 1, 40).astype(np.float32)
    saved = ref.bf16
    ref.bf16 = lambda a: np.asarray(a, np.float32)
    try:
        _, g = ref.gradients(p, x, t)
        for i in rng.choice(ref.PARAMS, 25, replace=False):
            h = 1e-3
            pp, pm = p.astype(np.float64).copy(), p.astype(np.float64).copy()
            pp[i] += h
            pm[i] -= h
            fp = np.mean((ref.forward(pp.astype(np.float32), x) - t) ** 2)
            fm = np.mean((ref.forward(pm.astype(np.float32), x) - t) ** 2)
            assert abs((fp - fm) / (2 * h) - g[i]) < 2e-3 * max(1.0, abs(g[i])), i
    finally:
        ref.bf16 = saved


def test_group_distribution_and_listwise_reference():
    lab = dict(wins=np.array([0, 5, 10, 0, 3, 3, 100, 4, 4]), culls=np.array([0, 2, 2, 0, 0, 0, 0, 0, 0]),
               wh=np.full(9, 100), group=np.array([0, 0, 0, 1, 1, 1, 1, 2, 2]))
    d = L.group_distribution(lab)
    assert np.allclose(d[:3], [0, 0.5, 0.5]) and np.allclose(d[3:7], np.array([0, 3, 3, 100]) / 106)
    assert np.allclose(d[7:], [0.5, 0.5])
    # listwise reference gradient against central differences (bf16 roundings off)
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.3, ref.PARAMS).astype(np.float32)
    x = rng.uniform(0, 1, (30, 16)).astype(np.float32)
    gs = np.array([0, 7, 19, 30])
    t = rng.uniform(0, 1, 30)
    for a, b in zip(gs[:-1], gs[1:]):
        t[a:b] /= t[a:b].sum()
    saved = ref.bf16
    ref.bf16 = lambda a: np.asarray(a, np.float32)
    try:
        _, g = ref.listwise_gradients(p, x, t, gs)
        for i in rng.choice(ref.PARAMS, 20, replace=False):
            h = 1e-3
            pp, pm = p.astype(np.float64).copy(), p.astype(np.float64).copy()
            pp[i] += h
            pm[i] -= h
            fp, _ = ref.listwise_gradients(pp.astype(np.float32), x, t, gs)
            fm, _ = ref.listwise_gradients(pm.astype(np.float32), x, t, gs)
            assert abs((fp - fm) / (2 * h) - g[i]) < 2e-3 * max(1.0, abs(g[i])), i
    finally:
        ref.bf16 = saved


def test_tracks_are_seeded_and_shaped():
    """Street and multi-view tracks: the same seeds give the same matrices,
    other seeds other ones; every view's matrix is finite, the eye stays at
    street level on the street paths, and the multi-view workload has its 256
    views (64 cascades, 96 cube faces, 96 probes) with query ranges that
    stay inside the pool."""
    a = L.street_tracks(3, 5, seed0=7000, n_occluders=10, queries=100)
    b = L.street_tracks(3, 5, seed0=7000, n_occluders=10, queries=100)
    c = L.street_tracks(3, 5, seed0=7100, n_occluders=10, queries=100)
    for x, y in zip(a, b):
        assert np.array_equal(x.mvps, y.mvps)
    assert not np.array_equal(a[0].mvps, c[0].mvps)
    for t in a:
        assert t.mvps.shape == (5, 16) and np.isfinite(t.mvps).all()
        eyes = np.stack([L._eye_of(np.asarray(m, np.float64).reshape(4, 4)) for m in t.mvps])
        assert (eyes[:, 1] > 0.5).all() and (eyes[:, 1] < 4.0).all()   # street level
        assert np.linalg.norm(eyes[-1] - eyes[0]) > 0                  # the camera moves
    rng = np.random.default_rng(0)
    centers = np.concatenate([rng.uniform(-300, 300, (386, 1)), rng.uniform(0, 40, (386, 1)),
                              rng.uniform(-300, 300, (386, 1)), np.ones((386, 1))], axis=1).astype(np.float32)
    quads = rng.integers(8, 2000, 386)
    mv = L.multiview_tracks(centers, quads, 100_000, frames=2, seed=3)
    kinds = [t.kind for t in mv]
    assert len(mv) == 256 and kinds.count("cascade") == 64 and kinds.count("cube") == 96
    for t in mv:
        assert t.width % 8 == 0 and t.height % 8 == 0 and len(t.occluders) > 0
        assert 0 <= t.query_start and t.query_start + t.query_count <= 100_000
        assert np.isfinite(t.mvps).all()


def test_heuristic_orders():
    """The baselines without the network: nearest-first sorts by distance of
    the occluder centre to the eye (Main.cpp:185-190), area and wins by their
    values, ties in command order."""
    from rasterizer_gb300 import api, scenes
    mvp = np.asarray(scenes.view_projection((0.0, 1.7, 0.0), (0.0, 0.0, 1.0)), np.float32).reshape(1, 16)
    z = [30.0, 10.0, 20.0, 10.0]
    occ = [api.Occluder(np.zeros(32, np.uint32), 4, np.zeros(4, np.float32), np.ones(4, np.float32),
                        np.zeros(4, np.float32), np.ones(4, np.float32), np.array([0, 1.7, d, 1], np.float32))
           for d in z]
    t = L.Track(640, 360, np.arange(4), mvp)
    feats = np.zeros((4, 16), np.float32)
    feats[:, 3] = [0.1, 0.3, 0.3, 0.2]
    full = {"features": feats, "wins": np.array([5, 9, 1, 9], np.uint32)}
    assert list(L.heuristic_order("nearest", t, occ, full, 0)) == [1, 3, 2, 0]
    assert list(L.heuristic_order("area", t, occ, full, 0)) == [1, 2, 3, 0]
    assert list(L.heuristic_order("wins", t, occ, full, 0)) == [1, 3, 0, 2]
    with pytest.raises(ValueError):
        L.heuristic_order("random", t, occ, full, 0)
