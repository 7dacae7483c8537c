"""The CPU oracle and the library's host bake against fixtures produced by the
reference itself (tests/golden/make_golden.py).  Runs on any host; on the
aarch64 GPU host this is what pins the portable oracle to the x86 reference."""
import json
import os

import numpy as np
import pytest

from oracle.bindings import Oracle
from rasterizer_gb300 import api, scenes

from helpers import boxes_occluders, city_occluders, to_baked
from golden.make_golden import CITY_FRAMES, digest, scene_digest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))
SMALL = np.load(os.path.join(HERE, "golden", "golden_small.npz"))


def test_coverage_tables():
    """The oracle's table (built on this host as Rasterizer.cpp:547-604 does)
    and the library's embedded table both equal the reference's."""
    assert digest(Oracle(8, 8).table()) == GOLDEN["coverage_table"]
    assert digest(api.coverage_table()) == GOLDEN["coverage_table"]
    assert np.array_equal(api.coverage_table(), SMALL["table"])


def test_scene_generators_are_stable():
    assert scenes.boxes_scene().digest() == GOLDEN["boxes"]["mesh"]
    assert scenes.city_scene().digest() == GOLDEN["city"]["mesh"]


def test_bake_matches_reference_bake():
    """QuadDecomposition + SAH + Occluder::bake of the library, byte-identical."""
    occ = boxes_occluders()
    assert len(occ) == GOLDEN["boxes"]["occluders"]
    assert scene_digest(to_baked(occ)) == GOLDEN["boxes"]["bake"]
    occ = city_occluders()
    assert len(occ) == GOLDEN["city"]["occluders"]
    assert sum(o.quads for o in occ) == GOLDEN["city"]["quads"]
    assert scene_digest(to_baked(occ)) == GOLDEN["city"]["bake"]


def test_small_frame_raw():
    sc = to_baked(boxes_occluders())
    orc = Oracle(320, 200)
    flags = orc.frame_plain(sc, SMALL["mvp"])
    qm, qM = scenes.query_boxes(1024, seed=45)
    vis, nc = orc.query(qm, qM)
    assert np.array_equal(flags, SMALL["flags"])
    assert np.array_equal(orc.depth(), SMALL["depth"])
    assert np.array_equal(orc.hiz(), SMALL["hiz"])
    assert np.array_equal(vis, SMALL["visible"]) and np.array_equal(nc, SMALL["needsClipping"])
    assert np.array_equal(orc.read_back(), SMALL["readback"])


def test_read_back_formats_consistent():
    """The oracle's read-back values (float linDepth, float depth, packed u16)
    reproduce its readBackDepth bytes, which are pinned to the reference."""
    from helpers import read_back_consistent
    sc = to_baked(boxes_occluders())
    orc = Oracle(320, 200)
    orc.frame_plain(sc, SMALL["mvp"])
    hiz = orc.hiz()[:40 * 25].reshape(25, 40)
    cleared = np.repeat(np.repeat(hiz == 1, 8, axis=0), 8, axis=1)
    lin, depth, packed = (orc.read_back_values(k) for k in ("linear", "depth", "packed"))
    assert cleared.any() and (~cleared).any()
    assert not read_back_consistent(orc.read_back(), lin, depth, packed, cleared)
    raw = orc.depth().reshape(25, 40, 8, 8).transpose(0, 2, 1, 3).reshape(200, 320)
    assert np.array_equal(np.where(cleared, 0, raw), packed)


def _check_frame(orc, flags, vis, nc, g):
    got = {"flags": digest(flags), "depth": digest(orc.depth()), "hiz": digest(orc.hiz()),
           "visible": digest(vis), "needsClipping": digest(nc), "readback": digest(orc.read_back())}
    bad = [k for k in got if got[k] != g[k]]
    assert not bad, f"oracle differs from the reference in {bad}"


def test_boxes_frame_1080p():
    sc = to_baked(boxes_occluders())
    orc = Oracle(1920, 1080)
    flags = orc.frame_plain(sc, scenes.boxes_camera())
    mins, maxs = scenes.query_boxes(4096, seed=43)
    vis, nc = orc.query(mins, maxs)
    _check_frame(orc, flags, vis, nc, GOLDEN["boxes"]["frames"][0])


def test_city_frames():
    """Six frames of the street-level path on one persistent rasterizer
    (near-clipped occluders and stale depth included)."""
    sc = to_baked(city_occluders())
    mvps, _ = scenes.camera_path(300, seed=7)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    orc = Oracle(1920, 1080)
    assert tuple(GOLDEN["city"]["frame_indices"]) == CITY_FRAMES
    for f, g in zip(CITY_FRAMES, GOLDEN["city"]["frames"]):
        flags = orc.frame_plain(sc, mvps[f])
        vis, nc = orc.query(mins, maxs)
        _check_frame(orc, flags, vis, nc, g)
        assert g["near_clipped"] == int(((flags & 3) == 3).sum())


def test_city_bake_fixture():
    """tests/golden/city_occluders.npz holds the reference's own bake of the
    city (the occluders the benchmark's CPU arms draw, with no native library
    of this project involved): same digest as the reference's bake, and the
    library's host bake gives the same bytes."""
    from oracle.bindings import load_baked_scene
    sc = load_baked_scene(os.path.join(HERE, "golden", "city_occluders.npz"))
    assert scene_digest(sc) == GOLDEN["city"]["bake"]
    lib = to_baked(city_occluders())
    assert len(lib) == len(sc)
    assert all(np.array_equal(a, b) for a, b in zip(lib.packed, sc.packed))


def test_gated_frame_loop_draws_front_to_back():
    """The gated, distance-sorted frame loop of Main.cpp:181-206 in the oracle:
    the drawing order ascends in squared distance, and every occluder it
    rasterises was visible against the buffer drawn so far, so the result
    never culls a box that the plain all-occluder frame shows."""
    sc = to_baked(city_occluders())
    mvps, eyes = scenes.camera_path(300, seed=7)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    orc, full = Oracle(1920, 1080), Oracle(1920, 1080)
    for f in (0, 150):
        orc.write_depth(np.zeros(1920 * 1080, np.uint16))
        order, flags = orc.frame_gated(sc, mvps[f], eyes[f])
        d = ((sc.centers[order, :3].astype(np.float64) - eyes[f][:3]) ** 2).sum(axis=1)
        assert np.all(np.diff(d) >= -1e-3 * np.maximum(d[1:], 1.0))
        assert sorted(order.tolist()) == list(range(len(sc)))
        full.write_depth(np.zeros(1920 * 1080, np.uint16))
        fflags = full.frame_plain(sc, mvps[f])
        assert (flags & 1).sum() <= (fflags & 1).sum()  # gating skips occluders already hidden
        vis, _ = orc.query(mins, maxs)
        fvis, _ = full.query(mins, maxs)
        assert not (fvis.astype(bool) & ~vis.astype(bool)).any()
