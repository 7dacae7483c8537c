"""Learned occluder selection: labels from the exact GPU rasteriser, training
on the device, and evaluation against the plain all-occluder frame.

The reference's frame loop draws every occluder whose bounds pass
queryVisibility, nearest first (SoftwareRasterizer/Main.cpp:184-206).  The
selector replaces that ordering: an MLP scores each occluder of a view from
screen-space and depth features of its bounds and from the pixels it won in
the previous frame, and each view draws only the top fraction of its
candidates.  A subset of the occluders can only leave depth farther (max-merge
of fewer fragments), so a selected frame culls a subset of what the full frame
culls; `evaluate` counts both the culls kept and any false culls.

Labels: for every candidate occluder of a frame, its pixel wins in the full
frame (the pixels whose final depth it produced), as log2(1 + wins) /
log2(1 + width * height).  Features 13 and 14 of a frame are the wins of the
previous frame of the same view, so labels are collected along tracks of
moving views.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from . import api

GATED = 2  # OCC_GATED: the device tests the bounds, as the plain loop's queryVisibility


@dataclass
class Track:
    """One view followed over frames."""
    width: int
    height: int
    occluders: np.ndarray  # indices into the scene's occluder list, in drawing order
    mvps: np.ndarray       # (frames, 16) float32
    query_start: int = 0
    query_count: int = 0
    kind: str = "view"


def wins_target(wins: np.ndarray, width: int, height: int) -> np.ndarray:
    return (np.log2(1.0 + wins.astype(np.float64)) / math.log2(1.0 + width * height)).astype(np.float32)


def _views(ctx, occluders, tracks, mins=None, maxs=None, frame=0, subsets=None):
    views = []
    for i, t in enumerate(tracks):
        r = api.Rasterizer(ctx, t.width, t.height)
        ids = t.occluders if subsets is None else subsets[i]
        sel = [occluders[k] for k in ids]
        v = dict(raster=r, mvp=t.mvps[frame], clear=True, occluders=sel, flags=np.full(len(sel), GATED, np.uint8))
        if mins is not None and t.query_count:
            v["mins"] = mins[t.query_start:t.query_start + t.query_count]
            v["maxs"] = maxs[t.query_start:t.query_start + t.query_count]
        views.append(v)
    return views


def _launch(b: api.PreparedBatch, tracks, f: int) -> None:
    for i, t in enumerate(tracks):
        b.setModelViewProjection(i, t.mvps[f])
    b.launch()
    if not b.check():  # scratch grown: re-run the previous frame (its wins feed this one), then this one
        if f > 0:
            for i, t in enumerate(tracks):
                b.setModelViewProjection(i, t.mvps[f - 1])
            b.launch()
            b.check()
            for i, t in enumerate(tracks):
                b.setModelViewProjection(i, t.mvps[f])
        b.launch()
        if not b.check():
            raise api.OccError("batch scratch still too small after growing")


def collect_labels(ctx, occluders, tracks: list[Track], group: int = 64, selector=None,
                   fraction: float = 0.2, mins=None, maxs=None) -> dict:
    """Runs the tracks with every occluder drawn and win counting on.  For
    every candidate occluder of every frame: features (N, 16), wins (N,),
    the view's pixel count, and a group id per (view, frame); with query
    boxes (`mins`, `maxs`, each track's range), also its cull credits (N,):
    samples of the boxes culled by depth whose pixels it owns.  With a
    `selector`, the features come from the same tracks run under that
    selector at `fraction` (its own previous-frame wins and draw flags, as
    it will see them), the wins from the full frames.  Tracks of a group of
    `group` views must have equal frame counts."""
    X, wins, wh, gid, culls = [], [], [], [], []
    g = 0
    for g0 in range(0, len(tracks), group):
        ts = tracks[g0:g0 + group]
        frames = len(ts[0].mvps)
        assert all(len(t.mvps) == frames for t in ts)
        views = _views(ctx, occluders, ts, mins, maxs)
        b = api.PreparedBatch(ctx, views)
        b.setSelection(None, trackWins=True)
        if mins is not None:
            b.setCullLabels(True)
        batches = [b]
        if selector is not None:
            sviews = _views(ctx, occluders, ts)
            sb = api.PreparedBatch(ctx, sviews)
            sb.setSelection(selector, fraction, trackWins=True)
            batches.append(sb)
            views += sviews
        for f in range(frames):
            for x in batches:
                _launch(x, ts, f)
            for i, t in enumerate(ts):
                s = b.selection(i)
                c = s["candidate"]
                feats = s["features"] if selector is None else batches[1].selection(i)["features"]
                n = int(c.sum())
                X.append(feats[c])
                wins.append(s["wins"][c])
                if mins is not None:
                    culls.append(b.cullLabels(i)[c])
                wh.append(np.full(n, t.width * t.height, np.int64))
                gid.append(np.full(n, g, np.int64))
                g += 1
        for x in batches:
            x.close()
        for v in views:
            v["raster"].close()
    out = dict(X=np.concatenate(X), wins=np.concatenate(wins), wh=np.concatenate(wh), group=np.concatenate(gid))
    if mins is not None:
        out["culls"] = np.concatenate(culls)
    return out


def concat_labels(parts: list[dict]) -> dict:
    out, off = [], 0
    for p in parts:
        q = dict(p)
        q["group"] = p["group"] + off
        off = int(q["group"].max()) + 1 if len(q["group"]) else off
        out.append(q)
    return {k: np.concatenate([q[k] for q in out]) for k in out[0]}


def targets(labels: dict, kind: str = "log_view") -> np.ndarray:
    """Regression targets.  "culls": log2(1 + cull credits) / 21; "mix": the
    mean of "culls" and "log_view"; "log_view": log2(1 + wins) /
    log2(1 + pixels of the view); "log_max": log2(1 + wins) / log2(1 + the
    largest wins of the same view and frame); "rank": the occluder's rank among
    the candidates of its view and frame, 1 for the most wins, 0 for none."""
    w = labels["wins"].astype(np.float64)
    if kind == "log_view":
        return (np.log2(1.0 + w) / np.log2(1.0 + labels["wh"])).astype(np.float32)
    if kind == "culls":  # cull credits: 16 samples per culled box, up to 100k boxes per view
        return (np.log2(1.0 + labels["culls"].astype(np.float64)) / 21.0).astype(np.float32)
    if kind == "mix":
        return (0.5 * targets(labels, "log_view") + 0.5 * targets(labels, "culls")).astype(np.float32)
    g = labels["group"]
    ng = int(g.max()) + 1 if len(g) else 0
    if kind == "log_max":
        mx = np.zeros(ng)
        np.maximum.at(mx, g, w)
        return (np.log2(1.0 + w) / np.log2(2.0 + mx[g])).astype(np.float32)
    if kind == "rank":
        order = np.lexsort((w, g))  # by group, then ascending wins
        gs = g[order]
        start = np.searchsorted(gs, np.arange(ng))
        cnt = np.bincount(g, minlength=ng)
        pos = np.arange(len(order)) - start[gs]
        r = np.zeros(len(w))
        r[order] = (pos + 1) / cnt[gs]
        r[w == 0] = 0.0
        return r.astype(np.float32)
    raise ValueError(kind)


def train(selector: api.OccluderSelector, X: np.ndarray, y: np.ndarray, steps: int = 3000, batch: int = 4096,
          lr: float = 2e-3, seed: int = 0, drop_prev: float = 0.3, positive_share: float = 0.0,
          weights: np.ndarray | None = None, log_every: int = 0):
    """Adam on mean squared error, minibatches drawn with replacement (in
    proportion to `weights` if given; with `positive_share` > 0, that share of
    each batch from rows with wins).  In a
    `drop_prev` share of the rows the previous-frame features are zeroed:
    occluders that were not drawn in the previous frame have no wins to show,
    so the ranking must also work from geometry alone.  Returns the loss history."""
    rng = np.random.default_rng(seed)
    pos = np.nonzero(y > 0)[0]
    cdf = None
    if weights is not None:
        cdf = np.cumsum(np.asarray(weights, np.float64))
        cdf /= cdf[-1]
    losses = []
    for it in range(steps):
        if cdf is None:
            idx = rng.integers(0, len(X), batch)
        else:
            idx = np.minimum(np.searchsorted(cdf, rng.random(batch), side="right"), len(X) - 1)
        if positive_share > 0 and len(pos):
            npos = int(batch * positive_share)
            idx[:npos] = pos[rng.integers(0, len(pos), npos)]
        xb = X[idx].copy()
        if drop_prev > 0:
            m = rng.random(batch) < drop_prev
            xb[m, 13] = 0.0
            xb[m, 14] = 0.0
        step_lr = lr * (0.5 * (1.0 + math.cos(math.pi * it / steps)) * 0.9 + 0.1)
        losses.append(selector.trainStep(xb, y[idx], lr=step_lr))
        if log_every and (it + 1) % log_every == 0:
            print(f"  step {it + 1}: loss {np.mean(losses[-log_every:]):.5f}", flush=True)
    return np.asarray(losses)


def group_distribution(labels: dict, key: str = "culls") -> np.ndarray:
    """Per row, its share of the group's total `key` (cull credits by
    default); groups with no credit at all fall back to pixel wins."""
    g = labels["group"]
    ng = int(g.max()) + 1 if len(g) else 0
    out = np.zeros(len(g))
    for k in (key, "wins"):
        v = labels[k].astype(np.float64)
        tot = np.zeros(ng)
        np.add.at(tot, g, v)
        use = (out == 0) & (tot[g] > 0)
        if k != key:
            have = np.zeros(ng, bool)
            np.logical_or.at(have, g, out > 0)
            use &= ~have[g]
        out[use] = v[use] / tot[g][use]
    return out.astype(np.float32)


def train_listwise(selector: api.OccluderSelector, labels: dict, dist: np.ndarray, source: np.ndarray,
                   steps: int = 6000, groups_per_step: int = 256, lr: float = 2e-3, seed: int = 0,
                   drop_prev: float = 0.3, log_every: int = 0):
    """Adam on the listwise loss: each step takes `groups_per_step` (view,
    frame) groups, half from street rows and half from multi-view rows
    (`source` 0/1 per row), and fits the softmax of each group's scores to the
    group's target distribution `dist`.  Returns the loss history."""
    rng = np.random.default_rng(seed)
    g = labels["group"]
    ng = int(g.max()) + 1
    starts = np.searchsorted(g, np.arange(ng + 1))
    sizes = starts[1:] - starts[:-1]
    gsrc = source[starts[:-1]]
    tot = np.zeros(ng)
    np.add.at(tot, g, dist)
    ok = (sizes > 1) & (tot > 0)
    pools = [np.nonzero(ok & (gsrc == k))[0] for k in (0, 1)]
    pools = [p for p in pools if len(p)]
    X = labels["X"]
    losses = []
    for it in range(steps):
        per = groups_per_step // len(pools)
        gs = np.concatenate([p[rng.integers(0, len(p), per)] for p in pools])
        idx = np.concatenate([np.arange(starts[k], starts[k + 1]) for k in gs])
        gstart = np.concatenate([[0], np.cumsum(sizes[gs])]).astype(np.uint32)
        xb = X[idx].copy()
        if drop_prev > 0:
            m = rng.random(len(idx)) < drop_prev
            xb[m, 13] = 0.0
            xb[m, 14] = 0.0
        step_lr = lr * (0.5 * (1.0 + math.cos(math.pi * it / steps)) * 0.9 + 0.1)
        losses.append(selector.trainStepListwise(xb, dist[idx], gstart, lr=step_lr))
        if log_every and (it + 1) % log_every == 0:
            print(f"  step {it + 1}: loss {np.mean(losses[-log_every:]):.5f}", flush=True)
    return np.asarray(losses)


@dataclass
class CullStats:
    """Culls of the selected frames against the full frames.  An occlusion
    cull is a box that is visible in an empty buffer (inside the frustum) but
    culled by the full frame; boxes outside the frustum are culled by any
    subset and are counted apart."""
    full: int = 0        # occlusion culls of the full frames
    kept: int = 0        # of those, culled by the selected frames too
    false: int = 0       # culled by a selected frame but visible in the full frame
    full_all: int = 0    # all culls of the full frames (frustum included)
    kept_all: int = 0
    candidates: int = 0  # candidate occluders over all views and frames
    drawn: int = 0       # occluders drawn
    quads_candidates: int = 0
    quads_drawn: int = 0

    @property
    def retained(self) -> float:
        return self.kept / max(self.full, 1)

    def add(self, culled: np.ndarray, full_frame: dict, drawn: np.ndarray, quads: np.ndarray) -> None:
        fu = full_frame["culled"]
        occ = fu & full_frame["visible_empty"]
        cand = full_frame["candidate"]
        self.full += int(occ.sum())
        self.kept += int((culled & occ).sum())
        self.false += int((culled & ~fu).sum())
        self.full_all += int(fu.sum())
        self.kept_all += int((culled & fu).sum())
        self.candidates += int(cand.sum())
        self.drawn += int(drawn.sum())
        self.quads_candidates += int(quads[cand].sum())
        self.quads_drawn += int(quads[drawn].sum())

    def add_culls(self, culled: np.ndarray, full_frame: dict) -> None:
        """Culls only (no selection statistics): `culled` against the full frame."""
        fu = full_frame["culled"]
        occ = fu & full_frame["visible_empty"]
        self.full += int(occ.sum())
        self.kept += int((culled & occ).sum())
        self.false += int((culled & ~fu).sum())
        self.full_all += int(fu.sum())
        self.kept_all += int((culled & fu).sum())

    def as_culls_dict(self) -> dict:
        return dict(occlusion_culls_full=self.full, occlusion_culls_kept=self.kept,
                    culls_retained=round(self.retained, 5), false_culls=self.false,
                    all_culls_full=self.full_all, all_culls_retained=round(self.kept_all / max(self.full_all, 1), 5))

    def as_dict(self) -> dict:
        return dict(occlusion_culls_full=self.full, occlusion_culls_kept=self.kept,
                    culls_retained=round(self.retained, 5), false_culls=self.false,
                    all_culls_full=self.full_all, all_culls_retained=round(self.kept_all / max(self.full_all, 1), 5),
                    drawn_share_of_candidates=round(self.drawn / max(self.candidates, 1), 4),
                    quads_drawn_share=round(self.quads_drawn / max(self.quads_candidates, 1), 4))


def _culled(b: api.PreparedBatch, i: int) -> np.ndarray:
    vis, _ = b.results(i)
    return ~vis


def run_full(ctx, occluders, tracks, mins, maxs):
    """The plain all-occluder frames and the same views with no occluder,
    depth zeroed per frame (each frame stands alone).  Returns per frame and
    view: culled boxes, boxes visible in the empty buffer, candidate flags,
    features and pixel wins."""
    views = _views(ctx, occluders, tracks, mins, maxs)
    b = api.PreparedBatch(ctx, views)
    b.setSelection(None, trackWins=True)
    b.setZeroDepth(True)
    empty_views = _views(ctx, occluders, tracks, mins, maxs, subsets=[[] for _ in tracks])
    e = api.PreparedBatch(ctx, empty_views)
    e.setZeroDepth(True)
    out = []
    for f in range(len(tracks[0].mvps)):
        _launch(b, tracks, f)
        _launch(e, tracks, f)
        row = []
        for i in range(len(tracks)):
            s = b.selection(i)
            row.append(dict(culled=_culled(b, i), visible_empty=~_culled(e, i), candidate=s["candidate"],
                            features=s["features"], wins=s["wins"]))
        out.append(row)
    for x in (b, e):
        x.close()
    for v in views + empty_views:
        v["raster"].close()
    return out


def _quads(occluders, ids):
    return np.array([occluders[k].quads for k in ids], np.int64)


def evaluate_learned(ctx, occluders, tracks, mins, maxs, selector, fraction: float, full,
                     use_prev: bool = True, second_pass: bool = False) -> CullStats:
    """The selector's frames (top `fraction` of each view's candidates, the
    previous-frame wins of the selected frames feeding the next unless
    `use_prev` is off; with `second_pass`, plus the other candidates still
    visible after the top-K pass) against `full`."""
    views = _views(ctx, occluders, tracks, mins, maxs)
    b = api.PreparedBatch(ctx, views)
    b.setSelection(selector, fraction, trackWins=use_prev)
    if second_pass:
        b.setSecondPass(True)
    b.setZeroDepth(True)
    st = CullStats()
    qs = [_quads(occluders, t.occluders) for t in tracks]
    for f in range(len(tracks[0].mvps)):
        _launch(b, tracks, f)
        for i in range(len(tracks)):
            s = b.selection(i)
            st.add(_culled(b, i), full[f][i], s["selected"], qs[i])
    b.close()
    for v in views:
        v["raster"].close()
    return st


def heuristic_order(kind: str, track: Track, occluders, full_frame: dict, frame: int):
    """Candidate ranking without the network: "nearest" = distance of the
    occluder's centre to the eye, as Main.cpp:185-190 sorts; "area" = largest
    screen rectangle first; "wins" = the full frame's own pixel wins (an upper
    reference for the label, not available before drawing)."""
    features = full_frame["features"]
    if kind == "nearest":
        m = np.asarray(track.mvps[frame], np.float64).reshape(4, 4)
        eye = _eye_of(m)
        c = np.stack([occluders[k].center[:3] for k in track.occluders]).astype(np.float64)
        return np.argsort(((c - eye) ** 2).sum(axis=1), kind="stable")
    if kind == "area":
        return np.argsort(-features[:, 3], kind="stable")
    if kind == "wins":
        return np.argsort(-full_frame["wins"].astype(np.int64), kind="stable")
    raise ValueError(kind)


def _eye_of(mvp: np.ndarray) -> np.ndarray:
    """Camera position of a row-vector view-projection matrix: the point that
    maps to clip x = y = w = 0 (w = 0 on the camera plane through the eye)."""
    a = mvp[:3, [0, 1, 3]].T
    b = -mvp[3, [0, 1, 3]]
    return np.linalg.solve(a, b)


def evaluate_heuristic(ctx, occluders, tracks, mins, maxs, kind: str, fraction: float, full) -> CullStats:
    """Top `fraction` of each view's candidates by a fixed ranking, drawn by
    the same rasteriser (one batch per frame), against `full`."""
    st = CullStats()
    rasters = [api.Rasterizer(ctx, t.width, t.height) for t in tracks]
    qs = [_quads(occluders, t.occluders) for t in tracks]
    for f in range(len(tracks[0].mvps)):
        subsets, chosen_masks = [], []
        for i, t in enumerate(tracks):
            cand = full[f][i]["candidate"]
            n = int(cand.sum())
            k = min(max(int(math.ceil(np.float32(fraction) * np.float32(n))), 1), n) if n else 0
            order = heuristic_order(kind, t, occluders, full[f][i], f)
            order = order[cand[order]][:k]
            mask = np.zeros(len(t.occluders), bool)
            mask[order] = True
            chosen_masks.append(mask)
            subsets.append(np.asarray(t.occluders)[mask])
        views = []
        for i, t in enumerate(tracks):
            r = rasters[i]
            r.writeDepthRaw(np.zeros(t.width * t.height, np.uint16))
            sel = [occluders[k] for k in subsets[i]]
            v = dict(raster=r, mvp=t.mvps[f], clear=True, occluders=sel, flags=np.full(len(sel), GATED, np.uint8))
            if t.query_count:
                v["mins"] = mins[t.query_start:t.query_start + t.query_count]
                v["maxs"] = maxs[t.query_start:t.query_start + t.query_count]
            views.append(v)
        res = api.execute_batch(ctx, views)
        for i in range(len(tracks)):
            st.add(~res[i][0], full[f][i], chosen_masks[i], qs[i])
    for r in rasters:
        r.close()
    return st


def street_tracks(n: int, frames: int, seed0: int, width: int = 1920, height: int = 1080, n_occluders: int = 0,
                  queries: int = 0):
    """`n` street-level camera paths through the city (seeds seed0..seed0+n-1)."""
    from . import scenes
    out = []
    for k in range(n):
        mvps, _ = scenes.camera_path(frames, seed=seed0 + k, width=width, height_px=height)
        out.append(Track(width, height, np.arange(n_occluders), mvps, 0, queries, "street"))
    return out


def multiview_tracks(centers, quads, n_query_pool: int, frames: int, seed: int, speed: float = 0.6):
    """The 256 views of the multi-view workload (seeded), each drifting over `frames` frames."""
    from . import scenes
    specs = scenes.multiview_workload(centers, quads, n_query_pool, seed=seed)
    return [Track(s.width, s.height, s.occluders, scenes.view_track(s, frames, seed * 1000 + j, speed),
                  s.query_start, s.query_count, s.kind) for j, s in enumerate(specs)]


def large_tracks(centers, quads, n_query_pool: int, frames: int, seed: int, grid: int = 128, speed: float = 0.6):
    """The large combined workload as tracks: the 3840x2160 main view (every
    occluder, the whole query pool) first, then its 63 auxiliary views drifting."""
    from . import scenes
    mvps, aux = scenes.large_workload(centers, quads, n_query_pool, seed=seed, frames=frames, grid=grid)
    main = Track(3840, 2160, np.arange(len(centers)), mvps, 0, n_query_pool, "main")
    return [main] + [Track(s.width, s.height, s.occluders, scenes.view_track(s, frames, seed * 1000 + j, speed),
                           s.query_start, s.query_count, s.kind) for j, s in enumerate(aux)]


@dataclass
class Recipe:
    """Training set-up: seeded street paths and multi-view workloads
    (off-policy round), then on-policy rounds whose features come from the
    network being trained (at the listed fractions)."""
    street_paths: int = 40
    street_frames: int = 250
    multiview_seeds: tuple = (101, 102, 103, 104, 105, 106, 107, 108)
    multiview_frames: int = 8
    rounds: tuple = ((0.15, 20, 120, (201, 202, 203, 204)), (0.3, 20, 120, (301, 302, 303, 304)))
    steps0: int = 6000
    steps: int = 6000
    batch: int = 4096          # rows per step (mean squared error)
    groups_per_step: int = 256  # (view, frame) groups per step (listwise)
    lr: float = 2e-3
    objective: str = "listwise"  # or "mse" on `target`
    target: str = "culls"        # listwise: distribution of cull credits; mse: a `targets` kind
    seed: int = 0

    def poses(self) -> int:
        n = self.street_paths * self.street_frames + len(self.multiview_seeds) * 256 * self.multiview_frames
        for _, sp, sf, ms in self.rounds:
            n += sp * sf + len(ms) * 256 * self.multiview_frames
        return n


def _recipe_data(ctx, occluders, centers, quads, n_query_pool, street_paths, street_frames, seed0, mseeds, mframes,
                 selector=None, fraction=0.2, mins=None, maxs=None):
    nq = n_query_pool if mins is not None else 0
    parts = [collect_labels(ctx, occluders, street_tracks(street_paths, street_frames, seed0,
                                                          n_occluders=len(occluders), queries=nq),
                            group=40, selector=selector, fraction=fraction, mins=mins, maxs=maxs)]
    n_street = len(parts[0]["wins"])
    for sd in mseeds:
        parts.append(collect_labels(ctx, occluders, multiview_tracks(centers, quads, n_query_pool, mframes, sd),
                                    group=64, selector=selector, fraction=fraction, mins=mins, maxs=maxs))
    lab = concat_labels(parts)
    src = np.zeros(len(lab["wins"]), np.int8)
    src[n_street:] = 1
    return lab, src


def train_selector(ctx, occluders, n_query_pool: int = 100_000, recipe: Recipe | None = None, log=print,
                   mins=None, maxs=None):
    """Trains a selector for the city scene's occluders end to end on the GPU:
    labels from the rasteriser, forward/backward/Adam on the device.  Street
    and multi-view data are sampled half and half.  With the query pool
    (`mins`, `maxs`) the labels are cull credits, else pixel wins.  The
    default objective is listwise: per view and frame, the softmax of the
    scores is fitted to the distribution of the labels, which is what a top-K
    choice needs.  Returns (selector, report)."""
    rc = recipe or Recipe()
    centers = np.stack([o.center for o in occluders])
    quads = np.array([o.quads for o in occluders])
    t = Timer()
    lab, src = _recipe_data(ctx, occluders, centers, quads, n_query_pool, rc.street_paths, rc.street_frames, 1000,
                            rc.multiview_seeds, rc.multiview_frames, mins=mins, maxs=maxs)
    labs, srcs = [lab], [src]
    report = dict(poses=rc.poses(), label_seconds=t.lap())

    def weights(s):
        return np.where(s == 0, 0.5 / max(int((s == 0).sum()), 1), 0.5 / max(int((s == 1).sum()), 1))

    def fit(net, lab, src, steps, seed, drop):
        if rc.objective == "listwise":
            dist = group_distribution(lab, rc.target if rc.target in lab else "wins")
            return train_listwise(net, lab, dist, src, steps=steps, groups_per_step=rc.groups_per_step, lr=rc.lr,
                                  seed=seed, drop_prev=drop)
        return train(net, lab["X"], targets(lab, rc.target), steps=steps, batch=rc.batch, lr=rc.lr, seed=seed,
                     drop_prev=drop, weights=weights(src))

    net = api.OccluderSelector(ctx, seed=rc.seed)
    losses = fit(net, lab, src, rc.steps0, rc.seed, 0.3)
    report["rounds"] = [dict(rows=int(len(lab["wins"])), final_loss=float(losses[-200:].mean()),
                             train_seconds=t.lap())]
    for k, (frac, sp, sf, ms) in enumerate(rc.rounds):
        lab, src = _recipe_data(ctx, occluders, centers, quads, n_query_pool, sp, sf, 2000 + 1000 * k, ms,
                                rc.multiview_frames, selector=net, fraction=frac, mins=mins, maxs=maxs)
        labs.append(lab)
        srcs.append(src)
        allab = concat_labels(labs)
        alsrc = np.concatenate(srcs)
        label_s = t.lap()
        nxt = api.OccluderSelector(ctx, seed=rc.seed + k + 1)
        losses = fit(nxt, allab, alsrc, rc.steps, rc.seed + k + 1, 0.15)
        net.close()
        net = nxt
        report["rounds"].append(dict(rows=int(len(allab["wins"])), on_policy_fraction=frac, label_seconds=label_s,
                                     final_loss=float(losses[-200:].mean()), train_seconds=t.lap()))
        if log:
            log(f"on-policy round {k + 1}: {report['rounds'][-1]}")
    return net, report


class Timer:
    def __init__(self):
        self.t = time.perf_counter()

    def lap(self) -> float:
        n = time.perf_counter()
        d, self.t = n - self.t, n
        return d
