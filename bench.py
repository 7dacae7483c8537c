"""Benchmark: views/s of the batched + learned path on one GB300, next to the
plain path and the reference's CPU algorithm.

Scene: a seeded 64x64 grid of extruded buildings, 259,534 triangles baked
into 386 occluders (129,768 quads); 100,000 query boxes (lognormal extents)
per view.

  value    (headline) batched + learned: 64 street-level 1920x1080 views
           (seeded camera paths, each view moving every step) per graph
           launch; each view draws the selector's top K of its candidate
           occluders (K = the smallest fraction keeping >= 99% of the
           occlusion culls on held-out validation views) in the zero-depth
           clear and answers its queries.  Device time per launch (CUDA
           events on the library's stream); the selector is trained first,
           on the GPU, outside the timed region.  `culls`: culls kept and
           false culls of the timed launches themselves against full frames
           at the same poses (and on held-out paths);
  e2e      the same launches through the public API with host data: 64
           matrices from the host, launch, every view's result bits back;
           e2e_dynamic_boxes: plus every view's boxes from the host each step;
  plain_single_view  the plain all-occluder loop, one 1080p view per launch
           along a 300-frame path (L2 flushed between frames), with its
           per-kernel times, roofline and end-to-end figure;
  batched  the 256-view mixed-resolution workload, one launch vs one launch per view;
  learned  training report, K sweep against the nearest-first ordering, the
           256-view workload with learned selection, and the large workload
           (2M-triangle city, 4K + 63 views) with its bake timings (host and
           GPU SAH, GPU Occluder::bake, baked-file load);
  cpu_baseline  the CPU oracle (portable restatement of the reference) on
           one host core, the reference's own frame loop (Main.cpp:181-206)
           on its own bake, on a bounded sample of the headline's views.

--impl reference times the same loop with all host cores on the headline's
views (the oracle port: the reference's AVX2 build cannot run on the Arm
host; the reference has no learned selection).  --cpu-compare (x86 with the
reference's sources) times the AVX2 build against the oracle on one core.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "views/sec @1080p: plain vs batched+learned on 1 GB300; culls kept vs full, 0 false"
W, H = 1920, 1080
NQ = 100_000
FRAMES = 300
L2_FLUSH_BYTES = 256 << 20
LEARNED_VIEWS = 64  # 1920x1080 street-level views per batched launch


def workload():
    from rasterizer_gb300 import scenes
    mesh = scenes.city_scene()
    mvps, eyes = scenes.camera_path(FRAMES, seed=7)
    mins, maxs = scenes.query_boxes(NQ, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    return mesh, mvps, mins, maxs


def workload_desc(mesh, occ):
    quads = sum(o.quads for o in occ)
    return (f"dense city 64x64 buildings ({mesh.triangles} tris -> {quads} quads in {len(occ)} occluders), "
            f"{W}x{H}, {FRAMES}-frame seeded street-level camera path, {NQ} lognormal query boxes per frame, "
            f"plain all-occluder loop gated on the GPU")


# ---- clocks -------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.tmp = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.tmp.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.tmp.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(self.device):
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.tmp.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "samples": len(sm), "reasons": sorted(reasons)}


# ---- CPU legs -------------------------------------------------------------------------

_CPU_STATE = None
CITY_FIXTURE = os.path.join(ROOT, "tests", "golden", "city_occluders.npz")


def headline_views():
    """(views, frames, 16) matrices and (views, frames, 4) eyes of the headline's street-level views."""
    from rasterizer_gb300 import scenes
    paths = [scenes.camera_path(64, seed=7000 + k) for k in range(LEARNED_VIEWS)]
    return np.stack([m for m, _ in paths]), np.stack([e for _, e in paths])


def headline_config(world: int) -> dict:
    """The workload both arms run (the same dict in both bench lines)."""
    return {"workload": f"{LEARNED_VIEWS} street-level 1920x1080 views of the dense city per step (seeded paths, "
                        f"259,534 tris baked into 386 occluders / 129,768 quads), {NQ} lognormal query boxes per view",
            "resolution": f"{W}x{H}", "views_per_step": LEARNED_VIEWS, "queries_per_view": NQ,
            "l2": f"inputs larger than L2 ({LEARNED_VIEWS} depth buffers of 4 MB per step)",
            "parallelism": f"replicas x{world}"}


def _cpu_state():
    """Per-process CPU state: the city's occluders as the reference bakes them
    (tests/golden/city_occluders.npz: no native library of this project is
    loaded), the headline's views, the queries and one Oracle rasterizer."""
    global _CPU_STATE
    if _CPU_STATE is None:
        from oracle.bindings import Oracle, load_baked_scene
        from rasterizer_gb300 import scenes
        scene = load_baked_scene(CITY_FIXTURE)
        mins, maxs = scenes.query_boxes(NQ, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
        mvps, eyes = headline_views()
        _CPU_STATE = (scene, mvps, eyes, mins, maxs, Oracle(W, H))
    return _CPU_STATE


def _cpu_frame(f: int) -> int:
    """One view on the CPU oracle with the reference's own frame loop
    (Main.cpp:181-206: occluders front to back, each queried against the live
    buffer before it is drawn) and all its queries: view f % 64 at frame f // 64."""
    scene, mvps, eyes, mins, maxs, orc = _cpu_state()
    v, t = f % LEARNED_VIEWS, (f // LEARNED_VIEWS) % mvps.shape[1]
    orc.frame_gated(scene, mvps[v, t], eyes[v, t])
    orc.query(mins, maxs)
    return 1


def _cpu_frame_plain(f: int) -> int:
    """The same view with the plain all-occluder loop (the parity loop)."""
    scene, mvps, eyes, mins, maxs, orc = _cpu_state()
    v, t = f % LEARNED_VIEWS, (f // LEARNED_VIEWS) % mvps.shape[1]
    orc.frame_plain(scene, mvps[v, t])
    orc.query(mins, maxs)
    return 1


def _timed_frames(fn, budget_s: float, max_frames: int):
    done, t0 = 0, time.perf_counter()
    while done < max_frames and time.perf_counter() - t0 < budget_s:
        fn(done)
        done += 1
    return done, time.perf_counter() - t0


def cpu_baseline(budget_s: float = 12.0, max_frames: int = 128):
    _cpu_state()
    _cpu_frame(0)  # warm-up
    done, secs = _timed_frames(_cpu_frame, budget_s, max_frames)
    pdone, psecs = _timed_frames(_cpu_frame_plain, budget_s / 3, max_frames)
    return {"value": done / secs, "unit": "views/s", "cores": 1, "kind": "port",
            "sample": f"{done} views of the headline workload (its 64 street views in order, then their next "
                      f"frames), the reference's own frame loop (Main.cpp:181-206, occluders front to back, "
                      f"each queried against the live buffer) on its own bake, all {NQ} queries each, 1 host "
                      f"thread, CPU oracle (portable restatement; the reference's AVX2 build does not run on "
                      f"the Arm host)",
            "plain_loop_views_per_s": pdone / psecs, "plain_loop_sample": f"{pdone} views, all-occluder loop"}


def _warm(_):
    _cpu_frame(0)
    return 0


def run_reference(args):
    """--impl reference: the reference's own frame loop on all host cores
    (oracle port), each step one round of the headline's 64 views spread
    over one process per core (16 cores: 4 views each)."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import bindings
    bindings.build_oracle()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_warm, range(cores), chunksize=1)
        for w in range(args.warmup):
            pool.map(_cpu_frame, range(w * LEARNED_VIEWS, (w + 1) * LEARNED_VIEWS), chunksize=1)
        # the steps' views as one stream of tasks: a worker takes the next view
        # as soon as it is free, so no step waits for its slowest view
        t0 = time.perf_counter()
        total = sum(pool.imap_unordered(_cpu_frame, range(args.steps * LEARNED_VIEWS), chunksize=1))
        dt = time.perf_counter() - t0
    value = total / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "views/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/u16",
            "data": "synthetic", "config": headline_config(1),
            "cpu_baseline": {"value": value, "unit": "views/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} steps of {LEARNED_VIEWS} views (the headline's 64 street "
                                       f"views, each step their next frame, one stream of tasks over the "
                                       f"workers), the reference's own frame loop "
                                       f"(Main.cpp:181-206) on its own bake (tests/golden/city_occluders.npz), "
                                       f"all {NQ} queries per view, {cores} worker processes; CPU oracle, because "
                                       f"the reference's AVX2 build cannot run on aarch64 (one x86 core: the "
                                       f"AVX2 build draws these views about 5x as fast as the oracle, "
                                       f"bench.py --cpu-compare)"},
            "e2e": {"value": value, "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_compare(frames: int = 16):
    """x86-64 with oracle/_ref only: one core, the headline's views, the
    reference's AVX2 build against the portable oracle, both frame loops
    (each frame followed by its 100k queries).  Prints one JSON line."""
    from oracle import bindings
    from oracle.bindings import Reference, ReferenceScene
    from rasterizer_gb300 import scenes
    if not bindings.reference_available():
        raise SystemExit("cpu-compare needs x86-64 and the reference sources")
    bindings.build_oracle()
    bindings.build_reference()
    scene, mvps, eyes, mins, maxs, orc = _cpu_state()
    mesh = scenes.city_scene()
    rs = ReferenceScene(mesh.vertices, mesh.indices)
    ref, scratch = Reference(W, H), Reference(W, H)
    out = {"host": os.uname().machine, "frames": frames, "queries_per_frame": NQ}
    legs = {
        "oracle_gated": lambda v, t: orc.frame_gated(scene, mvps[v, t], eyes[v, t]),
        "reference_gated": lambda v, t: rs.frame_gated(ref, mvps[v, t], eyes[v, t]),
        "oracle_plain": lambda v, t: orc.frame_plain(scene, mvps[v, t]),
        "reference_plain": lambda v, t: rs.frame_plain(ref, scratch, mvps[v, t]),
    }
    for name, frame in legs.items():
        q = (lambda: orc.query(mins, maxs)) if name.startswith("oracle") else (lambda: ref.query(mins, maxs))
        frame(0, 0)
        q()
        t0 = time.perf_counter()
        for f in range(frames):
            frame(f % LEARNED_VIEWS, f // LEARNED_VIEWS)
            q()
        out[name + "_views_per_s"] = frames / (time.perf_counter() - t0)
    out["oracle_over_reference_gated"] = out["oracle_gated_views_per_s"] / out["reference_gated_views_per_s"]
    out["oracle_over_reference_plain"] = out["oracle_plain_views_per_s"] / out["reference_plain_views_per_s"]
    rs.close()
    print(json.dumps(out), flush=True)


# ---- GPU leg --------------------------------------------------------------------------

def algorithmic_bytes(q_setup: int, nq: int):
    """Per-launch algorithmic bytes: packed quads read (16 B/quad), depth
    written once (2 B/pixel), hiZ cleared and written (2+2 B/block), query
    boxes read (32 B) and two result bits written per query."""
    blocks = (W // 8) * (H // 8)
    return {
        "k_setup": 16 * q_setup,
        "k_raster": 2 * W * H + 4 * blocks,
        "k_query": 32 * nq + nq // 4,
        "frame": 16 * q_setup + 2 * W * H + 4 * blocks + 32 * nq + nq // 4,
    }


def max_over_ranks(ms: float, world: int, device) -> float:
    """Device time of a replica; with several ranks, the maximum over ranks."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def views_per_s(steps: int, world: int, device_ms: float) -> float:
    """Whole-job throughput: every rank renders `steps` views in the slowest rank's time."""
    return world * steps / (device_ms * 1e-3)


def load_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def run_batched(ctx_dev: int, occ, steps: int):
    """The 256-view workload: every view's occluder subset gated on the GPU and
    its queries answered, all views in one prepared batch (one CUDA graph
    launch) versus the same views one single-view launch at a time.  Returns
    a dict for the bench line."""
    import torch
    from rasterizer_gb300 import api, scenes
    centers = np.stack([o.center for o in occ])
    quads = np.array([o.quads for o in occ])
    pmin, pmax = scenes.query_boxes(NQ, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    specs = scenes.multiview_workload(centers, quads, NQ)
    ctx = api.Context(ctx_dev)
    views = []
    for s in specs:
        sel = [occ[i] for i in s.occluders]
        views.append(dict(raster=api.Rasterizer(ctx, s.width, s.height), mvp=s.mvp, clear=True, occluders=sel,
                          flags=np.full(len(sel), 2, np.uint8), mins=pmin[s.query_start:s.query_start + s.query_count],
                          maxs=pmax[s.query_start:s.query_start + s.query_count]))
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", ctx_dev))

    def timed(launch, reps):
        for _ in range(2):
            launch()
        ctx.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            launch()
        b.record(stream)
        ctx.synchronize()
        return a.elapsed_time(b) / reps

    batch = api.PreparedBatch(ctx, views)
    ok = batch.check()
    ms_batched = timed(batch.launch, steps)
    ok = batch.check() and ok
    batch.close()
    singles = [api.PreparedBatch(ctx, [v]) for v in views]

    def all_single():
        for b in singles:
            b.launch()

    ms_single = timed(all_single, max(1, steps // 2))
    ok = all(b.check() for b in singles) and ok
    for b in singles:
        b.close()
    n = len(views)
    return {"views": n, "pixels": int(sum(s.width * s.height for s in specs)),
            "quads_set_up": int(sum(int(quads[s.occluders].sum()) for s in specs)),
            "queries": int(sum(s.query_count for s in specs)),
            "batched_views_per_s": n / (ms_batched * 1e-3), "batched_ms_per_launch": ms_batched,
            "single_view_views_per_s": n / (ms_single * 1e-3), "single_view_ms_per_round": ms_single,
            "speedup": ms_single / ms_batched, "capacity_ok": bool(ok),
            "note": "64x1024^2 cascades + 96x512^2 cube faces + 96 probe views 256x128..1920x1080, "
                    "per-view occluder subsets 1k-200k tris, 10k-100k queries per view; all occluders gated on the "
                    "GPU (no learned selection yet)"}


def _time_launches(ctx, stream, launch, reps, before=None):
    """Mean device ms per launch: CUDA events on the library's stream around
    each launch (`before(i)` runs outside the events)."""
    import torch
    for i in range(3):
        if before:
            before(i)
        launch()
    ctx.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for i, (a, b) in enumerate(evs):
        if before:
            before(i)
        a.record(stream)
        launch()
        b.record(stream)
    ctx.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / reps


def run_learned(ctx, occ, pmin, pmax, world, rank, dev, args):
    """Learned occluder selection.  Trains the selector on the GPU (labels from
    the rasteriser over seeded poses), picks per workload the smallest
    candidate fraction K that keeps >= 99% of the occlusion culls on held-out
    validation views, reports culls kept vs the full frames, false culls and
    the nearest-first ranking at the same K on held-out test views, and times
    the batched + learned launch (the headline) against the plain batched one."""
    import torch
    from rasterizer_gb300 import api, learned as L
    centers = np.stack([o.center for o in occ])
    quads = np.array([o.quads for o in occ])
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    t = L.Timer()
    net, report = L.train_selector(ctx, occ, NQ, log=None, mins=pmin, maxs=pmax)
    out = {"training": dict(report, seconds=t.lap())}
    fracs = (0.05, 0.1, 0.2, 0.35, 0.5)

    def pick(tracks_val):
        full = L.run_full(ctx, occ, tracks_val, pmin, pmax)
        for f in fracs:
            if L.evaluate_learned(ctx, occ, tracks_val, pmin, pmax, net, f, full).retained >= 0.99:
                return f
        return 1.0

    # ---- street level, 1920x1080 ----
    k_st = pick(L.street_tracks(6, 30, seed0=6000, n_occluders=len(occ), queries=NQ))
    test = L.street_tracks(8, 30, seed0=5000, n_occluders=len(occ), queries=NQ)
    full = L.run_full(ctx, occ, test, pmin, pmax)
    sweep = {}
    for f in fracs:
        a = L.evaluate_learned(ctx, occ, test, pmin, pmax, net, f, full)
        b = L.evaluate_heuristic(ctx, occ, test, pmin, pmax, "nearest", f, full)
        sweep[str(f)] = {"learned": a.as_dict(), "nearest_first": b.as_dict()}

    paths = L.street_tracks(LEARNED_VIEWS, 64, seed0=7000, n_occluders=len(occ), queries=NQ)
    views = L._views(ctx, occ, paths, pmin, pmax)

    def mover(bt, tracks, frames):
        stacked = np.stack([tr.mvps[:frames] for tr in tracks], axis=1)  # (frames, views, 16)

        def before(i):
            bt.setModelViewProjections(stacked[i % frames])
        return before

    plain = api.PreparedBatch(ctx, views)
    ms_plain = _time_launches(ctx, stream, plain.launch, 50, mover(plain, paths, 64))
    ok = plain.check()
    plain.close()

    # headline: batched + learned launches in the zero-depth clear (each frame
    # stands alone, so its culls compare with the full frame at the same
    # poses), barrier + synchronize around the timed region; each launch's
    # result bits are copied out behind its end event (outside the timing)
    sel = api.PreparedBatch(ctx, views)
    sel.setSelection(net, k_st, trackWins=True)
    sel.setZeroDepth(True)
    move = mover(sel, paths, 64)
    for i in range(args.warmup):
        move(i)
        sel.launch()
    ok = sel.check() and ok
    tuning = sel.autotune(5)  # launch shapes for this batch, picked before the timed region
    for i in range(args.warmup):
        move(i)
        sel.launch()
    ok = sel.check() and ok
    kept = min(args.steps, 64)  # launches whose bits are kept for the cull count
    words = sel.resultWords()
    bits = torch.empty((kept, words), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(dev.index) if rank == 0 else None
    time.sleep(0.3 if sampler else 0)
    _barrier(world)
    ctx.synchronize()
    torch.cuda.synchronize()
    for i in range(args.steps):
        move(i)
        starts[i].record(stream)
        sel.launch()
        ends[i].record(stream)
        if i < kept:
            sel.resultsAllAsync(bits[i])
    ctx.synchronize()
    torch.cuda.synchronize()
    _barrier(world)
    clocks = sampler.stop() if sampler else None
    ok = sel.check() and ok
    dev_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(starts, ends)), world, dev)
    stats = sel.stats()
    prof = sel.profile(20)
    kern = dict(zip(["setup", "scan", "fill", "walk", "raster", "query", "selection"], [float(x) for x in prof]))
    # culls kept and false culls of those timed launches, against the full
    # frames (every candidate, zero-depth clear) at the same poses
    timed_tracks = [L.Track(t.width, t.height, t.occluders, t.mvps[[i % 64 for i in range(kept)]], t.query_start,
                            t.query_count, t.kind) for t in paths]
    full_timed = L.run_full(ctx, occ, timed_tracks, pmin, pmax)
    res_first = sel.resultsAll()[2]
    timed_culls = L.CullStats()
    for i in range(kept):
        for v in range(LEARNED_VIEWS):
            a0 = int(res_first[v])
            vis = api.unpack_bits(bits[i, a0:a0 + (NQ + 31) // 32], NQ)
            timed_culls.add_culls(~vis, full_timed[i][v])
    del full_timed
    # end to end through the public API: the step's 64 matrices from the
    # host, launch, every view's result bits back to the host
    e2e_steps = 50
    sel.resultsAll()
    t1 = time.perf_counter()
    for i in range(e2e_steps):
        move(i)
        sel.launch()
        vis_words, nc_words, _ = sel.resultsAll()
    e2e_s = time.perf_counter() - t1
    # the same with every view's query boxes uploaded from the host each step
    # (moving objects: the reference takes every query's box from the caller),
    # two box sets alternating, page-locked
    nbox = LEARNED_VIEWS * NQ
    box_sets = []
    for j in range(2):
        lo = torch.empty((nbox, 4), dtype=torch.float32, pin_memory=True).numpy()
        hi = torch.empty((nbox, 4), dtype=torch.float32, pin_memory=True).numpy()
        shift = np.float32(0.25 * j)
        lo[:] = np.tile(pmin, (LEARNED_VIEWS, 1)) + shift
        hi[:] = np.tile(pmax, (LEARNED_VIEWS, 1)) + shift
        lo[:, 3] = hi[:, 3] = 1.0
        box_sets.append((lo, hi))
    for i in range(3):
        sel.setQueries(*box_sets[i % 2])
        sel.launch()
        sel.resultsAll()
    t1 = time.perf_counter()
    for i in range(e2e_steps):
        move(i)
        sel.setQueries(*box_sets[i % 2])
        sel.launch()
        vis_words, nc_words, _ = sel.resultsAll()
    e2e_dyn_s = time.perf_counter() - t1
    sel.close()
    for v in views:
        v["raster"].close()
    blocks = (W // 8) * (H // 8)
    raster_bytes = LEARNED_VIEWS * (2 * W * H + 4 * blocks)  # depth written once, hiZ cleared + written
    out["street_1080p"] = {
        "k_fraction": k_st, "test_views": f"{len(test)} held-out paths x 30 frames", "sweep": sweep,
        "at_k": sweep.get(str(k_st)), "views_per_launch": LEARNED_VIEWS,
        "batched_plain_views_per_s": LEARNED_VIEWS / (ms_plain * 1e-3),
        "batched_learned_views_per_s": world * LEARNED_VIEWS * args.steps / (dev_ms * 1e-3),
        "kernels_ms_per_launch": kern, "work_last_launch": stats, "autotune": tuning, "capacity_ok": bool(ok)}
    headline = {
        "value": world * LEARNED_VIEWS * args.steps / (dev_ms * 1e-3), "ms_per_step": dev_ms / args.steps,
        "clocks": clocks, "kernels": kern,
        "culls_timed": dict(timed_culls.as_culls_dict(), launches=kept, views=kept * LEARNED_VIEWS,
                            against="full frames (every candidate, zero-depth clear) at the same poses"),
        "roofline": {"bound": "hbm", "kernel": "k_raster", "unit": "GB/s",
                     "achieved": raster_bytes / (kern["raster"] * 1e-3) / 1e9, "algorithmic_bytes": raster_bytes},
        "e2e": {"value": world * LEARNED_VIEWS * e2e_steps / e2e_s, "unit": "views/s",
                "h2d_bytes_per_step": stats["table_bytes"], "d2h_bytes_per_step": int(vis_words.nbytes + nc_words.nbytes),
                "path": "PreparedBatch.setModelViewProjections (64 matrices) / launch / resultsAll (every view's "
                        "bits, one copy) through the Python mirror of the C ABI, wall clock"},
        "e2e_dynamic_boxes": {
            "value": world * LEARNED_VIEWS * e2e_steps / e2e_dyn_s, "unit": "views/s",
            "h2d_bytes_per_step": stats["table_bytes"] + 2 * 16 * nbox,
            "d2h_bytes_per_step": int(vis_words.nbytes + nc_words.nbytes),
            "path": "as e2e, plus PreparedBatch.setQueries: every view's 100k boxes (min and max float4) from "
                    "page-locked host memory each step, two box sets alternating"},
        # kernels per graph launch (the ncu launch list agrees): k_features and
        # k_select_view, then the flush's k_chunk_gate, k_setup, k_scan, k_fill,
        # k_walk_prep, k_raster, k_query
        "launches_per_step": 2 + 7}
    # ---- the 256-view workload (mixed resolutions) ----
    k_mv = pick(L.multiview_tracks(centers, quads, NQ, frames=4, seed=9))
    test = L.multiview_tracks(centers, quads, NQ, frames=4, seed=3)
    full = L.run_full(ctx, occ, test, pmin, pmax)
    a = L.evaluate_learned(ctx, occ, test, pmin, pmax, net, k_mv, full)
    b = L.evaluate_heuristic(ctx, occ, test, pmin, pmax, "nearest", k_mv, full)
    views = L._views(ctx, occ, test, pmin, pmax)
    plain = api.PreparedBatch(ctx, views)
    ms_plain = _time_launches(ctx, stream, plain.launch, 20, mover(plain, test, 4))
    ok = plain.check()
    plain.close()
    sel = api.PreparedBatch(ctx, views)
    sel.setSelection(net, k_mv, trackWins=True)
    sel.launch()
    sel.check()
    tuning_mv = sel.autotune(3)
    ms_sel = _time_launches(ctx, stream, sel.launch, 20, mover(sel, test, 4))
    ok = sel.check() and ok
    kern_mv = dict(zip(["setup", "scan", "fill", "walk", "raster", "query", "selection"],
                       [float(x) for x in sel.profile(5)]))
    sel.close()
    for v in views:
        v["raster"].close()
    out["multiview_256"] = {"k_fraction": k_mv, "learned": a.as_dict(), "nearest_first": b.as_dict(),
                            "batched_plain_views_per_s": len(test) / (ms_plain * 1e-3),
                            "batched_learned_views_per_s": len(test) / (ms_sel * 1e-3),
                            "batched_learned_ms_per_launch": ms_sel, "kernels_ms_per_launch": kern_mv,
                            "autotune": tuning_mv,
                            "capacity_ok": bool(ok)}
    if not args.no_large:
        out["large_4k_plus_63"] = run_large(ctx, net, dev)
    out["seconds"] = t.lap() + out["training"]["seconds"]
    net.close()
    return out, headline


LARGE_NQ = 1_000_000


def _gpu_bake_timing(ctx, sets, lo, hi, host_occ, reps: int = 5) -> dict:
    """Occluder::bake of every occluder in one GPU launch
    (occ_occluders_bake_device), device time with CUDA events on the
    library's stream, inputs already on the device; checked byte for byte
    against the host bake."""
    import torch
    from rasterizer_gb300 import api
    from rasterizer_gb300._lib import check, lib
    n = len(sets)
    starts = np.zeros(n + 1, np.uint32)
    starts[1:] = np.cumsum([len(s) for s in sets])
    boxes = np.tile(np.concatenate([lo, hi]), (n, 1)).astype(np.float32)
    dev = torch.device("cuda", ctx.device)
    dv = torch.from_numpy(np.concatenate(sets).astype(np.float32)).to(dev)
    dp = torch.empty(int(starts[-1]), dtype=torch.int32, device=dev)
    db = torch.empty(20 * n, dtype=torch.float32, device=dev)
    torch.cuda.synchronize(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    call = lambda: check(lib().occ_occluders_bake_device(ctx.handle, n, dv.data_ptr(), starts.ctypes.data,
                                                         boxes.ctypes.data, dp.data_ptr(), db.data_ptr()), "bake")
    call()  # warm-up (scratch allocation)
    ctx.synchronize()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    packed = dp.cpu().numpy().view(np.uint32)
    bounds = db.cpu().numpy().reshape(n, 20)
    same = all(np.array_equal(packed[starts[k]:starts[k + 1]], o.packed[:8 * o.packetCount])
               and np.array_equal(bounds[k, 8:20].view(np.uint32),
                                  np.concatenate([o.boundsMin, o.boundsMax, o.center]).view(np.uint32))
               for k, o in enumerate(host_occ))
    return {"occluders": n, "quads": int(starts[-1]) // 4, "seconds": statistics.median(times),
            "identical_to_host": bool(same), "launches": 1}


def run_large(ctx, net, dev):
    """The large combined workload: a seeded 2M-triangle city (128x128
    buildings), one 3840x2160 main view plus 63 mixed-resolution views in one
    launch, 1M query boxes; K chosen for >= 99 % of the occlusion culls on a
    validation variant; culls kept against the plain all-occluder frames, and
    views/s and queries/s of the plain and the learned launch (autotuned)."""
    import torch
    from rasterizer_gb300 import api, learned as L, scenes
    t = L.Timer()
    mesh = scenes.city_scene(grid=128, target_tris=2_000_000)
    t.lap()
    # the scene preparation of api.scene_batches step by step: quads, per-quad
    # boxes, SAH batches (host), and the same batches on the GPU
    v = np.ascontiguousarray(mesh.vertices, np.float32).reshape(-1, 4)
    q = api.QuadDecomposition.decompose(mesh.indices, v)
    decompose_s = t.lap()
    pad = (-q.size) % 32
    if pad:
        q = np.concatenate([q, np.full(pad, q[0], np.uint32)])
    corners = v[q.reshape(-1, 4)]
    qboxes = api._quad_boxes(corners)
    t.lap()
    batches = api.SurfaceAreaHeuristic.generateBatches(qboxes, 512, 8)
    sah_host_s = t.lap()
    sah_gpu_times = []
    for _ in range(3):
        gb = api.SurfaceAreaHeuristic.generateBatchesDevice(ctx, qboxes, 512, 8, timed=sah_gpu_times)
    sah_same = len(gb) == len(batches) and all(np.array_equal(a, b) for a, b in zip(gb, batches))
    del gb
    ref_lo, ref_hi = api._box_of(v)
    sets = [np.ascontiguousarray(corners[b].reshape(-1, 4)) for b in batches]
    prep_s = decompose_s + sah_host_s
    t.lap()
    occ = [api.Occluder.bake(s, ref_lo, ref_hi) for s in sets]              # Occluder::bake per batch (host)
    host_bake_s = t.lap()
    native = api.bake_scene(mesh.vertices, mesh.indices)                    # the same in one native call
    native_s = t.lap()
    native_same = len(native) == len(occ) and all(
        a.packetCount == b.packetCount and np.array_equal(a.packed[:8 * a.packetCount], b.packed[:8 * b.packetCount])
        for a, b in zip(native, occ))
    del native
    bake_s = prep_s + host_bake_s
    gpu_bake = _gpu_bake_timing(ctx, sets, ref_lo, ref_hi, occ)
    t.lap()
    # the baked occluder file: save once, then time a load against the bake
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "city2m.occ")
        api.save_occluders(path, occ)
        t0 = time.perf_counter()
        loaded = api.load_occluders(path)
        load_s = time.perf_counter() - t0
        file_bytes = os.path.getsize(path)
    same = len(loaded) == len(occ) and all(
        a.packetCount == b.packetCount and np.array_equal(a.packed[:8 * a.packetCount], b.packed)
        for a, b in zip(occ, loaded))
    del loaded
    t.lap()
    centers = np.stack([o.center for o in occ])
    quads = np.array([o.quads for o in occ])
    pmin, pmax = scenes.query_boxes(LARGE_NQ, seed=45, footprint=600.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    val = L.large_tracks(centers, quads, LARGE_NQ, frames=2, seed=6)
    fval = L.run_full(ctx, occ, val, pmin, pmax)
    k = 1.0
    for f in (0.05, 0.1, 0.2, 0.35, 0.5):
        if L.evaluate_learned(ctx, occ, val, pmin, pmax, net, f, fval).retained >= 0.99:
            k = f
            break
    test = L.large_tracks(centers, quads, LARGE_NQ, frames=2, seed=5)
    full = L.run_full(ctx, occ, test, pmin, pmax)
    a = L.evaluate_learned(ctx, occ, test, pmin, pmax, net, k, full)
    b = L.evaluate_heuristic(ctx, occ, test, pmin, pmax, "nearest", k, full)
    views = L._views(ctx, occ, test, pmin, pmax)
    nq = sum(tr.query_count for tr in test)

    stacked = np.stack([tr.mvps[:2] for tr in test], axis=1)

    def mover(bt):
        def before(i):
            bt.setModelViewProjections(stacked[i % 2])
        return before

    out = {}
    for name, frac in (("plain", None), ("learned", k)):
        bt = api.PreparedBatch(ctx, views)
        if frac is not None:
            bt.setSelection(net, frac, trackWins=True)
        bt.launch()
        bt.check()
        tuned = bt.autotune(3)["tuned"]
        ms = _time_launches(ctx, stream, bt.launch, 20, mover(bt))
        ok = bt.check()
        out[name] = {"ms_per_launch": ms, "views_per_s": len(test) / (ms * 1e-3),
                     "queries_per_s": nq / (ms * 1e-3), "autotune": tuned, "capacity_ok": bool(ok)}
        bt.close()
    for v in views:
        v["raster"].close()
    return {"workload": f"2M-triangle city ({mesh.triangles} tris -> {int(quads.sum())} quads in {len(occ)} "
                        f"occluders), one 3840x2160 main view + 63 mixed views per launch, {nq} query boxes "
                        f"per launch ({LARGE_NQ} pool)",
            "bake_seconds": bake_s,
            "bake_steps_seconds": {"decompose": decompose_s, "sah_host": sah_host_s,
                                   "occluder_bake_host": host_bake_s},
            "gpu_sah": {"quads": int(len(qboxes)), "batches": len(batches), "seconds": min(sah_gpu_times),
                        "identical_to_host": bool(sah_same), "host_seconds": sah_host_s,
                        "note": "occ_sah_generate_batches_device, boxes already on the device, best of 3"},
            "scene_bake_one_call": {"seconds": native_s, "identical": bool(native_same)},
            "gpu_bake": gpu_bake,
            "baked_file": {"load_seconds": load_s, "bytes": file_bytes, "identical": bool(same),
                           "speedup_vs_bake": bake_s / max(load_s, 1e-9)},
            "k_fraction": k, "learned": a.as_dict(), "nearest_first": b.as_dict(),
            "plain": out["plain"], "batched_learned": out["learned"],
            "speedup_vs_plain_batched": out["learned"]["views_per_s"] / out["plain"]["views_per_s"],
            "seconds": t.lap() + bake_s}


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_plain(ctx, r, occ, mvps, mins, maxs, world, dev, args):
    """The plain all-occluder path, one 1920x1080 view per launch along the
    camera path (L2 flushed between frames), its per-kernel times and the same
    frames end to end through the reference-facing API."""
    import torch
    from rasterizer_gb300 import api
    flags = np.full(len(occ), 2, np.uint8)  # OCC_GATED
    batch = api.PreparedBatch(ctx, [dict(raster=r, mvp=mvps[0], clear=True, occluders=occ, flags=flags,
                                         mins=mins, maxs=maxs)])
    for attempt in range(3):  # size the scratch for every frame of the path
        for f in range(FRAMES):
            batch.setModelViewProjection(0, mvps[f])
            batch.launch()
        if batch.check():
            break
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)

    def flush_l2(i):
        with torch.cuda.stream(stream):
            flush.fill_(i)

    steps = min(args.steps, 3000)
    for i in range(args.warmup):
        batch.setModelViewProjection(0, mvps[i % FRAMES])
        batch.launch()
        flush_l2(i)
    ctx.synchronize()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    _barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        batch.setModelViewProjection(0, mvps[i % FRAMES])
        starts[i].record(stream)
        batch.launch()
        ends[i].record(stream)
        flush_l2(i)
    ctx.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    _barrier(world)
    ok = batch.check()
    dev_ms = max_over_ranks(sum(s.elapsed_time(e) for s, e in zip(starts, ends)), world, dev)
    prof = batch.profile(min(steps, 300))
    names = ["k_setup", "k_scan", "k_fill", "k_walk_prep", "k_raster", "k_query"]
    kern = {n: float(v) for n, v in zip(names, prof)}
    top = max(kern, key=kern.get)
    q_setup = sum(o.quads for o in occ)
    alg = algorithmic_bytes(q_setup, NQ)
    peak, peak_note = hbm_peak()
    traffic = load_traffic()
    roof_kernel = top if top in alg else "k_query"
    achieved = alg[roof_kernel] / (kern[roof_kernel] * 1e-3) / 1e9
    frame_ms = sum(kern.values())
    # end to end through the reference-facing API with host buffers
    e2e_steps = max(10, min(steps // 10, 100))
    for i in range(3):
        r.clear()
        r.setModelViewProjection(mvps[i])
        r.rasterizeMany(occ, flags)
        r.queryVisibilityBatch(mins, maxs)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for i in range(e2e_steps):
        r.clear()
        r.setModelViewProjection(mvps[i % FRAMES])
        r.rasterizeMany(occ, flags)
        r.queryVisibilityBatch(mins, maxs)
    e2e_s = time.perf_counter() - t1
    h2d = NQ * 32 + 216 + 96 * len(occ) + 32 * ((q_setup + 255) // 256) + 12
    d2h = 2 * 4 * ((NQ + 31) // 32) + 4 * len(occ) + 48
    batch.close()
    return {
        "value": views_per_s(steps, world, dev_ms), "unit": "views/s", "steps": steps,
        "ms_per_step": dev_ms / steps, "queries_per_s": views_per_s(steps, world, dev_ms) * NQ,
        "wall_views_per_s": world * steps / wall, "kernels_ms": kern,
        "l2": "flushed between steps (256 MB write, outside the timed events)",
        "roofline": {"bound": "hbm", "kernel": roof_kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_note, "traffic": traffic.get(roof_kernel),
                     "algorithmic_bytes": alg[roof_kernel],
                     "frame_achieved": alg["frame"] / (frame_ms * 1e-3) / 1e9},
        "e2e": {"value": world * e2e_steps / e2e_s, "unit": "views/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": "Rasterizer.clear/setModelViewProjection/rasterizeMany(gated)/queryVisibilityBatch "
                        "(Python mirror -> C ABI), host numpy buffers, wall clock"},
        "capacity_ok": bool(ok)}


def hbm_peak():
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_gpu(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    # CPU baseline first (rank 0, N=1 only), before any GPU work
    cpu = cpu_baseline() if (rank == 0 and world == 1 and not args.no_cpu) else None

    from rasterizer_gb300 import api
    mesh, mvps, mins, maxs = workload()
    occ = api.bake_scene(mesh.vertices, mesh.indices)
    ctx = api.Context(local)
    r = api.Rasterizer(ctx, W, H)
    plain = run_plain(ctx, r, occ, mvps, mins, maxs, world, dev, args)
    batched = run_batched(local, occ, steps=5) if not args.no_batched else None
    learned, head = (None, None) if args.no_learned else run_learned(ctx, occ, mins, maxs, world, rank, dev, args)
    peak, peak_note = hbm_peak()
    traffic = load_traffic()

    line = {"metric": METRIC, "n_gpus": world, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/u16", "data": "synthetic"}
    if head is not None:
        k = learned["street_1080p"]["k_fraction"]
        at_k = learned["street_1080p"]["at_k"] or {}
        roof = dict(head["roofline"], peak=peak, peak_source=peak_note,
                    frac=head["roofline"]["achieved"] / peak, traffic=traffic.get("k_raster_batched"))
        line.update({
            "value": head["value"], "unit": "views/s", "steps": args.steps, "ms_per_step": head["ms_per_step"],
            "config": headline_config(world),
            "method": f"batched + learned: each view draws the selector's top {k:.0%} of its candidate occluders "
                      f"in the zero-depth clear (every frame stands alone), one CUDA graph launch per step",
            "culls": dict(head["culls_timed"], held_out_paths=at_k.get("learned")),
            "timing": "CUDA events on the library stream around each batched graph launch; max over ranks",
            "roofline": roof, "e2e": head["e2e"], "e2e_dynamic_boxes": head["e2e_dynamic_boxes"],
            "clocks": head["clocks"],
            "gpu_launches": head["launches_per_step"] * args.steps, "kernels_ms": head["kernels"]})
    else:
        line.update({"value": plain["value"], "unit": "views/s", "steps": plain["steps"],
                     "ms_per_step": plain["ms_per_step"], "roofline": plain["roofline"], "e2e": plain["e2e"],
                     "gpu_launches": 7 * plain["steps"], "kernels_ms": plain["kernels_ms"],
                     "config": {"workload": workload_desc(mesh, occ), "parallelism": f"replicas x{world}"}})
    line["plain_single_view"] = dict(plain, workload=workload_desc(mesh, occ))
    if batched is not None:
        line["batched"] = batched
    if learned is not None:
        line["learned"] = learned
        if batched is not None:
            line["learned"]["multiview_256"]["speedup_vs_single_view_plain"] = (
                learned["multiview_256"]["batched_learned_views_per_s"] / batched["single_view_views_per_s"])
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    r.close()
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def run_profile_frames(frames: int, start: int = 0):
    """A short GPU-only run for profilers: prepare the batch, then `frames`
    graph launches along the camera path (no CPU leg, no timing)."""
    from rasterizer_gb300 import api
    mesh, mvps, mins, maxs = workload()
    occ = api.bake_scene(mesh.vertices, mesh.indices)
    ctx = api.Context(0)
    r = api.Rasterizer(ctx, W, H)
    flags = np.full(len(occ), 2, np.uint8)
    batch = api.PreparedBatch(ctx, [dict(raster=r, mvp=mvps[start], clear=True, occluders=occ, flags=flags,
                                         mins=mins, maxs=maxs)])
    for f in range(frames):
        batch.setModelViewProjection(0, mvps[(start + f) % FRAMES])
        batch.launch()
    ok = batch.check()
    vis, _ = batch.results(0)
    print(json.dumps({"frames": frames, "capacity_ok": ok, "visible_last": int(vis.sum())}), flush=True)
    batch.close()
    r.close()
    ctx.close()


def run_profile_learned(frames: int, views: int, train_steps: int, extras: bool = False):
    """A short GPU-only run for profilers: the headline's batched + learned
    launch (first `views` street views, untrained selector at K = 5 % in the
    zero-depth clear: the same kernels and the same number of drawn occluders
    per view), `frames` graph launches, then `train_steps` listwise training
    steps on random rows.
    With `extras`, the first launch also runs the second pass and the cull
    labels (every kernel of the library then runs at least once)."""
    from rasterizer_gb300 import api, learned as L, scenes
    mesh = scenes.city_scene()
    occ = api.bake_scene(mesh.vertices, mesh.indices)
    pmin, pmax = scenes.query_boxes(NQ, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    ctx = api.Context(0)
    net = api.OccluderSelector(ctx, seed=0)
    paths = L.street_tracks(views, 64, seed0=7000, n_occluders=len(occ), queries=NQ)
    vs = L._views(ctx, occ, paths, pmin, pmax)
    b = api.PreparedBatch(ctx, vs)
    b.setSelection(net, 0.05, trackWins=True)
    b.setZeroDepth(True)
    if extras:
        b.setSecondPass(True)
        b.setCullLabels(True)
        b.launch()
        b.setSecondPass(False)
        b.setCullLabels(False)
    for f in range(frames):
        for v, tr in enumerate(paths):
            b.setModelViewProjection(v, tr.mvps[f % 64])
        b.launch()
    ok = b.check()
    rng = np.random.default_rng(0)
    x = rng.uniform(0, 1, (4096, 16)).astype(np.float32)
    y = rng.uniform(0, 1, 4096).astype(np.float32)
    gs = np.arange(0, 4097, 64, dtype=np.uint32)  # 64 groups of 64 rows
    for a, b_ in zip(gs[:-1], gs[1:]):
        y[a:b_] /= y[a:b_].sum()
    for _ in range(train_steps):
        net.trainStepListwise(x, y, gs, 1e-3)
    print(json.dumps({"frames": frames, "views": views, "capacity_ok": ok, "stats": b.stats()}), flush=True)
    b.close()
    net.close()
    ctx.close()


def run_profile_misc():
    """A short GPU-only run for profilers: the kernels outside the batched
    frame -- the GPU bake of a scene's occluders, a plain 1080p frame and its
    100k queries one box per thread, query2D, the no-allocation query path,
    a hiZ upload (per-tile minimum) and the four read-back formats."""
    import ctypes as C
    from rasterizer_gb300 import api, scenes
    from rasterizer_gb300._lib import check, lib
    mesh = scenes.boxes_scene()
    sets, lo, hi = api.scene_batches(mesh.vertices, mesh.indices)
    ctx = api.Context(0)
    occ = api.bake_on_gpu(ctx, sets, lo, hi)
    r = api.Rasterizer(ctx, W, H)
    r.clear()
    r.setModelViewProjection(scenes.boxes_camera(W, H))
    r.rasterizeMany(occ, np.full(len(occ), 2, np.uint8))
    r.flush()
    mins, maxs = scenes.query_boxes(NQ, seed=43)
    vis, _ = r.queryVisibilityBatch(mins, maxs)
    seen = r.query2D(0, 255, 0, 127, 40000)
    n = 4096
    a, b = np.ascontiguousarray(mins[:n], np.float32), np.ascontiguousarray(maxs[:n], np.float32)
    vb, nb = np.zeros(n // 32, np.uint32), np.zeros(n // 32, np.uint32)
    check(lib().occ_raster_query_batch_noalloc(r.handle, n, a.ctypes.data, b.ctypes.data, vb.ctypes.data,
                                               nb.ctypes.data), "occ_raster_query_batch_noalloc")
    r.writeHiZ(r.readHiZ())
    sums = {f: float(np.asarray(r.readBack(f), np.float64).sum()) for f in ("rgba8", "linear", "depth", "packed")}
    print(json.dumps({"occluders": len(occ), "visible": int(vis.sum()), "query2d": bool(seen),
                      "noalloc_visible": int(np.unpackbits(vb.view(np.uint8)).sum()), "readback_sums": sums}),
          flush=True)
    r.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-run", type=int, default=0, metavar="FRAMES",
                    help="only launch FRAMES frames (for ncu); prints a status line")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=30)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-view batched leg")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-selection leg (training included)")
    ap.add_argument("--no-large", action="store_true", help="skip the 2M-triangle 4K + 63-view leg")
    ap.add_argument("--profile-learned", type=int, default=0, metavar="FRAMES",
                    help="only launch the batched + learned frame FRAMES times (for ncu); prints a status line")
    ap.add_argument("--profile-views", type=int, default=LEARNED_VIEWS, help="views per launch for --profile-learned")
    ap.add_argument("--profile-train", type=int, default=0, help="training steps after --profile-learned")
    ap.add_argument("--profile-misc", action="store_true",
                    help="only launch the kernels outside the batched frame once each (for ncu)")
    ap.add_argument("--cpu-compare", action="store_true",
                    help="x86-64 with the reference's sources: one core, the reference's AVX2 build against the "
                         "portable oracle on the headline's views (both frame loops)")
    ap.add_argument("--profile-extras", action="store_true",
                    help="--profile-learned: first launch with the second pass and the cull labels")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.cpu_compare:
        cpu_compare()
    elif args.profile_misc:
        run_profile_misc()
    elif args.profile_learned:
        run_profile_learned(args.profile_learned, args.profile_views, args.profile_train, args.profile_extras)
    elif args.profile_run:
        run_profile_frames(args.profile_run)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
