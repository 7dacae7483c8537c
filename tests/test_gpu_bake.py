"""GPU bake (Occluder::bake on the device, many occluders per launch) against
the host bake, byte for byte; occluders registered from device memory;
queries from device memory."""
import numpy as np
import pytest

from rasterizer_gb300 import api, scenes
from oracle.bindings import Oracle

from helpers import gpu_plain_frame, mismatch_report, to_baked

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def _same(a: api.Occluder, b: api.Occluder) -> list[str]:
    bad = []
    if a.packetCount != b.packetCount or not np.array_equal(a.packed[:8 * a.packetCount], b.packed[:8 * b.packetCount]):
        bad.append("packed")
    for f in ("refMin", "refMax", "boundsMin", "boundsMax", "center"):
        if not np.array_equal(getattr(a, f).view(np.uint32), getattr(b, f).view(np.uint32)):
            bad.append(f)
    return bad


@pytest.mark.parametrize("scene", ["boxes", "city"])
def test_gpu_bake_equals_host_bake(ctx, scene):
    mesh = scenes.boxes_scene() if scene == "boxes" else scenes.city_scene()
    sets, lo, hi = api.scene_batches(mesh.vertices, mesh.indices)
    host = [api.Occluder.bake(s, lo, hi) for s in sets]
    gpu = api.bake_on_gpu(ctx, sets, lo, hi)
    bad = [(k, _same(h, g)) for k, (h, g) in enumerate(zip(host, gpu)) if _same(h, g)]
    assert not bad, bad[:5]


def test_gpu_bake_special_values(ctx):
    """Degenerate quads (zero normals: NaN centroids), NaN and infinite
    coordinates, signed zeros, coordinates outside the reference box, large
    occluders (more quads than the CTA has threads): bytes as on the host."""
    rng = np.random.default_rng(7)
    sets = []
    for k in range(24):
        nq = int(rng.choice([8, 16, 64, 504, 1024]))
        v = rng.normal(0, 10, (4 * nq, 4)).astype(np.float32)
        v[:, 3] = 1.0
        if k % 4 == 1:
            v[: 4 * (nq // 2)] = v[0]                       # degenerate quads
        if k % 4 == 2:
            idx = rng.integers(0, len(v), 8)
            v[idx, rng.integers(0, 3, 8)] = rng.choice(np.array([np.nan, np.inf, -np.inf, -0.0, 0.0], np.float32), 8)
        if k % 4 == 3:
            v[:, :3] = np.round(v[:, :3])                    # ties in the bounds, signed zeros
            v[rng.integers(0, len(v), 16), 0] = -0.0
        sets.append(v)
    lo = np.array([-20, -20, -20, 1], np.float32)
    hi = np.array([20, 20, 20, 1], np.float32)
    host = [api.Occluder.bake(s, lo, hi) for s in sets]
    gpu = api.bake_on_gpu(ctx, sets, lo, hi)
    bad = [(k, _same(h, g)) for k, (h, g) in enumerate(zip(host, gpu)) if _same(h, g)]
    assert not bad, bad[:5]


def test_device_upload_rasterizes_like_host_upload(ctx):
    """Occluders baked on the GPU and registered from device memory draw the
    same frame as the host-baked ones (and as the oracle)."""
    from rasterizer_gb300._lib import lib, check
    import ctypes as C
    mesh = scenes.boxes_scene()
    sets, lo, hi = api.scene_batches(mesh.vertices, mesh.indices)
    n = len(sets)
    starts = np.zeros(n + 1, np.uint32)
    starts[1:] = np.cumsum([len(s) for s in sets])
    boxes = np.tile(np.concatenate([lo, hi]), (n, 1)).astype(np.float32)
    dev = torch.device("cuda", 0)
    dv = torch.from_numpy(np.concatenate(sets)).to(dev)
    dp = torch.empty(int(starts[-1]), dtype=torch.int32, device=dev)
    db = torch.empty(20 * n, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    check(lib().occ_occluders_bake_device(ctx.handle, n, dv.data_ptr(), starts.ctypes.data, boxes.ctypes.data,
                                          dp.data_ptr(), db.data_ptr()), "bake")
    ctx.synchronize()
    bounds = db.cpu().numpy().reshape(n, 20)
    ids = []
    for k in range(n):
        oid = C.c_uint32()
        b = np.ascontiguousarray(bounds[k])
        check(lib().occ_occluder_upload_device(ctx.handle, dp.data_ptr() + 4 * int(starts[k]),
                                               int(starts[k + 1] - starts[k]) // 8, b.ctypes.data, C.byref(oid)),
              "upload")
        ids.append(oid.value)
    host = api.bake_scene(mesh.vertices, mesh.indices)
    mvp = scenes.boxes_camera()
    r1, r2 = api.Rasterizer(ctx, 640, 360), api.Rasterizer(ctx, 640, 360)
    for r in (r1, r2):
        r.clear()
        r.setModelViewProjection(mvp)
    ctx.synchronize()
    for k, o in enumerate(host):  # the device-registered occluders carry the same bounds
        assert np.array_equal(bounds[k, 8:12].view(np.uint32), o.boundsMin.view(np.uint32))
    id_arr, flags = np.array(ids, np.uint32), np.full(n, 2, np.uint8)  # kept alive across the call
    check(lib().occ_raster_rasterize_many(r1.handle, n, id_arr.ctypes.data, flags.ctypes.data), "rasterize_many")
    gpu_plain_frame(r2, host, mvp)
    orc = Oracle(640, 360)
    orc.frame_plain(to_baked(host), mvp)
    assert not mismatch_report("depth", r1.readDepthRaw(), orc.depth())
    assert not mismatch_report("depth", r2.readDepthRaw(), orc.depth())


def test_query_batch_device(ctx):
    """occ_raster_query_batch_device (device buffers, asynchronous) == the
    host-buffer batch query."""
    from rasterizer_gb300._lib import lib, check
    from helpers import boxes_occluders
    occ = boxes_occluders()
    mvp = scenes.boxes_camera()
    r = api.Rasterizer(ctx, 1920, 1080)
    gpu_plain_frame(r, occ, mvp)
    mins, maxs = scenes.query_boxes(10_000, seed=43)
    hv, hn = r.queryVisibilityBatch(mins, maxs)
    dev = torch.device("cuda", 0)
    dm = torch.from_numpy(np.ascontiguousarray(mins, np.float32)).to(dev)
    dM = torch.from_numpy(np.ascontiguousarray(maxs, np.float32)).to(dev)
    words = (len(mins) + 31) // 32
    dvb = torch.zeros(words, dtype=torch.int32, device=dev)
    dnb = torch.zeros(words, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    check(lib().occ_raster_query_batch_device(r.handle, len(mins), dm.data_ptr(), dM.data_ptr(), dvb.data_ptr(),
                                              dnb.data_ptr()), "query_batch_device")
    ctx.synchronize()
    vb = dvb.cpu().numpy().view(np.uint32)
    nb = dnb.cpu().numpy().view(np.uint32)
    assert np.array_equal(api.unpack_bits(vb, len(mins)), hv) and np.array_equal(api.unpack_bits(nb, len(mins)), hn)


# ---- SAH batching on the GPU ---------------------------------------------------------

def _scene_quad_boxes(mesh):
    """The per-quad boxes the scene preparation hands to SAH (Main.cpp:86-128)."""
    v = np.ascontiguousarray(mesh.vertices, np.float32).reshape(-1, 4)
    q = api.QuadDecomposition.decompose(mesh.indices, v)
    pad = (-q.size) % 32
    if pad:
        q = np.concatenate([q, np.full(pad, q[0], np.uint32)])
    return api._quad_boxes(v[q.reshape(-1, 4)])


def _tied_boxes(n, seed, snap):
    """Boxes with many equal centres and centres of -0 and +0 (equal under `<`)."""
    rng = np.random.default_rng(seed)
    lo = rng.uniform(-50, 50, (n, 4)).astype(np.float32)
    if snap:
        lo = np.round(lo / snap) * snap
    lo[:, 3] = 1.0
    hi = (lo + np.round(rng.uniform(0, 3, (n, 4)))).astype(np.float32)
    hi[:, 3] = 1.0
    z = rng.integers(0, n, n // 10)
    lo[z[::2], 0], hi[z[::2], 0] = np.float32(-0.0), np.float32(-0.0)
    lo[z[1::2], 0], hi[z[1::2], 0] = np.float32(0.0), np.float32(0.0)
    return np.ascontiguousarray(np.concatenate([lo, hi], axis=1), np.float32)


def _same_batches(a, b):
    return len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("case", ["boxes", "city", "tied8", "tied0", "tied25", "small-target"])
def test_gpu_sah_equals_host(ctx, case):
    """SurfaceAreaHeuristic::generateBatches on the GPU (level by level: stable
    radix sorts, segmented area scans, first cheapest split by atomicMin)
    gives the host's batches byte for byte, the host being pinned to the
    reference (Castle and Sponza on x86, tied and signed-zero centres)."""
    target, gran = 512, 8
    if case == "boxes":
        boxes = _scene_quad_boxes(scenes.boxes_scene())
    elif case == "city":
        boxes = _scene_quad_boxes(scenes.city_scene())
    elif case == "small-target":
        boxes, target, gran = _tied_boxes(4000, 7, 4.0), 40, 4
    else:
        snap = {"tied8": 8.0, "tied0": 0.0, "tied25": 25.0}[case]
        boxes = _tied_boxes(6000, 1 + len(case), snap)
    host = api.SurfaceAreaHeuristic.generateBatches(boxes, target, gran)
    dev = api.SurfaceAreaHeuristic.generateBatchesDevice(ctx, boxes, target, gran)
    assert len(host) > 1
    assert _same_batches(dev, host)


def test_gpu_sah_large_city_and_edges(ctx):
    """The 2M-triangle city's million quads; inputs of at most two granules
    (one batch); a NaN centre is refused (the host form handles it)."""
    boxes = _scene_quad_boxes(scenes.city_scene(grid=128, target_tris=2_000_000))
    t = []
    dev = api.SurfaceAreaHeuristic.generateBatchesDevice(ctx, boxes, 512, 8, timed=t)
    host = api.SurfaceAreaHeuristic.generateBatches(boxes, 512, 8)
    assert len(host) > 1000 and _same_batches(dev, host)
    small = _tied_boxes(16, 3, 0.0)
    assert _same_batches(api.SurfaceAreaHeuristic.generateBatchesDevice(ctx, small, 512, 8),
                         api.SurfaceAreaHeuristic.generateBatches(small, 512, 8))
    bad = _tied_boxes(100, 4, 0.0)
    bad[5, 1] = np.nan
    with pytest.raises(api.OccError) as e:
        api.SurfaceAreaHeuristic.generateBatchesDevice(ctx, bad, 8, 2)
    assert e.value.status == -5
