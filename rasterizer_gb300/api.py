"""Python mirror of the reference's Rasterizer / Occluder API over the C ABI.

Names and argument meanings follow SoftwareRasterizer/Rasterizer.h:10-61,
Occluder.h:7-21, QuadDecomposition.h:5-10 and SurfaceAreaHeuristic.h:5-12;
vectors (__m128 in the reference) are float4 numpy arrays.  The reference's
asserts become ValueError; GPU or allocation failures raise OccError.
"""
from __future__ import annotations

import ctypes as C
import os
import itertools
import weakref
from dataclasses import dataclass, field

import numpy as np

from ._lib import OccError, ViewWork, check, lib

P = C.c_void_p


def _f32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(P)


def unpack_bits(words: np.ndarray, n: int) -> np.ndarray:
    """Query result words (bit i%32 of word i/32) -> bool array of n."""
    b = np.unpackbits(np.ascontiguousarray(words, np.uint32).view(np.uint8), bitorder="little")
    return b[:n].astype(bool)


_context_serial = itertools.count(1)


def _context_open(child) -> bool:
    """True while the context that made `child` is open.  A context's close()
    closes its children first; only when the garbage collector finalises a
    context before a child whose weak entry it had already dropped (objects
    in one reference cycle, e.g. at interpreter exit) is the child's native
    object gone with the context, and the child must not touch it."""
    ctx = getattr(child, "ctx", None)
    return ctx is None or getattr(ctx, "handle", None) is not None


class Context:
    """One GPU and one CUDA stream; owns the uploaded occluders.  Closing it
    first closes the rasterizers, batches and selectors made on it."""

    def __init__(self, device: int = 0):
        h = P()
        check(lib().occ_ctx_create(device, C.byref(h)), "occ_ctx_create")
        self.handle = h.value
        self.device = device
        self.serial = next(_context_serial)  # never reused, unlike the handle's address
        self._children = weakref.WeakSet()

    def _adopt(self, child) -> None:
        self._children.add(child)

    def close(self):
        if getattr(self, "handle", None):
            for c in list(getattr(self, "_children", ())):
                c.close()
            lib().occ_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        check(lib().occ_ctx_synchronize(self.handle), "occ_ctx_synchronize")

    @property
    def stream(self) -> int:
        return lib().occ_ctx_stream(self.handle) or 0


@dataclass
class Occluder:
    """A baked occluder (Occluder.h:7-21): packed 11/11/10 vertex words in
    groups of 8 quads, the quantisation box and the bounds (w = 1)."""

    packed: np.ndarray          # uint32, packetCount * 8 words
    packetCount: int            # 32-byte vectors (4 per 8 quads)
    refMin: np.ndarray
    refMax: np.ndarray
    boundsMin: np.ndarray
    boundsMax: np.ndarray
    center: np.ndarray
    ids: dict = field(default_factory=dict, repr=False)  # context serial -> occluder id

    @staticmethod
    def bake(vertices, refMin, refMax) -> "Occluder":
        """Occluder::bake (Occluder.cpp:7-181): vertices (4 per quad, a multiple
        of 32: whole packets of 8 quads; the reference asserts a multiple of 16
        at :9 but packs 32 at a time at :108-122, reading past its array)."""
        v = _f32(vertices).reshape(-1, 4)
        if len(v) == 0 or len(v) % 32:
            raise ValueError("vertex count must be a positive multiple of 32 (8 quads per packet)")
        rmin, rmax = _f32(refMin, (4,)), _f32(refMax, (4,))
        packed = np.zeros(len(v), np.uint32)
        pc = C.c_uint32()
        bmin, bmax, ctr = np.zeros(4, np.float32), np.zeros(4, np.float32), np.zeros(4, np.float32)
        check(lib().occ_occluder_bake(_ptr(v), len(v), _ptr(rmin), _ptr(rmax), _ptr(packed), C.byref(pc),
                                      _ptr(bmin), _ptr(bmax), _ptr(ctr)), "occ_occluder_bake")
        return Occluder(packed, pc.value, rmin, rmax, bmin, bmax, ctr)

    @property
    def quads(self) -> int:
        return self.packetCount * 2

    def upload(self, ctx: Context) -> int:
        """Copies the packed data to the GPU once per context; returns its id."""
        if ctx.serial in self.ids:
            return self.ids[ctx.serial]
        oid = C.c_uint32()
        check(lib().occ_occluder_upload(ctx.handle, _ptr(self.packed), self.packetCount, _ptr(self.refMin),
                                        _ptr(self.refMax), _ptr(self.boundsMin), _ptr(self.boundsMax),
                                        C.byref(oid)), "occ_occluder_upload")
        self.ids[ctx.serial] = oid.value
        return oid.value


class QuadDecomposition:
    @staticmethod
    def decompose(indices, vertices) -> np.ndarray:
        """QuadDecomposition::decompose (QuadDecomposition.cpp:346-445)."""
        idx = np.ascontiguousarray(indices, np.uint32)
        v = _f32(vertices).reshape(-1, 4)
        out = np.zeros(max(4 * (idx.size // 3), 1), np.uint32)
        n = C.c_uint32()
        check(lib().occ_quad_decompose(_ptr(idx), idx.size, _ptr(v), len(v), _ptr(out), C.byref(n)),
              "occ_quad_decompose")
        return out[:n.value].copy()


class SurfaceAreaHeuristic:
    @staticmethod
    def generateBatches(aabbs, targetSize: int, splitGranularity: int) -> list[np.ndarray]:
        """SurfaceAreaHeuristic::generateBatches (SurfaceAreaHeuristic.cpp:96-104);
        aabbs: (n, 8) float32 rows of min4, max4."""
        a = _f32(aabbs).reshape(-1, 8)
        n = len(a)
        flat = np.zeros(max(n, 1), np.uint32)
        offs = np.zeros(n + 2, np.uint32)
        nb = C.c_uint32()
        check(lib().occ_sah_generate_batches(_ptr(a), n, targetSize, splitGranularity, _ptr(flat), _ptr(offs),
                                             C.byref(nb)), "occ_sah_generate_batches")
        return [flat[offs[i]:offs[i + 1]].copy() for i in range(nb.value)]

    @staticmethod
    def generateBatchesDevice(ctx: "Context", aabbs, targetSize: int, splitGranularity: int,
                              timed: list | None = None) -> list[np.ndarray]:
        """The same batches computed on the GPU (occ_sah_generate_batches_device).
        aabbs: (n, 8) float32 on the host (copied to the device first) or a
        device tensor.  With `timed` (a list), appends the call's seconds
        (inputs already on the device)."""
        import time
        import torch
        dev = torch.device("cuda", ctx.device)
        if isinstance(aabbs, torch.Tensor):
            d = aabbs.to(dev, torch.float32).contiguous()
        else:
            d = torch.from_numpy(_f32(aabbs).reshape(-1, 8)).to(dev)
        n = d.shape[0]
        flat = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        offs = np.zeros(n + 2, np.uint32)
        nb = C.c_uint32()
        torch.cuda.synchronize(dev)  # the upload ran on torch's stream
        t0 = time.perf_counter()
        check(lib().occ_sah_generate_batches_device(ctx.handle, d.data_ptr(), n, targetSize, splitGranularity,
                                                    flat.data_ptr(), _ptr(offs), C.byref(nb)),
              "occ_sah_generate_batches_device")
        if timed is not None:
            timed.append(time.perf_counter() - t0)
        f = flat.cpu().numpy().view(np.uint32)
        return [f[offs[i]:offs[i + 1]].copy() for i in range(nb.value)]


def scene_batches(vertices, indices, targetSize: int = 512, splitGranularity: int = 8):
    """The demo's scene preparation up to the bake (Main.cpp:86-128): quads,
    padding to a multiple of 8 quads, per-quad boxes, SAH batches.  Returns
    (per-occluder vertex arrays, 4 per quad; refMin; refMax = the box of all
    vertices)."""
    v = _f32(vertices).reshape(-1, 4)
    q = QuadDecomposition.decompose(indices, v)
    pad = (-q.size) % 32
    if pad:
        q = np.concatenate([q, np.full(pad, q[0], np.uint32)])
    corners = v[q.reshape(-1, 4)]                     # (nq, 4, 4)
    aabbs = _quad_boxes(corners)
    batches = SurfaceAreaHeuristic.generateBatches(aabbs, targetSize, splitGranularity)
    refMin, refMax = _box_of(v)
    return [np.ascontiguousarray(corners[b].reshape(-1, 4)) for b in batches], refMin, refMax


def bake_scene(vertices, indices, targetSize: int = 512, splitGranularity: int = 8) -> list[Occluder]:
    """The demo's scene preparation (Main.cpp:86-128) in one native call
    (occ_scene_bake): scene_batches, then one occluder per batch quantised in
    the box of all vertices."""
    v = _f32(vertices).reshape(-1, 4)
    idx = np.ascontiguousarray(indices, np.uint32).ravel()
    quads = idx.size // 3 + 7
    cap_count, cap_words = quads // 8 + 1, 4 * quads
    counts = np.zeros(max(cap_count, 1), np.uint32)
    packed = np.zeros(max(cap_words, 1), np.uint32)
    bounds = np.zeros((max(cap_count, 1), 20), np.float32)
    n, w = C.c_uint32(), C.c_uint64()
    check(lib().occ_scene_bake(_ptr(v), len(v), _ptr(idx), idx.size, targetSize, splitGranularity, cap_count,
                               cap_words, C.byref(n), C.byref(w), _ptr(counts), _ptr(packed), _ptr(bounds)),
          "occ_scene_bake")
    out, pos = [], 0
    for k in range(n.value):
        c = int(counts[k])
        b = bounds[k]
        out.append(Occluder(packed[pos:pos + 8 * c].copy(), c, b[0:4].copy(), b[4:8].copy(), b[8:12].copy(),
                            b[12:16].copy(), b[16:20].copy()))
        pos += 8 * c
    return out


def bake_on_gpu(ctx: Context, vertex_sets, refMin, refMax) -> list[Occluder]:
    """Occluder::bake for every vertex array of `vertex_sets` in one GPU
    launch (occ_occluders_bake_device; the same bytes as Occluder.bake), all
    quantised in [refMin, refMax]; returns host copies.  Device buffers come
    from PyTorch."""
    import torch
    n = len(vertex_sets)
    if n == 0:
        return []
    sets = [_f32(s).reshape(-1, 4) for s in vertex_sets]
    starts = np.zeros(n + 1, np.uint32)
    starts[1:] = np.cumsum([len(s) for s in sets])
    boxes = np.tile(np.concatenate([_f32(refMin, (4,)), _f32(refMax, (4,))]), (n, 1)).astype(np.float32)
    dev = torch.device("cuda", ctx.device)
    dv = torch.from_numpy(np.concatenate(sets)).to(dev)
    dp = torch.empty(int(starts[-1]), dtype=torch.int32, device=dev)
    db = torch.empty(20 * n, dtype=torch.float32, device=dev)
    torch.cuda.synchronize(dev)  # the uploads run on torch's stream, the bake on the context's
    check(lib().occ_occluders_bake_device(ctx.handle, n, dv.data_ptr(), _ptr(starts), _ptr(boxes), dp.data_ptr(),
                                          db.data_ptr()), "occ_occluders_bake_device")
    ctx.synchronize()
    packed = dp.cpu().numpy().view(np.uint32)
    bounds = db.cpu().numpy().reshape(n, 20)
    out = []
    for k in range(n):
        words = packed[starts[k]:starts[k + 1]].copy()
        b = bounds[k]
        out.append(Occluder(words, len(words) // 8, b[0:4].copy(), b[4:8].copy(), b[8:12].copy(), b[12:16].copy(),
                            b[16:20].copy()))
    return out


def load_mesh_bin(directory: str | None = None, vertex_path: str | None = None, index_path: str | None = None):
    """The reference demo's mesh files (Main.cpp:56-84): VertexBuffer.bin
    (float4 vertices) and IndexBuffer.bin (u32 triangle indices) in
    `directory`, or at the two paths given.  Returns (vertices (n, 4) float32,
    indices uint32)."""
    if directory is not None:
        vertex_path = vertex_path or os.path.join(directory, "VertexBuffer.bin")
        index_path = index_path or os.path.join(directory, "IndexBuffer.bin")
    if not vertex_path or not index_path:
        raise ValueError("give a directory or both file paths")
    vp, ip = os.fsencode(vertex_path), os.fsencode(index_path)
    nv, ni = C.c_uint32(), C.c_uint32()
    check(lib().occ_mesh_load_bin(vp, ip, None, C.byref(nv), None, C.byref(ni)), "occ_mesh_load_bin")
    v = np.zeros((max(nv.value, 1), 4), np.float32)
    i = np.zeros(max(ni.value, 1), np.uint32)
    check(lib().occ_mesh_load_bin(vp, ip, _ptr(v), C.byref(nv), _ptr(i), C.byref(ni)), "occ_mesh_load_bin")
    return v[:nv.value].copy(), i[:ni.value].copy()


def save_occluders(path: str, occluders: list[Occluder]) -> None:
    """Writes baked occluders to one file (versioned, hashed), so that a
    program can load them instead of baking again."""
    n = len(occluders)
    counts = np.array([o.packetCount for o in occluders], np.uint32)
    bufs = [np.ascontiguousarray(o.packed[:8 * o.packetCount], np.uint32) for o in occluders]
    ptrs = (C.c_void_p * max(n, 1))(*[b.ctypes.data for b in bufs])
    bounds = np.zeros((max(n, 1), 20), np.float32)
    for k, o in enumerate(occluders):
        bounds[k] = np.concatenate([o.refMin, o.refMax, o.boundsMin, o.boundsMax, o.center])
    check(lib().occ_occluders_save(os.fsencode(path), n, _ptr(counts), C.cast(ptrs, C.c_void_p), _ptr(bounds)),
          "occ_occluders_save")


def load_occluders(path: str) -> list[Occluder]:
    """Occluders written by save_occluders, in the same order."""
    p = os.fsencode(path)
    n, w = C.c_uint32(), C.c_uint64()
    check(lib().occ_occluders_file_info(p, C.byref(n), C.byref(w)), "occ_occluders_file_info")
    counts = np.zeros(max(n.value, 1), np.uint32)
    packed = np.zeros(max(w.value, 1), np.uint32)
    bounds = np.zeros((max(n.value, 1), 20), np.float32)
    check(lib().occ_occluders_load(p, n.value, w.value, _ptr(counts), _ptr(packed), _ptr(bounds)),
          "occ_occluders_load")
    out, pos = [], 0
    for k in range(n.value):
        c = int(counts[k])
        b = bounds[k]
        out.append(Occluder(packed[pos:pos + 8 * c].copy(), c, b[0:4].copy(), b[4:8].copy(), b[8:12].copy(),
                            b[12:16].copy(), b[16:20].copy()))
        pos += 8 * c
    return out


def _xmin(a, b):  # minps: the second operand unless a < b
    return np.where(a < b, a, b)


def _xmax(a, b):
    return np.where(a > b, a, b)


def _quad_boxes(corners: np.ndarray) -> np.ndarray:
    lo = np.full((len(corners), 4), np.inf, np.float32)
    hi = np.full((len(corners), 4), -np.inf, np.float32)
    for k in range(4):
        lo = _xmin(lo, corners[:, k])
        hi = _xmax(hi, corners[:, k])
    return np.ascontiguousarray(np.concatenate([lo, hi], axis=1), np.float32)


def _box_of(v: np.ndarray):
    """Running minps/maxps over the vertices in order (Main.cpp:109-113)."""
    if np.isnan(v).any():  # NaN makes the running result order dependent: replay it
        lo = np.full(4, np.inf, np.float32)
        hi = np.full(4, -np.inf, np.float32)
        for p in v:
            lo = _xmin(lo, p)
            hi = _xmax(hi, p)
        return lo.astype(np.float32), hi.astype(np.float32)
    lo = v.min(axis=0).astype(np.float32)
    hi = v.max(axis=0).astype(np.float32)
    # on a tie the running form keeps the later element: only the sign of zero can differ
    for res in (lo, hi):
        for a in range(4):
            if res[a] == 0 and len(v):
                zeros = np.nonzero(v[:, a] == 0)[0]
                res[a] = v[zeros[-1], a]
    return lo, hi


class Rasterizer:
    """Rasterizer (Rasterizer.h:10-61) on the GPU."""

    def __init__(self, ctx: Context, width: int, height: int):
        if width % 8 or height % 8 or width <= 0 or height <= 0:
            raise ValueError("width and height must be positive multiples of 8 (Rasterizer.cpp:68)")
        self.ctx = ctx
        self.width, self.height = width, height
        h = P()
        check(lib().occ_raster_create(ctx.handle, width, height, C.byref(h)), "occ_raster_create")
        self.handle = h.value
        ctx._adopt(self)

    def close(self):
        if getattr(self, "handle", None):
            if _context_open(self):
                lib().occ_raster_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def blocks(self) -> int:
        return (self.width // 8) * (self.height // 8)

    def setModelViewProjection(self, matrix) -> None:
        m = _f32(matrix).reshape(16)
        check(lib().occ_raster_set_mvp(self.handle, _ptr(m)), "occ_raster_set_mvp")

    def clear(self) -> None:
        check(lib().occ_raster_clear(self.handle), "occ_raster_clear")

    def rasterize(self, occluder: Occluder, possiblyNearClipped: bool) -> None:
        oid = occluder.upload(self.ctx)
        check(lib().occ_raster_rasterize(self.handle, oid, int(bool(possiblyNearClipped))), "occ_raster_rasterize")

    def rasterizeMany(self, occluders, flags=None) -> None:
        """Many rasterize calls; flags per occluder: 1 = near-clip variant,
        2 = decide visibility and variant on the GPU from the bounds."""
        ids = np.array([o.upload(self.ctx) for o in occluders], np.uint32)
        fl = None if flags is None else np.ascontiguousarray(flags, np.uint8)
        check(lib().occ_raster_rasterize_many(self.handle, len(ids), _ptr(ids), _ptr(fl)), "occ_raster_rasterize_many")

    def flush(self) -> None:
        check(lib().occ_raster_flush(self.handle), "occ_raster_flush")

    def commandFlags(self, n: int) -> np.ndarray:
        out = np.zeros(n, np.uint8)
        check(lib().occ_raster_command_flags(self.handle, n, _ptr(out)), "occ_raster_command_flags")
        return out

    def queryVisibility(self, boundsMin, boundsMax):
        """Rasterizer::queryVisibility -> (visible, needsClipping)."""
        a, b = _f32(boundsMin, (4,)), _f32(boundsMax, (4,))
        v, c = C.c_int(), C.c_int()
        check(lib().occ_raster_query_visibility(self.handle, _ptr(a), _ptr(b), C.byref(v), C.byref(c)),
              "occ_raster_query_visibility")
        return bool(v.value), bool(c.value)

    def queryVisibilityBatch(self, mins, maxs):
        """Many queryVisibility calls -> (visible bool[n], needsClipping bool[n])."""
        a, b = _f32(mins).reshape(-1, 4), _f32(maxs).reshape(-1, 4)
        n = len(a)
        vw = np.zeros((n + 31) // 32, np.uint32)
        nw = np.zeros((n + 31) // 32, np.uint32)
        check(lib().occ_raster_query_batch(self.handle, n, _ptr(a), _ptr(b), _ptr(vw), _ptr(nw)),
              "occ_raster_query_batch")
        return unpack_bits(vw, n), unpack_bits(nw, n)

    def query2D(self, minX, maxX, minY, maxY, maxZ) -> bool:
        v = C.c_int()
        check(lib().occ_raster_query2d(self.handle, minX, maxX, minY, maxY, maxZ, C.byref(v)), "occ_raster_query2d")
        return bool(v.value)

    def readBackDepth(self) -> np.ndarray:
        """Rasterizer::readBackDepth -> (height, width, 4) uint8."""
        out = np.zeros((self.height, self.width, 4), np.uint8)
        check(lib().occ_raster_read_back_depth(self.handle, _ptr(out)), "occ_raster_read_back_depth")
        return out

    def readBack(self, format: str = "rgba8") -> np.ndarray:
        """readBackDepth and its intermediate values, (height, width[, 4]):
        "rgba8" (the reference's bytes), "linear" (float linDepth), "depth"
        (float depth), "packed" (the u16 packed depth, block layout undone).
        Cleared blocks are 0."""
        kinds = {"rgba8": (0, np.uint8, 4), "linear": (1, np.float32, 1), "depth": (2, np.float32, 1),
                 "packed": (3, np.uint16, 1)}
        if format not in kinds:
            raise ValueError(f"unknown read-back format {format!r}")
        code, dt, ch = kinds[format]
        out = np.zeros((self.height, self.width, ch) if ch > 1 else (self.height, self.width), dt)
        check(lib().occ_raster_read_back(self.handle, code, _ptr(out)), "occ_raster_read_back")
        return out

    def readDepthRaw(self) -> np.ndarray:
        out = np.zeros(self.width * self.height, np.uint16)
        check(lib().occ_raster_read_depth_raw(self.handle, _ptr(out)), "occ_raster_read_depth_raw")
        return out

    def readHiZ(self) -> np.ndarray:
        n = C.c_uint32()
        check(lib().occ_raster_read_hiz(self.handle, None, C.byref(n)), "occ_raster_read_hiz")
        out = np.zeros(n.value, np.uint16)
        check(lib().occ_raster_read_hiz(self.handle, _ptr(out), C.byref(n)), "occ_raster_read_hiz")
        return out

    def writeDepthRaw(self, depth) -> None:
        d = np.ascontiguousarray(depth, np.uint16)
        check(lib().occ_raster_write_depth_raw(self.handle, _ptr(d)), "occ_raster_write_depth_raw")

    def writeHiZ(self, hiz) -> None:
        h = np.ascontiguousarray(hiz, np.uint16)
        check(lib().occ_raster_write_hiz(self.handle, _ptr(h)), "occ_raster_write_hiz")


class _WorkSet:
    """Keeps the numpy buffers of an occ_view_work array alive."""

    def __init__(self, ctx: Context, views: list[dict]):
        self.keep = []
        self.arr = (ViewWork * len(views))()
        self.nq = []
        self.ncmd = []
        for i, vw in enumerate(views):
            r: Rasterizer = vw["raster"]
            w = self.arr[i]
            w.raster = r.handle
            if vw.get("mvp") is not None:
                m = _f32(vw["mvp"]).reshape(16)
                self.keep.append(m)
                w.mvp = _ptr(m)
            w.clear = int(vw.get("clear", True))
            occs = vw.get("occluders", [])
            ids = np.array([o.upload(ctx) for o in occs], np.uint32)
            self.keep.append(ids)
            w.numOccluders = len(ids)
            w.occluders = _ptr(ids)
            self.ncmd.append(len(ids))
            if vw.get("flags") is not None:
                fl = np.ascontiguousarray(vw["flags"], np.uint8)
                self.keep.append(fl)
                w.flags = _ptr(fl)
            mins = vw.get("mins")
            n = 0 if mins is None else len(mins)
            self.nq.append(n)
            w.numQueries = n
            if n:
                a, b = _f32(vw["mins"]).reshape(-1, 4), _f32(vw["maxs"]).reshape(-1, 4)
                vb = np.zeros((n + 31) // 32, np.uint32)
                nb = np.zeros((n + 31) // 32, np.uint32)
                self.keep += [a, b, vb, nb]
                w.queryMins, w.queryMaxs = _ptr(a), _ptr(b)
                w.visibleBits, w.needsClippingBits = _ptr(vb), _ptr(nb)
                vw["_bits"] = (vb, nb)
        self.views = views


def execute_batch(ctx: Context, views: list[dict]):
    """Rasterise and query many views in one batch of kernels.  Each view is a
    dict: raster, mvp, clear, occluders, flags, mins, maxs.  Returns per view
    (visible bool[n], needsClipping bool[n])."""
    ws = _WorkSet(ctx, views)
    check(lib().occ_batch_execute(ctx.handle, len(views), ws.arr), "occ_batch_execute")
    out = []
    for vw, n in zip(views, ws.nq):
        if n:
            vb, nb = vw.pop("_bits")
            out.append((unpack_bits(vb, n), unpack_bits(nb, n)))
        else:
            out.append((np.zeros(0, bool), np.zeros(0, bool)))
    return out


class PreparedBatch:
    """occ_batch: tables and query boxes resident on the GPU, the frame's
    kernels captured in a CUDA graph; launch() is asynchronous."""

    def __init__(self, ctx: Context, views: list[dict]):
        self.ctx = ctx
        self.ws = _WorkSet(ctx, views)
        h = P()
        check(lib().occ_batch_prepare(ctx.handle, len(views), self.ws.arr, C.byref(h)), "occ_batch_prepare")
        self.handle = h.value
        ctx._adopt(self)

    def close(self):
        if getattr(self, "handle", None):
            if _context_open(self):
                lib().occ_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setModelViewProjection(self, view: int, matrix) -> None:
        m = _f32(matrix).reshape(16)
        check(lib().occ_batch_set_mvp(self.handle, view, _ptr(m)), "occ_batch_set_mvp")

    def setModelViewProjections(self, matrices, first: int = 0) -> None:
        """Matrices of views first, first+1, ... in one call ((n, 16) floats)."""
        m = _f32(matrices).reshape(-1, 16)
        check(lib().occ_batch_set_mvps(self.handle, first, len(m), _ptr(m)), "occ_batch_set_mvps")

    def launch(self) -> None:
        check(lib().occ_batch_launch(self.handle), "occ_batch_launch")

    def resultsAll(self, unpack: bool = False):
        """Every view's result bits in one copy: (visible words, needs-clipping
        words, first word of each view); with `unpack`, a list of per-view
        (visible, needsClipping) bool arrays."""
        if not hasattr(self, "_words"):
            w = C.c_uint32()
            check(lib().occ_batch_result_words(self.handle, C.byref(w)), "occ_batch_result_words")
            self._words = w.value
            self._vis = np.zeros(max(w.value, 1), np.uint32)
            self._nc = np.zeros(max(w.value, 1), np.uint32)
            self._first = np.zeros(len(self.ws.nq), np.uint32)
        check(lib().occ_batch_results_all(self.handle, _ptr(self._vis), _ptr(self._nc), _ptr(self._first)),
              "occ_batch_results_all")
        if not unpack:
            return self._vis, self._nc, self._first
        out = []
        for v, n in enumerate(self.ws.nq):
            a = int(self._first[v])
            nw = (n + 31) // 32
            out.append((unpack_bits(self._vis[a:a + nw], n), unpack_bits(self._nc[a:a + nw], n)))
        return out

    def resultsAllAsync(self, visible: np.ndarray, needsClipping: np.ndarray | None = None) -> None:
        """Queues the copy of every view's result bits into `visible` /
        `needsClipping` (uint32, resultWords() words; page-locked memory keeps
        it asynchronous) behind the launches queued so far; read them after
        ctx.synchronize()."""
        n = self.resultWords()
        for a in (visible, needsClipping):
            if a is not None and (a.dtype != np.uint32 or a.size < n or not a.flags.c_contiguous):
                raise ValueError(f"result buffers must be contiguous uint32 arrays of {n} words")
        check(lib().occ_batch_results_all_async(self.handle, _ptr(visible),
                                                None if needsClipping is None else _ptr(needsClipping)),
              "occ_batch_results_all_async")

    def resultWords(self) -> int:
        w = C.c_uint32()
        check(lib().occ_batch_result_words(self.handle, C.byref(w)), "occ_batch_result_words")
        return w.value

    def setQueries(self, mins, maxs, first: int = 0, count: int | None = None) -> None:
        """New query boxes for views first .. first+count-1 (each view's
        number of boxes, the views back to back: (n, 4) float32).  Queued on
        the context's stream ahead of the next launch: keep the arrays alive
        and unchanged until the stream has run the copies."""
        count = len(self.ws.nq) - first if count is None else count
        need = int(sum(self.ws.nq[first:first + count]))
        mins, maxs = _f32(mins).reshape(-1, 4), _f32(maxs).reshape(-1, 4)
        if len(mins) != need or len(maxs) != need:
            raise ValueError(f"expected {need} boxes for views {first}..{first + count - 1}")
        self._query_hold = (mins, maxs)  # kept alive until the next call
        check(lib().occ_batch_set_queries(self.handle, first, count, _ptr(mins), _ptr(maxs)), "occ_batch_set_queries")

    def check(self) -> bool:
        """True if every launch since the last check fitted the scratch; on
        False the batch has been re-sized and the frames must be re-run."""
        s = lib().occ_batch_check(self.handle)
        if s == 0:
            return True
        if s == -4:
            return False
        check(s, "occ_batch_check")
        return False

    def profile(self, iterations: int) -> np.ndarray:
        """Mean ms of (setup, scan, list fill, row walk, raster, query, selection)
        over `iterations` frames launched kernel by kernel with CUDA events in
        between (selection is 0 unless setSelection enabled it)."""
        out = np.zeros(7, np.float32)
        check(lib().occ_batch_profile(self.handle, iterations, _ptr(out)), "occ_batch_profile")
        return out

    def setSelection(self, mlp: "OccluderSelector | None", fraction: float = 1.0, trackWins: bool = False) -> None:
        """With `mlp`, each launch rasterises only the top ceil(fraction x
        candidates) occluders of every view by the network's score; with
        `trackWins`, each launch counts per occluder the pixels whose final
        depth it produced (read with selection())."""
        check(lib().occ_batch_set_selection(self.handle, mlp.handle if mlp is not None else None, float(fraction),
                                            int(bool(trackWins))), "occ_batch_set_selection")
        self._selector = mlp  # the captured launch reads the network's weights

    # occ_batch_autotune / occ_batch_set_tuning layout (OCC_TUNING_FIELDS entries)
    TUNING_KEYS = ("setup_ctas_per_sm", "fill_ctas_per_sm", "walk_ctas_per_sm", "raster_ctas_per_sm",
                   "raster_units_per_fetch", "query_rounds", "raster_unit_rows", "raster_threads_per_unit",
                   "super_tile_blocks")

    def autotune(self, iterations: int = 5) -> dict:
        """Picks the launch shapes of the persistent kernels by timing the
        batch's own frame stage by stage; returns the choice and the stage
        times before and after."""
        tuned = np.zeros(len(self.TUNING_KEYS), np.uint32)
        before = np.zeros(7, np.float32)
        after = np.zeros(7, np.float32)
        check(lib().occ_batch_autotune(self.handle, iterations, _ptr(tuned), _ptr(before), _ptr(after)),
              "occ_batch_autotune")
        names = ("setup", "scan", "fill", "walk", "raster", "query", "selection")
        return {"tuned": {k: int(v) for k, v in zip(self.TUNING_KEYS, tuned)},
                "ms_before": {k: float(v) for k, v in zip(names, before)},
                "ms_after": {k: float(v) for k, v in zip(names, after)}}

    def setTuning(self, tuned: dict) -> None:
        """Sets launch shapes directly (keys as `autotune()["tuned"]`; missing
        keys or 0: the default)."""
        t = np.array([int(tuned.get(k, 0)) for k in self.TUNING_KEYS], np.uint32)
        check(lib().occ_batch_set_tuning(self.handle, _ptr(t)), "occ_batch_set_tuning")

    def stats(self) -> dict:
        """Work counts of the last launch."""
        out = np.zeros(7, np.uint32)
        check(lib().occ_batch_stats(self.handle, _ptr(out)), "occ_batch_stats")
        keys = ("rows", "checkpoints", "list_entries", "active_chunks", "active_tiles", "chunks", "table_bytes")
        return {k: int(v) for k, v in zip(keys, out)}

    def setSecondPass(self, enable: bool) -> None:
        """After the top-K pass, also draw every other candidate whose bounds
        are still visible against that pass's buffer (needs a selector)."""
        check(lib().occ_batch_set_second_pass(self.handle, int(bool(enable))), "occ_batch_set_second_pass")

    def setCullLabels(self, enable: bool) -> None:
        """Per launch, credit each occluder with the sample pixels it owns in
        the screen rectangles of the boxes culled by depth (needs trackWins)."""
        check(lib().occ_batch_set_cull_labels(self.handle, int(bool(enable))), "occ_batch_set_cull_labels")

    def cullLabels(self, view: int) -> np.ndarray:
        n = self.ws.ncmd[view]
        out = np.zeros(n, np.uint32)
        if n:
            check(lib().occ_batch_read_cull_labels(self.handle, view, _ptr(out)), "occ_batch_read_cull_labels")
        return out

    def setZeroDepth(self, enable: bool) -> None:
        """Zero each cleared view's depth at the start of every launch, so a
        frame's queries do not see depth left by earlier frames in cleared
        blocks (which the reference's queryVisibility reads)."""
        check(lib().occ_batch_set_zero_depth(self.handle, int(bool(enable))), "occ_batch_set_zero_depth")

    def selection(self, view: int) -> dict:
        """Per occluder of `view` after the last launch: features (n x 16, the
        previous-launch wins among them), wins, candidate, selected (drawn by
        either pass), second_pass (drawn by the second pass), score."""
        n = self.ws.ncmd[view]
        out = dict(features=np.zeros((n, 16), np.float32), wins=np.zeros(n, np.uint32),
                   candidate=np.zeros(n, np.uint8), selected=np.zeros(n, np.uint8), score=np.zeros(n, np.float32))
        if n:
            check(lib().occ_batch_read_selection(self.handle, view, _ptr(out["features"]), _ptr(out["wins"]),
                                                 _ptr(out["candidate"]), _ptr(out["selected"]), _ptr(out["score"])),
                  "occ_batch_read_selection")
        out["candidate"] = out["candidate"].astype(bool)
        out["second_pass"] = out["selected"] == 2
        out["selected"] = out["selected"] != 0
        return out

    def results(self, view: int):
        n = self.ws.nq[view]
        vb = np.zeros(max((n + 31) // 32, 1), np.uint32)
        nb = np.zeros(max((n + 31) // 32, 1), np.uint32)
        check(lib().occ_batch_results(self.handle, view, _ptr(vb), _ptr(nb)), "occ_batch_results")
        return unpack_bits(vb, n), unpack_bits(nb, n)


class OccluderSelector:
    """The learned occluder selector: an MLP 16 -> 64 -> 64 -> 1 with ReLU
    (bf16 tensor-core inference, fp32 master weights, Adam), trained on the
    device.  Parameters are a flat float32 vector: W1 (64 x 16, row n holds the
    weights into hidden unit n), b1 (64), W2 (64 x 64, same), b2 (64), w3 (64), b3."""

    FEATURES = 16
    HIDDEN = 64

    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        h = P()
        check(lib().occ_mlp_create(ctx.handle, seed, C.byref(h)), "occ_mlp_create")
        self.handle = h.value
        ctx._adopt(self)
        self.nparams = lib().occ_mlp_param_count()

    def close(self):
        if getattr(self, "handle", None):
            if _context_open(self):
                lib().occ_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams, np.float32)
        check(lib().occ_mlp_get_params(self.handle, _ptr(out)), "occ_mlp_get_params")
        return out

    def setParams(self, p) -> None:
        p = _f32(p).reshape(self.nparams)
        check(lib().occ_mlp_set_params(self.handle, _ptr(p)), "occ_mlp_set_params")

    CHECKPOINT_VERSION = 1

    def save(self, path) -> None:
        """Weights and Adam state with a format header (resume with load)."""
        p = np.zeros(self.nparams, np.float32)
        m = np.zeros_like(p)
        v = np.zeros_like(p)
        step = C.c_uint32()
        check(lib().occ_mlp_get_state(self.handle, _ptr(p), _ptr(m), _ptr(v), C.byref(step)), "occ_mlp_get_state")
        header = np.array([self.CHECKPOINT_VERSION, self.FEATURES, self.HIDDEN, self.nparams, step.value], np.int64)
        with open(path, "wb") as f:
            np.savez(f, magic=np.frombuffer(b"OCCMLP", np.uint8), header=header, params=p, adam_m=m, adam_v=v)

    def load(self, path) -> None:
        with np.load(path) as z:
            if bytes(z["magic"]) != b"OCCMLP":
                raise ValueError(f"{path}: not an occluder-selector checkpoint")
            ver, feats, hidden, n, step = (int(x) for x in z["header"])
            if ver != self.CHECKPOINT_VERSION or feats != self.FEATURES or hidden != self.HIDDEN or n != self.nparams:
                raise ValueError(f"{path}: checkpoint version {ver} ({feats}-{hidden}, {n} params) does not match")
            p, m, v = (np.ascontiguousarray(z[k], np.float32) for k in ("params", "adam_m", "adam_v"))
        check(lib().occ_mlp_set_state(self.handle, _ptr(p), _ptr(m), _ptr(v), step), "occ_mlp_set_state")

    def forward(self, features) -> np.ndarray:
        x = _f32(features).reshape(-1, self.FEATURES)
        out = np.zeros(len(x), np.float32)
        check(lib().occ_mlp_forward(self.handle, len(x), _ptr(x), _ptr(out)), "occ_mlp_forward")
        return out

    def gradients(self, features, targets):
        x = _f32(features).reshape(-1, self.FEATURES)
        t = _f32(targets).reshape(len(x))
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        check(lib().occ_mlp_gradients(self.handle, len(x), _ptr(x), _ptr(t), C.byref(loss), _ptr(g)),
              "occ_mlp_gradients")
        return float(loss.value), g

    def gradientsListwise(self, features, targets, group_start):
        x = _f32(features).reshape(-1, self.FEATURES)
        t = _f32(targets).reshape(len(x))
        gs = np.ascontiguousarray(group_start, np.uint32)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        check(lib().occ_mlp_gradients_listwise(self.handle, len(x), _ptr(x), _ptr(t), len(gs) - 1, _ptr(gs),
                                               C.byref(loss), _ptr(g)), "occ_mlp_gradients_listwise")
        return float(loss.value), g

    def trainStepListwise(self, features, targets, group_start, lr: float = 1e-3) -> float:
        """One Adam step on the listwise loss: rows in groups (group_start[g]
        .. group_start[g+1]), targets a distribution within each group."""
        x = _f32(features).reshape(-1, self.FEATURES)
        t = _f32(targets).reshape(len(x))
        gs = np.ascontiguousarray(group_start, np.uint32)
        loss = C.c_float()
        check(lib().occ_mlp_train_step_listwise(self.handle, len(x), _ptr(x), _ptr(t), len(gs) - 1, _ptr(gs),
                                                float(lr), C.byref(loss)), "occ_mlp_train_step_listwise")
        return float(loss.value)

    def trainStep(self, features, targets, lr: float = 1e-3) -> float:
        x = _f32(features).reshape(-1, self.FEATURES)
        t = _f32(targets).reshape(len(x))
        loss = C.c_float()
        check(lib().occ_mlp_train_step(self.handle, len(x), _ptr(x), _ptr(t), float(lr), C.byref(loss)),
              "occ_mlp_train_step")
        return float(loss.value)


def coverage_table() -> np.ndarray:
    t = np.zeros(4096, np.int64)
    check(lib().occ_coverage_table(_ptr(t)), "occ_coverage_table")
    return t


def build_coverage_table() -> np.ndarray:
    t = np.zeros(4096, np.int64)
    check(lib().occ_build_coverage_table(_ptr(t)), "occ_build_coverage_table")
    return t


__all__ = ["Context", "Occluder", "QuadDecomposition", "SurfaceAreaHeuristic", "Rasterizer", "bake_scene",
           "execute_batch", "PreparedBatch", "OccluderSelector", "OccError", "coverage_table", "build_coverage_table", "unpack_bits"]
