"""ctypes bindings for the oracle libraries (test infrastructure only).

* ``Oracle``     -- the portable C restatement (oracle.c), any host.
* ``Reference``  -- the reference's own sources compiled here (oracle/_ref, x86-64
                    only); used to pin the restatement and the library's bake.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
# where the reference's sources lie; OCC_REF_DIR overrides the default
REF_SOURCES = os.environ.get("OCC_REF_DIR", "/root/reference/SoftwareRasterizer")

P = C.c_void_p
U32 = C.c_uint32


def _ptr(a):
    return None if a is None else a.ctypes.data_as(P)


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


def reference_available() -> bool:
    return platform.machine() in ("x86_64", "AMD64") and os.path.isdir(REF_SOURCES)


def build_reference() -> str | None:
    if not reference_available():
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_SOURCES}"], check=True)
    return REF_SO


_oracle_lib = None
_ref_lib = None


def oracle_lib():
    global _oracle_lib
    if _oracle_lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        lib = C.CDLL(ORACLE_SO)
        lib.orc_create.restype = P
        lib.orc_create.argtypes = [U32, U32, P]
        lib.orc_destroy.argtypes = [P]
        lib.orc_set_block_index_wrap.argtypes = [P, C.c_int]
        lib.orc_set_mvp.argtypes = [P, P]
        lib.orc_clear.argtypes = [P]
        lib.orc_rasterize.argtypes = [P, P, U32, P, P, C.c_int]
        lib.orc_query.argtypes = [P, P, P, P]
        lib.orc_query2d.argtypes = [P, U32, U32, U32, U32, U32]
        lib.orc_query_batch.argtypes = [P, U32, P, P, P, P]
        lib.orc_read_back.argtypes = [P, P]
        lib.orc_read_back_values.argtypes = [P, C.c_int, P]
        lib.orc_read_depth.argtypes = [P, P]
        lib.orc_read_hiz.argtypes = [P, P]
        lib.orc_read_hiz.restype = U32
        lib.orc_read_table.argtypes = [P, P]
        lib.orc_write_depth.argtypes = [P, P]
        lib.orc_write_hiz.argtypes = [P, P]
        lib.orc_read_counters.argtypes = [P, P]
        lib.orc_frame_plain.argtypes = [P, U32, P, P, P, P, P, P]
        lib.orc_frame_gated.argtypes = [P, U32, P, P, P, P, P, P, P, P, P]
        lib.orc_setup_dump.restype = U32
        lib.orc_setup_dump.argtypes = [P, P, U32, P, P, C.c_int, P]
        _oracle_lib = lib
    return _oracle_lib


def ref_lib():
    global _ref_lib
    if _ref_lib is None:
        if not os.path.exists(REF_SO):
            if build_reference() is None:
                raise RuntimeError("reference oracle needs x86-64 and the reference sources")
        lib = C.CDLL(REF_SO)
        lib.ref_decompose.restype = U32
        lib.ref_decompose.argtypes = [P, U32, P, U32, P]
        lib.ref_sah.restype = U32
        lib.ref_sah.argtypes = [P, U32, U32, U32, P, P]
        lib.ref_bake.restype = U32
        lib.ref_bake.argtypes = [P, U32, P, P, P, P, P, P]
        lib.ref_scene_build.restype = P
        lib.ref_scene_build.argtypes = [P, U32, P, U32]
        lib.ref_scene_count.restype = U32
        lib.ref_scene_count.argtypes = [P]
        lib.ref_scene_quad_indices.restype = U32
        lib.ref_scene_quad_indices.argtypes = [P, P]
        lib.ref_scene_batch.restype = U32
        lib.ref_scene_batch.argtypes = [P, U32, P]
        lib.ref_scene_occluder.restype = U32
        lib.ref_scene_occluder.argtypes = [P, U32, P, P, P, P, P, P]
        lib.ref_scene_free.argtypes = [P]
        lib.ref_raster_create.restype = P
        lib.ref_raster_create.argtypes = [U32, U32]
        lib.ref_raster_destroy.argtypes = [P]
        lib.ref_raster_set_mvp.argtypes = [P, P]
        lib.ref_raster_clear.argtypes = [P]
        lib.ref_raster_rasterize.argtypes = [P, P, U32, P, P, C.c_int]
        lib.ref_raster_rasterize_scene.argtypes = [P, P, U32, C.c_int]
        lib.ref_raster_query.restype = C.c_int
        lib.ref_raster_query.argtypes = [P, P, P, P]
        lib.ref_raster_query_batch.argtypes = [P, U32, P, P, P, P]
        lib.ref_raster_query2d.restype = C.c_int
        lib.ref_raster_query2d.argtypes = [P, U32, U32, U32, U32, U32]
        lib.ref_raster_read_depth.argtypes = [P, P]
        lib.ref_raster_read_hiz.restype = U32
        lib.ref_raster_read_hiz.argtypes = [P, P]
        lib.ref_raster_read_table.argtypes = [P, P]
        lib.ref_raster_read_back.argtypes = [P, P]
        lib.ref_frame_plain.argtypes = [P, P, P, P, U32, P, P]
        lib.ref_frame_gated.argtypes = [P, P, P, P]
        lib.ref_time_plain.restype = C.c_double
        lib.ref_time_plain.argtypes = [P, P, P, U32, P, U32, P, P, P, P]
        _ref_lib = lib
    return _ref_lib


class BakedScene:
    """Occluders as plain arrays: packed words, packet counts, ref/bounds boxes."""

    def __init__(self, packed: list[np.ndarray], ref: np.ndarray, bounds: np.ndarray, centers: np.ndarray):
        self.packed = packed            # list of uint32 arrays (packets*8 words), 32-byte aligned
        self.packets = np.array([p.size // 8 for p in packed], dtype=np.uint32)
        self.ref = np.ascontiguousarray(ref, np.float32)        # (n, 8): refMin4, refMax4
        self.bounds = np.ascontiguousarray(bounds, np.float32)  # (n, 8): boundsMin4, boundsMax4
        self.centers = np.ascontiguousarray(centers, np.float32)

    def __len__(self):
        return len(self.packed)

    @property
    def quads(self) -> int:
        return int(self.packets.sum()) * 2


def aligned_u32(n: int) -> np.ndarray:
    buf = np.zeros(n + 16, dtype=np.uint32)
    off = (-buf.ctypes.data % 32) // 4
    return buf[off:off + n]


def save_baked_scene(path, sc: "BakedScene") -> None:
    """A baked scene as one npz: the packed words back to back, per occluder
    packet counts, quantisation boxes, bounds and centres."""
    np.savez_compressed(path, packed=np.concatenate([p[:8 * int(k)] for p, k in zip(sc.packed, sc.packets)]),
                        packets=sc.packets, ref=sc.ref, bounds=sc.bounds, centers=sc.centers)


def load_baked_scene(path) -> "BakedScene":
    """The inverse of save_baked_scene (32-byte aligned packed arrays)."""
    z = np.load(path)
    packed, at = [], 0
    for k in z["packets"]:
        buf = aligned_u32(8 * int(k))
        buf[:] = z["packed"][at:at + 8 * int(k)]
        packed.append(buf)
        at += 8 * int(k)
    return BakedScene(packed, z["ref"], z["bounds"], z["centers"])


class Oracle:
    """One orc_raster (the portable restatement)."""

    def __init__(self, width: int, height: int, table: np.ndarray | None = None):
        self.lib = oracle_lib()
        self.width, self.height = width, height
        self.h = self.lib.orc_create(width, height, _ptr(table))
        if not self.h:
            raise ValueError("bad size")

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    __del__ = close

    def set_block_index_wrap(self, wrap: bool):
        self.lib.orc_set_block_index_wrap(self.h, int(wrap))

    def set_mvp(self, m):
        m = np.ascontiguousarray(m, np.float32)
        self.lib.orc_set_mvp(self.h, _ptr(m))

    def clear(self):
        self.lib.orc_clear(self.h)

    def rasterize(self, packed, packets, ref_min, ref_max, near_clip: bool):
        rmin = np.ascontiguousarray(ref_min, np.float32)
        rmax = np.ascontiguousarray(ref_max, np.float32)
        self.lib.orc_rasterize(self.h, _ptr(packed), int(packets), _ptr(rmin), _ptr(rmax), int(near_clip))

    def query(self, mins, maxs):
        n = len(mins)
        vis = np.zeros(n, np.uint8)
        nc = np.zeros(n, np.uint8)
        self.lib.orc_query_batch(self.h, n, _ptr(np.ascontiguousarray(mins, np.float32)),
                                 _ptr(np.ascontiguousarray(maxs, np.float32)), _ptr(vis), _ptr(nc))
        return vis, nc

    def depth(self):
        d = np.zeros(self.width * self.height, np.uint16)
        self.lib.orc_read_depth(self.h, _ptr(d))
        return d

    def hiz(self):
        h = np.zeros(self.lib.orc_read_hiz(self.h, None), np.uint16)
        self.lib.orc_read_hiz(self.h, _ptr(h))
        return h

    def table(self):
        t = np.zeros(4096, np.int64)
        self.lib.orc_read_table(self.h, _ptr(t))
        return t

    def read_back(self):
        out = np.zeros(self.width * self.height * 4, np.uint8)
        self.lib.orc_read_back(self.h, _ptr(out))
        return out

    def read_back_values(self, format: str):
        """(height, width) float linDepth ("linear"), float depth ("depth") or
        u16 packed depth ("packed"), row-major; 0 in cleared blocks."""
        code, dt = {"linear": (1, np.float32), "depth": (2, np.float32), "packed": (3, np.uint16)}[format]
        out = np.zeros((self.height, self.width), dt)
        self.lib.orc_read_back_values(self.h, code, _ptr(out))
        return out

    def write_depth(self, d):
        self.lib.orc_write_depth(self.h, _ptr(np.ascontiguousarray(d, np.uint16)))

    def write_hiz(self, h):
        self.lib.orc_write_hiz(self.h, _ptr(np.ascontiguousarray(h, np.uint16)))

    def counters(self):
        c = np.zeros(5, np.uint64)
        self.lib.orc_read_counters(self.h, _ptr(c))
        return c

    def setup_dump(self, packed, packets, ref_min, ref_max, near_clip: bool) -> np.ndarray:
        """(n, 6) int32: minX, minY, maxX, maxY, maxZ, mode of each valid quad."""
        out = np.zeros((int(packets) * 2, 6), np.int32)
        n = self.lib.orc_setup_dump(self.h, _ptr(packed), int(packets),
                                    _ptr(np.ascontiguousarray(ref_min, np.float32)),
                                    _ptr(np.ascontiguousarray(ref_max, np.float32)), int(near_clip), _ptr(out))
        return out[:n]

    def frame_gated(self, scene: BakedScene, mvp, eye):
        """Main.cpp:181-206: occluders front to back by squared centre distance
        to `eye`, each queried against the live buffer before it is drawn.
        Returns (drawing order, per-occluder flags visible | nearClip << 1)."""
        n = len(scene)
        ptrs = (P * n)(*[scene.packed[i].ctypes.data for i in range(n)])
        packets = np.ascontiguousarray(scene.packets, np.uint32)
        order = np.zeros(n, np.uint32)
        flags = np.zeros(n, np.uint8)
        e = np.zeros(4, np.float32)
        e[:3] = np.asarray(eye, np.float32)[:3]
        self.lib.orc_frame_gated(self.h, n, C.cast(ptrs, P), _ptr(packets), _ptr(np.ascontiguousarray(scene.ref)),
                                 _ptr(np.ascontiguousarray(scene.bounds)),
                                 _ptr(np.ascontiguousarray(scene.centers, np.float32)), _ptr(e),
                                 _ptr(np.ascontiguousarray(mvp, np.float32)), _ptr(order), _ptr(flags))
        return order, flags

    def frame_plain(self, scene: BakedScene, mvp, order=None):
        idx = np.arange(len(scene)) if order is None else np.asarray(order)
        ptrs = (P * len(idx))(*[scene.packed[i].ctypes.data for i in idx])
        packets = np.ascontiguousarray(scene.packets[idx], np.uint32)
        ref = np.ascontiguousarray(scene.ref[idx])
        bounds = np.ascontiguousarray(scene.bounds[idx])
        flags = np.zeros(len(idx), np.uint8)
        m = np.ascontiguousarray(mvp, np.float32)
        self.lib.orc_frame_plain(self.h, len(idx), C.cast(ptrs, P), _ptr(packets), _ptr(ref), _ptr(bounds),
                                 _ptr(m), _ptr(flags))
        return flags


class Reference:
    """One reference Rasterizer compiled from the reference's sources (x86-64)."""

    def __init__(self, width: int, height: int):
        self.lib = ref_lib()
        self.width, self.height = width, height
        self.h = self.lib.ref_raster_create(width, height)

    def close(self):
        if self.h:
            self.lib.ref_raster_destroy(self.h)
            self.h = None

    __del__ = close

    def set_mvp(self, m):
        self.lib.ref_raster_set_mvp(self.h, _ptr(np.ascontiguousarray(m, np.float32)))

    def clear(self):
        self.lib.ref_raster_clear(self.h)

    def rasterize(self, packed, packets, ref_min, ref_max, near_clip: bool):
        self.lib.ref_raster_rasterize(self.h, _ptr(packed), int(packets),
                                      _ptr(np.ascontiguousarray(ref_min, np.float32)),
                                      _ptr(np.ascontiguousarray(ref_max, np.float32)), int(near_clip))

    def query(self, mins, maxs):
        n = len(mins)
        vis = np.zeros(n, np.uint8)
        nc = np.zeros(n, np.uint8)
        self.lib.ref_raster_query_batch(self.h, n, _ptr(np.ascontiguousarray(mins, np.float32)),
                                        _ptr(np.ascontiguousarray(maxs, np.float32)), _ptr(vis), _ptr(nc))
        return vis, nc

    def depth(self):
        d = np.zeros(self.width * self.height, np.uint16)
        self.lib.ref_raster_read_depth(self.h, _ptr(d))
        return d

    def hiz(self):
        h = np.zeros(self.lib.ref_raster_read_hiz(self.h, None), np.uint16)
        self.lib.ref_raster_read_hiz(self.h, _ptr(h))
        return h

    def table(self):
        t = np.zeros(4096, np.int64)
        self.lib.ref_raster_read_table(self.h, _ptr(t))
        return t

    def read_back(self):
        out = np.zeros(self.width * self.height * 4, np.uint8)
        self.lib.ref_raster_read_back(self.h, _ptr(out))
        return out

    def frame_plain_packed(self, scratch: "Reference", scene: BakedScene, mvp, order=None):
        """The parity-mode loop over arbitrary packed occluders (same as orc_frame_plain)."""
        idx = range(len(scene)) if order is None else order
        self.clear()
        self.set_mvp(mvp)
        scratch.set_mvp(mvp)
        flags = np.zeros(len(idx), np.uint8)
        for k, i in enumerate(idx):
            v, c = scratch.query(scene.bounds[i:i + 1, :4], scene.bounds[i:i + 1, 4:])
            flags[k] = int(v[0]) | (int(c[0]) << 1)
            if v[0]:
                self.rasterize(scene.packed[i], scene.packets[i], scene.ref[i, :4], scene.ref[i, 4:], bool(c[0]))
        return flags


class ReferenceScene:
    """A scene baked and held by the reference's own code (Main.cpp:86-128),
    drawn by its frame loops (x86-64)."""

    def __init__(self, vertices: np.ndarray, indices: np.ndarray):
        self.lib = ref_lib()
        v = np.ascontiguousarray(vertices, np.float32)
        i = np.ascontiguousarray(indices, np.uint32)
        self.h = self.lib.ref_scene_build(_ptr(i), i.size, _ptr(v), len(v))

    def close(self):
        if self.h:
            self.lib.ref_scene_free(self.h)
            self.h = None

    __del__ = close

    def __len__(self):
        return self.lib.ref_scene_count(self.h)

    def frame_plain(self, r: "Reference", scratch: "Reference", mvp):
        self.lib.ref_frame_plain(r.h, scratch.h, self.h, None, len(self), _ptr(np.ascontiguousarray(mvp, np.float32)),
                                 None)

    def frame_gated(self, r: "Reference", mvp, eye):
        e = np.zeros(4, np.float32)
        e[:3] = np.asarray(eye, np.float32)[:3]
        self.lib.ref_frame_gated(r.h, self.h, _ptr(np.ascontiguousarray(mvp, np.float32)), _ptr(e))


def reference_bake_scene(vertices: np.ndarray, indices: np.ndarray) -> BakedScene:
    """Scene baked by the reference's own pipeline (Main.cpp:86-128)."""
    lib = ref_lib()
    v = np.ascontiguousarray(vertices, np.float32)
    i = np.ascontiguousarray(indices, np.uint32)
    s = lib.ref_scene_build(_ptr(i), i.size, _ptr(v), len(v))
    try:
        n = lib.ref_scene_count(s)
        packed, ref, bounds, centers = [], np.zeros((n, 8), np.float32), np.zeros((n, 8), np.float32), np.zeros((n, 4), np.float32)
        for k in range(n):
            pk = lib.ref_scene_occluder(s, k, None, None, None, None, None, None)
            buf = aligned_u32(pk * 8)
            rmin = np.zeros(4, np.float32); rmax = np.zeros(4, np.float32)
            bmin = np.zeros(4, np.float32); bmax = np.zeros(4, np.float32); c = np.zeros(4, np.float32)
            lib.ref_scene_occluder(s, k, _ptr(buf), _ptr(rmin), _ptr(rmax), _ptr(bmin), _ptr(bmax), _ptr(c))
            packed.append(buf)
            ref[k, :4], ref[k, 4:] = rmin, rmax
            bounds[k, :4], bounds[k, 4:] = bmin, bmax
            centers[k] = c
        return BakedScene(packed, ref, bounds, centers)
    finally:
        lib.ref_scene_free(s)
