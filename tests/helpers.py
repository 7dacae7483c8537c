"""Shared helpers of the parity tests: scenes, the oracle frame and the GPU frame."""
from __future__ import annotations

import functools

import numpy as np

from rasterizer_gb300 import api, scenes
from oracle.bindings import BakedScene, Oracle, aligned_u32


def to_baked(occluders: list[api.Occluder]) -> BakedScene:
    """The library's bake output in the oracle's plain-array form."""
    packed = []
    for o in occluders:
        buf = aligned_u32(o.packed.size)
        buf[:] = o.packed
        packed.append(buf)
    ref = np.stack([np.concatenate([o.refMin, o.refMax]) for o in occluders]).astype(np.float32)
    bounds = np.stack([np.concatenate([o.boundsMin, o.boundsMax]) for o in occluders]).astype(np.float32)
    centers = np.stack([o.center for o in occluders]).astype(np.float32)
    return BakedScene(packed, ref, bounds, centers)


@functools.lru_cache(maxsize=None)
def boxes_occluders():
    m = scenes.boxes_scene()
    return api.bake_scene(m.vertices, m.indices)


@functools.lru_cache(maxsize=None)
def city_occluders(grid: int = 64, target: int = 260_000):
    m = scenes.city_scene(grid=grid, target_tris=target)
    return api.bake_scene(m.vertices, m.indices)


@functools.lru_cache(maxsize=None)
def large_city_occluders():
    """The 2M-triangle city (128 x 128 buildings)."""
    return city_occluders(grid=128, target=2_000_000)


def canonical_depth(depth: np.ndarray, hiz: np.ndarray, blocks: int) -> np.ndarray:
    """Depth with cleared blocks (hiZ == 1) read as 0, as readBackDepth does."""
    d = depth.reshape(blocks, 64).copy()
    d[hiz[:blocks] == 1] = 0
    return d.ravel()


def gpu_plain_frame(r: api.Rasterizer, occluders, mvp):
    """The plain all-occluder frame on the GPU: clear, matrix, every occluder
    gated on the GPU from its bounds."""
    r.clear()
    r.setModelViewProjection(mvp)
    r.rasterizeMany(occluders, np.full(len(occluders), 2, np.uint8))
    r.flush()
    return r.commandFlags(len(occluders))


def mismatch_report(name, a, b) -> str:
    bad = np.nonzero(a != b)[0]
    if bad.size == 0:
        return ""
    i = bad[0]
    return f"{name}: {bad.size} mismatches, first at {i}: gpu {a[i]} oracle {b[i]}"


def special_boxes(n: int, seed: int, footprint: float = 100.0, nan: bool = True):
    """n query boxes, about half of them with one or two coordinates replaced
    by NaN (unless `nan` is off), infinities, huge, tiny or signed-zero values
    (and a few with w != 1): the x86 NaN and overflow rules of queryVisibility."""
    rng = np.random.default_rng(seed)
    mins, maxs = scenes.query_boxes(n, seed=seed, footprint=footprint)
    special = [np.inf, -np.inf, 1e30, -1e30, 3.4e38, -3.4e38, 1e-40, -0.0, 0.0, 2.0] + ([np.nan] if nan else [])
    special = np.array(special, np.float32)
    for i in range(n):
        if rng.random() < 0.5:
            for _ in range(int(rng.integers(1, 3))):
                which = mins if rng.random() < 0.5 else maxs
                which[i, int(rng.integers(0, 3))] = special[int(rng.integers(0, len(special)))]
        if rng.random() < 0.03:
            (mins if rng.random() < 0.5 else maxs)[i, 3] = special[int(rng.integers(0, len(special)))]
    return mins, maxs


def encode_linear(lin: np.ndarray) -> np.ndarray:
    """readBackDepth's bytes from its linear depth (Rasterizer.cpp:383-395):
    d = uint(25600 * lin), RGBA = (d / 100, d % 256, 0, 255); cleared pixels
    (packed depth 0 from a cleared block) are all zero.  (height, width, 4)."""
    s = np.float32(100 * 256) * lin.astype(np.float32)
    d = s.astype(np.uint64).astype(np.uint32)
    out = np.zeros(lin.shape + (4,), np.uint8)
    out[..., 0] = (d // 100).astype(np.uint8)
    out[..., 1] = (d % 256).astype(np.uint8)
    out[..., 3] = 255
    return out


def read_back_consistent(rgba: np.ndarray, lin: np.ndarray, depth: np.ndarray, packed: np.ndarray,
                         cleared: np.ndarray) -> list[str]:
    """The read-back formats agree with each other: bytes from linDepth,
    linDepth from depth, depth from the packed value; cleared pixels zero."""
    errs = []
    enc = encode_linear(lin)
    enc[cleared] = 0
    if not np.array_equal(enc, rgba.reshape(enc.shape)):
        errs.append("rgba8 != encode(linear)")
    d = (packed.astype(np.uint32) << 12).view(np.float32) * np.float32(3.9623753e+28)
    d[cleared] = 0
    if not np.array_equal(d, depth):
        errs.append("depth != packed << 12 * 1/bias")
    one, a, b, half = np.float32(1.0), np.float32(1000.25), np.float32(999.75), np.float32(0.5)
    l = half / (a - (one - depth) * b)
    l[cleared] = 0
    if not np.array_equal(l, lin):
        errs.append("linear != 0.5 / (1000.25 - (1 - depth) * 999.75)")
    return errs
