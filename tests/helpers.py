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
