"""Seeded synthetic scenes, camera matrices and query boxes.

The reference demo loads meshes from disk and builds its matrices with
DirectXMath (Main.cpp:56-84, Main.cpp:172-178).  The workloads here are
synthetic stand-ins with the shapes the benchmark configurations name:

* ``boxes_scene``   -- 64 axis-aligned boxes on a 200x200 ground quad (~770 tris)
* ``city_scene``    -- a grid of extruded buildings with tessellated facades
* ``query_boxes``   -- axis-aligned query boxes (float4 min/max, w = 1)
* ``camera_path``   -- a seeded Catmull-Rom street-level camera path

Vertex positions are snapped to multiples of 1/64 so that the same seed gives
the same float32 mesh on x86-64 and aarch64 hosts even if a transcendental
function differs in its last bit between the two.  Matrices follow the
reference's convention: row-vector, row-major ``float[16]`` as produced by
``XMMatrixLookToLH * XMMatrixPerspectiveFovLH`` (Main.cpp:172-178).
"""
from __future__ import annotations

import hashlib
import math
from dataclasses import dataclass

import numpy as np

SNAP = 64.0


def _snap(a: np.ndarray) -> np.ndarray:
    return (np.round(np.asarray(a, dtype=np.float64) * SNAP) / SNAP).astype(np.float32)


@dataclass
class Mesh:
    vertices: np.ndarray  # (N, 4) float32, w = 1
    indices: np.ndarray   # (3T,) uint32

    @property
    def triangles(self) -> int:
        return self.indices.size // 3

    def digest(self) -> str:
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(self.vertices, dtype=np.float32).tobytes())
        h.update(np.ascontiguousarray(self.indices, dtype=np.uint32).tobytes())
        return h.hexdigest()[:16]


class _MeshBuilder:
    def __init__(self) -> None:
        self.verts: list[np.ndarray] = []
        self.tris: list[np.ndarray] = []
        self.count = 0

    def add(self, verts: np.ndarray, tris: np.ndarray) -> None:
        self.verts.append(np.asarray(verts, dtype=np.float64))
        self.tris.append(np.asarray(tris, dtype=np.int64) + self.count)
        self.count += len(verts)

    def quad_grid(self, origin, du, dv, nu: int, nv: int) -> None:
        """A planar grid of nu x nv cells spanned by du, dv; two triangles per cell.
        Winding follows the cross product du x dv (clockwise seen from that side
        in the left-handed convention used here)."""
        origin = np.asarray(origin, np.float64)
        du = np.asarray(du, np.float64)
        dv = np.asarray(dv, np.float64)
        iu, iv = np.meshgrid(np.arange(nu + 1), np.arange(nv + 1), indexing="ij")
        pts = origin + (iu[..., None] / nu) * du + (iv[..., None] / nv) * dv
        pts = pts.reshape(-1, 3)
        idx = np.arange((nu + 1) * (nv + 1)).reshape(nu + 1, nv + 1)
        a = idx[:-1, :-1].ravel()
        b = idx[1:, :-1].ravel()
        c = idx[1:, 1:].ravel()
        d = idx[:-1, 1:].ravel()
        tris = np.stack([a, d, c, a, c, b], axis=1).reshape(-1, 3)
        self.add(pts, tris)

    def box(self, lo, hi, nseg=(1, 1, 1)) -> None:
        """Closed axis-aligned box, faces wound outward, each face a grid."""
        x0, y0, z0 = lo
        x1, y1, z1 = hi
        sx, sy, sz = nseg
        ex, ey, ez = x1 - x0, y1 - y0, z1 - z0
        # -z face (normal -z), +z face, -x, +x, +y (roof), -y (floor)
        self.quad_grid((x0, y0, z0), (0, ey, 0), (ex, 0, 0), sy, sx)
        self.quad_grid((x0, y0, z1), (ex, 0, 0), (0, ey, 0), sx, sy)
        self.quad_grid((x0, y0, z0), (0, 0, ez), (0, ey, 0), sz, sy)
        self.quad_grid((x1, y0, z0), (0, ey, 0), (0, 0, ez), sy, sz)
        self.quad_grid((x0, y1, z0), (0, 0, ez), (ex, 0, 0), 1, 1)
        self.quad_grid((x0, y0, z0), (ex, 0, 0), (0, 0, ez), 1, 1)

    def build(self) -> Mesh:
        v = np.concatenate(self.verts, axis=0)
        t = np.concatenate(self.tris, axis=0)
        verts = np.ones((len(v), 4), dtype=np.float32)
        verts[:, :3] = _snap(v)
        return Mesh(verts, t.astype(np.uint32).ravel())


def boxes_scene(seed: int = 42, nboxes: int = 64, footprint: float = 100.0, ground: float = 200.0) -> Mesh:
    """64 axis-aligned boxes (edge sizes U(0.5, 8)) placed uniformly in a
    footprint x footprint square resting on y = 0, plus a ground quad."""
    rng = np.random.default_rng(seed)
    mb = _MeshBuilder()
    half = footprint / 2
    for _ in range(nboxes):
        size = rng.uniform(0.5, 8.0, size=3)
        cx, cz = rng.uniform(-half, half, size=2)
        lo = (cx - size[0] / 2, 0.0, cz - size[2] / 2)
        hi = (cx + size[0] / 2, size[1], cz + size[2] / 2)
        mb.box(lo, hi)
    g = ground / 2
    mb.quad_grid((-g, 0.0, -g), (0, 0, ground), (ground, 0, 0), 1, 1)
    return mb.build()


def city_scene(seed: int = 1, grid: int = 64, cell: float = 16.0, target_tris: int = 260_000,
               mu: float = 2.5, sigma: float = 0.6) -> Mesh:
    """A grid x grid city of extruded buildings (footprints U(4, 12), heights
    lognormal(mu, sigma)), facades tessellated so the whole scene has about
    ``target_tris`` triangles, on a ground quad."""
    rng = np.random.default_rng(seed)
    fw = rng.uniform(4.0, 12.0, size=(grid, grid))
    fd = rng.uniform(4.0, 12.0, size=(grid, grid))
    h = np.clip(rng.lognormal(mu, sigma, size=(grid, grid)), 2.0, 150.0)
    jx = rng.uniform(-1.0, 1.0, size=(grid, grid))
    jz = rng.uniform(-1.0, 1.0, size=(grid, grid))
    # facade tessellation density chosen to hit the triangle target
    perim_area = (2 * (fw + fd) * h).sum()
    per_building_fixed = 4  # roof + floor
    budget = max(target_tris - per_building_fixed * grid * grid - 2, grid * grid * 8)
    cell_area = 2.0 * perim_area / budget  # two triangles per facade cell
    step = math.sqrt(cell_area)
    mb = _MeshBuilder()
    origin = -grid * cell / 2
    for i in range(grid):
        for j in range(grid):
            cx = origin + (i + 0.5) * cell + jx[i, j]
            cz = origin + (j + 0.5) * cell + jz[i, j]
            w, d, hh = fw[i, j], fd[i, j], h[i, j]
            nx = max(1, int(round(w / step)))
            nz = max(1, int(round(d / step)))
            ny = max(1, int(round(hh / step)))
            mb.box((cx - w / 2, 0.0, cz - d / 2), (cx + w / 2, hh, cz + d / 2), (nx, ny, nz))
    g = grid * cell
    mb.quad_grid((origin - cell, 0.0, origin - cell), (0, 0, g + 2 * cell), (g + 2 * cell, 0, 0), 1, 1)
    return mb.build()


def city_streets(grid: int = 64, cell: float = 16.0) -> np.ndarray:
    """Street centre-line coordinates (between building rows)."""
    origin = -grid * cell / 2
    return origin + np.arange(grid + 1) * cell


def query_boxes(n: int, seed: int, footprint: float = 100.0, ext_lo: float = 0.2, ext_hi: float = 2.0,
                lognormal: tuple[float, float] | None = None, y_range: tuple[float, float] = (0.0, 4.0)):
    """n axis-aligned query boxes as (mins, maxs), each (n, 4) float32 with w = 1.
    Centres uniform in the footprint; extents uniform(ext_lo, ext_hi) or lognormal."""
    rng = np.random.default_rng(seed)
    half = footprint / 2
    c = np.empty((n, 3))
    c[:, 0] = rng.uniform(-half, half, n)
    c[:, 2] = rng.uniform(-half, half, n)
    c[:, 1] = rng.uniform(y_range[0], y_range[1], n)
    if lognormal is None:
        e = rng.uniform(ext_lo, ext_hi, size=(n, 3))
    else:
        e = np.clip(rng.lognormal(lognormal[0], lognormal[1], size=(n, 3)), 0.05, 200.0)
    mins = np.ones((n, 4), np.float32)
    maxs = np.ones((n, 4), np.float32)
    mins[:, :3] = _snap(c - e / 2)
    maxs[:, :3] = _snap(c + e / 2)
    return mins, maxs


# ---- matrices -----------------------------------------------------------------

def perspective_fov_lh(fov_y: float, aspect: float, near: float, far: float) -> np.ndarray:
    """Left-handed perspective projection, row-vector convention (same layout as
    DirectXMath's XMMatrixPerspectiveFovLH, written from the formula)."""
    h = math.cos(0.5 * fov_y) / math.sin(0.5 * fov_y)
    w = h / aspect
    r = far / (far - near)
    return np.array([[w, 0, 0, 0], [0, h, 0, 0], [0, 0, r, 1], [0, 0, -r * near, 0]], dtype=np.float64)


def look_to_lh(eye, direction, up) -> np.ndarray:
    """Left-handed view matrix looking along ``direction`` (row-vector convention)."""
    eye = np.asarray(eye, np.float64)
    z = np.asarray(direction, np.float64)
    z = z / np.linalg.norm(z)
    x = np.cross(np.asarray(up, np.float64), z)
    x = x / np.linalg.norm(x)
    y = np.cross(z, x)
    m = np.eye(4)
    m[:3, 0] = x
    m[:3, 1] = y
    m[:3, 2] = z
    m[3, :3] = [-np.dot(x, eye), -np.dot(y, eye), -np.dot(z, eye)]
    return m


def view_projection(eye, direction, up=(0.0, 1.0, 0.0), fov_y: float = math.radians(60.0),
                    aspect: float = 16.0 / 9.0, near: float = 1.0, far: float = 5000.0) -> np.ndarray:
    """float[16] row-major model-view-projection, as Main.cpp:172-178 memcpy's it."""
    m = look_to_lh(eye, direction, up) @ perspective_fov_lh(fov_y, aspect, near, far)
    return np.ascontiguousarray(m.astype(np.float32).ravel())


def boxes_camera(width: int = 1920, height: int = 1080) -> np.ndarray:
    """The boxes scene's fixed camera: eye at height 1.7 in front of the
    footprint, looking along +z, 60 degree vertical field of view."""
    return view_projection((0.0, 1.7, -60.0), (0.0, 0.0, 1.0), aspect=width / height)


def camera_path(frames: int, seed: int, grid: int = 64, cell: float = 16.0, ctrl: int = 12,
                height: float = 1.7, width: int = 1920, height_px: int = 1080):
    """A seeded street-level Catmull-Rom camera path through the city.
    Returns (mvps (frames, 16) float32, eyes (frames, 4) float32)."""
    rng = np.random.default_rng(seed)
    streets = city_streets(grid, cell)
    # control points on street intersections near the city centre (random walk)
    i, j = grid // 2, grid // 2
    pts = []
    for _ in range(ctrl + 3):
        pts.append((streets[i], streets[j]))
        if rng.random() < 0.5:
            i = int(np.clip(i + rng.choice([-2, -1, 1, 2]), 1, grid - 1))
        else:
            j = int(np.clip(j + rng.choice([-2, -1, 1, 2]), 1, grid - 1))
    pts = np.asarray(pts, np.float64)
    out = np.empty((frames, 16), np.float32)
    eyes = np.ones((frames, 4), np.float32)
    aspect = width / height_px
    for f in range(frames):
        t = f / max(frames - 1, 1) * ctrl
        k = min(int(t), ctrl - 1)
        u = t - k
        p0, p1, p2, p3 = pts[k], pts[k + 1], pts[k + 2], pts[k + 3]
        pos = 0.5 * ((2 * p1) + (-p0 + p2) * u + (2 * p0 - 5 * p1 + 4 * p2 - p3) * u * u
                     + (-p0 + 3 * p1 - 3 * p2 + p3) * u ** 3)
        tan = 0.5 * ((-p0 + p2) + 2 * (2 * p0 - 5 * p1 + 4 * p2 - p3) * u
                     + 3 * (-p0 + 3 * p1 - 3 * p2 + p3) * u * u)
        if np.linalg.norm(tan) < 1e-6:
            tan = p2 - p1
        # sway the camera towards the facades so near-clipped occluders occur
        side = np.array([-tan[1], tan[0]]) / (np.linalg.norm(tan) + 1e-12)
        pos = pos + side * (3.5 * math.sin(0.37 * f))
        yaw = 0.6 * math.sin(0.11 * f + 1.0)
        c, s = math.cos(yaw), math.sin(yaw)
        d2 = np.array([c * tan[0] - s * tan[1], s * tan[0] + c * tan[1]])
        eye = (pos[0], height, pos[1])
        direction = (d2[0], -0.05, d2[1])
        out[f] = view_projection(eye, direction, aspect=aspect)
        eyes[f, :3] = eye
    return out, eyes


# ---- many views of one scene ----------------------------------------------------------

@dataclass
class ViewSpec:
    kind: str            # "cascade", "cube", "probe"
    width: int
    height: int
    mvp: np.ndarray      # float[16]
    eye: np.ndarray      # (3,)
    occluders: np.ndarray  # indices into the scene's occluder list, nearest first
    query_start: int
    query_count: int
    camera: dict = None  # view_projection arguments (eye, direction, up, fov_y, aspect, near)

    def moved(self, offset) -> np.ndarray:
        """The view's matrix with the eye displaced by `offset` (3,)."""
        cam = dict(self.camera)
        cam["eye"] = np.asarray(cam["eye"], np.float64) + np.asarray(offset, np.float64)
        return view_projection(**cam)


def view_track(spec: ViewSpec, frames: int, seed: int, speed: float = 0.6) -> np.ndarray:
    """(frames, 16) matrices of `spec` with its eye drifting horizontally
    `speed` units per frame along a seeded direction (frame 0 = spec.mvp)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0, 2 * math.pi)
    step = speed * np.array([math.cos(a), 0.0, math.sin(a)])
    return np.stack([spec.mvp if f == 0 else spec.moved(step * f) for f in range(frames)]).astype(np.float32)


def _pick_occluders(centers: np.ndarray, tris: np.ndarray, eye, budget: int) -> np.ndarray:
    """Occluders nearest to the eye until their triangles reach `budget` (>= 1)."""
    d = ((centers[:, :3] - np.asarray(eye)[None, :]) ** 2).sum(axis=1)
    order = np.argsort(d, kind="stable")
    total = np.cumsum(tris[order])
    n = int(np.searchsorted(total, budget) + 1)
    return order[:max(1, min(n, len(order)))].astype(np.uint32)


def multiview_workload(centers: np.ndarray, quads: np.ndarray, n_query_pool: int, seed: int = 3,
                       grid: int = 64, cell: float = 16.0, counts=(64, 96, 96)):
    """256 views of the city by default: `counts[0]` 1024x1024 shadow-cascade
    views (perspective spot views from above along one light direction),
    `counts[1]` 512x512 cube-map faces (groups of six around street-level
    probes), `counts[2]` probe views of random size (multiples of 8 between
    256x128 and 1920x1080).  Each view draws the occluders nearest to its eye
    up to a budget of 1k-200k triangles (a quad counts as two), and queries a
    contiguous range of 10k-100k boxes of the query pool."""
    rng = np.random.default_rng(seed)
    tris = 2 * np.asarray(quads, np.int64)
    half = grid * cell / 2
    streets = city_streets(grid, cell)
    views: list[ViewSpec] = []

    def queries():
        n = int(rng.integers(10_000, min(100_000, n_query_pool) + 1))
        start = int(rng.integers(0, n_query_pool - n + 1))
        return start, n

    light = np.array([0.35, -1.0, 0.25])
    light /= np.linalg.norm(light)
    for k in range(counts[0]):
        target = np.array([rng.uniform(-half * 0.6, half * 0.6), 0.0, rng.uniform(-half * 0.6, half * 0.6)])
        eye = target - light * 400.0
        cam = dict(eye=eye, direction=light, up=(0.0, 0.0, 1.0), fov_y=math.radians(25.0), aspect=1.0, near=1.0)
        mvp = view_projection(**cam)
        budget = int(rng.integers(1_000, 200_001))
        s, n = queries()
        views.append(ViewSpec("cascade", 1024, 1024, mvp, eye, _pick_occluders(centers, tris, eye, budget), s, n,
                              cam))
    faces = [((1, 0, 0), (0, 1, 0)), ((-1, 0, 0), (0, 1, 0)), ((0, 1, 0), (0, 0, -1)),
             ((0, -1, 0), (0, 0, 1)), ((0, 0, 1), (0, 1, 0)), ((0, 0, -1), (0, 1, 0))]
    for p in range((counts[1] + 5) // 6):
        eye = np.array([rng.choice(streets), 1.7 + rng.uniform(0, 6), rng.choice(streets)])
        budget = int(rng.integers(1_000, 200_001))
        occ = _pick_occluders(centers, tris, eye, budget)
        for d, up in faces:
            if len(views) >= counts[0] + counts[1]:
                break
            cam = dict(eye=eye, direction=d, up=up, fov_y=math.radians(90.0), aspect=1.0, near=0.5)
            mvp = view_projection(**cam)
            s, n = queries()
            views.append(ViewSpec("cube", 512, 512, mvp, eye, occ, s, n, cam))
    for k in range(counts[2]):
        w = int(rng.integers(32, 241)) * 8
        h = int(rng.integers(16, 136)) * 8
        eye = np.array([rng.choice(streets) + rng.uniform(-3, 3), 1.7, rng.choice(streets) + rng.uniform(-3, 3)])
        yaw = rng.uniform(0, 2 * math.pi)
        d = (math.cos(yaw), -0.05, math.sin(yaw))
        cam = dict(eye=eye, direction=d, fov_y=math.radians(60.0), aspect=w / h)
        mvp = view_projection(**cam)
        budget = int(rng.integers(1_000, 200_001))
        s, n = queries()
        views.append(ViewSpec("probe", w, h, mvp, eye, _pick_occluders(centers, tris, eye, budget), s, n, cam))
    return views


def large_workload(centers: np.ndarray, quads: np.ndarray, n_query_pool: int, seed: int = 5, frames: int = 1,
                   grid: int = 128, cell: float = 16.0):
    """The large combined workload over a grid x grid city: a 3840x2160
    street-level main view (a seeded camera path, `frames` frames) drawing
    every occluder and querying the whole pool, plus 63 auxiliary views of
    mixed resolution (16 cascades 1024x1024, 24 cube faces 512x512, 23 probe
    views) as in `multiview_workload`.  Returns (main mvps (frames, 16),
    auxiliary ViewSpecs)."""
    mvps, _ = camera_path(frames, seed=seed, grid=grid, cell=cell, width=3840, height_px=2160)
    aux = multiview_workload(centers, quads, n_query_pool, seed=seed, grid=grid, cell=cell, counts=(16, 24, 23))
    return mvps, aux
