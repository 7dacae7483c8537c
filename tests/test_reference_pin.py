"""x86-64 only: the oracle and the library's host code against the reference
compiled from its own sources (oracle/_ref), on the reference's own meshes
(Castle, Sponza) and on randomised cameras.  Skipped where the reference
sources or an x86-64 host are missing (e.g. on the aarch64 GPU host)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import bindings
from oracle.bindings import Oracle, Reference, reference_bake_scene
from rasterizer_gb300 import api, scenes

from helpers import to_baked

pytestmark = pytest.mark.skipif(not bindings.reference_available(), reason="needs x86-64 and the reference sources")

MESHES = {
    # (camera eye, direction, up, vertical fov, width, height): the demo's poses (Main.cpp:28-40)
    "Castle": ((27.0, 2.0, 47.0), (0.142582759, 0.0611068942, -0.987894833), (0, 1, 0), 0.628, 1280, 720),
    "Sponza": ((0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0, 0, 1), 1.04, 1920, 1080),
}


def _mesh(name):
    d = os.path.join(bindings.REF_SOURCES, name)
    v = np.fromfile(os.path.join(d, "VertexBuffer.bin"), dtype=np.float32).reshape(-1, 4)
    i = np.fromfile(os.path.join(d, "IndexBuffer.bin"), dtype=np.uint32)
    return v, i


def test_mesh_loader_reads_the_reference_meshes():
    """load_mesh_bin reads the reference's own mesh files (Main.cpp:56-84) as
    the demo does: whole files, float4 vertices, u32 indices."""
    for name in MESHES:
        v, i = api.load_mesh_bin(os.path.join(bindings.REF_SOURCES, name))
        rv, ri = _mesh(name)
        assert np.array_equal(v.view(np.uint32), rv.view(np.uint32)) and np.array_equal(i, ri)


@pytest.fixture(scope="module", params=list(MESHES))
def mesh(request):
    v, i = _mesh(request.param)
    return request.param, v, i, reference_bake_scene(v, i)


def test_library_bake_byte_identical(mesh):
    name, v, i, ref = mesh
    mine = to_baked(api.bake_scene(v, i))
    assert len(mine) == len(ref)
    for k in range(len(ref)):
        assert np.array_equal(mine.packed[k], ref.packed[k]), f"{name} occluder {k} packed words"
        assert np.array_equal(mine.bounds[k].view(np.uint32), ref.bounds[k].view(np.uint32))
        assert np.array_equal(mine.centers[k].view(np.uint32), ref.centers[k].view(np.uint32))
        assert np.array_equal(mine.ref[k], ref.ref[k])


def test_decomposition_stage(mesh):
    name, v, i, _ = mesh
    L = bindings.ref_lib()
    out = np.zeros(4 * (i.size // 3), np.uint32)
    n = L.ref_decompose(bindings._ptr(i), i.size, bindings._ptr(v), len(v), bindings._ptr(out))
    assert np.array_equal(api.QuadDecomposition.decompose(i, v), out[:n])


def test_sah_stage():
    rng = np.random.default_rng(0)
    for n in (17, 100, 1000, 5000):
        lo = rng.normal(0, 50, size=(n, 4)).astype(np.float32)
        boxes = np.concatenate([lo, lo + rng.uniform(0, 5, size=(n, 4)).astype(np.float32)], axis=1)
        L = bindings.ref_lib()
        flat = np.zeros(n, np.uint32)
        offs = np.zeros(n + 1, np.uint32)
        nb = L.ref_sah(bindings._ptr(boxes), n, 512 if n > 600 else 40, 8, bindings._ptr(flat), bindings._ptr(offs))
        mine = api.SurfaceAreaHeuristic.generateBatches(boxes, 512 if n > 600 else 40, 8)
        assert len(mine) == nb
        for b in range(nb):
            assert np.array_equal(mine[b], flat[offs[b]:offs[b + 1]])


def _poses(name, count, seed):
    eye, d, up, fov, w, h = MESHES[name]
    rng = np.random.default_rng(seed)
    out = [scenes.view_projection(eye, d, up, fov_y=fov, aspect=w / h)]
    for _ in range(count):
        e = np.asarray(eye) + rng.normal(0, 3.0, 3)
        dd = np.asarray(d) + rng.normal(0, 0.6, 3)
        out.append(scenes.view_projection(e, dd, up, fov_y=fov, aspect=w / h))
    return out, w, h


def test_oracle_matches_reference_frames(mesh):
    """Plain frames, queries and read-back on a persistent rasterizer."""
    name, v, i, sc = mesh
    mvps, w, h = _poses(name, 5, 1)
    ref, scratch, orc = Reference(w, h), Reference(w, h), Oracle(w, h)
    mins, maxs = scenes.query_boxes(3000, seed=2, footprint=60.0 if name == "Sponza" else 250.0, y_range=(-10, 15))
    nc_total = 0
    for m in mvps:
        rf = ref.frame_plain_packed(scratch, sc, m)
        of = orc.frame_plain(sc, m)
        assert np.array_equal(rf, of)
        nc_total += int(((rf & 3) == 3).sum())
        assert np.array_equal(ref.depth(), orc.depth())
        assert np.array_equal(ref.hiz(), orc.hiz())
        rv, rn = ref.query(mins, maxs)
        ov, on = orc.query(mins, maxs)
        assert np.array_equal(rv, ov) and np.array_equal(rn, on)
        assert np.array_equal(ref.read_back(), orc.read_back())
    assert nc_total > 0


def test_forced_near_clip_variant():
    """rasterize<true> on every occluder (on Sponza it changes 2,348 pixels
    against rasterize<false>): the oracle must follow the variant."""
    v, i = _mesh("Sponza")
    sc = reference_bake_scene(v, i)
    eye, d, up, fov, w, h = MESHES["Sponza"]
    m = scenes.view_projection(eye, d, up, fov_y=fov, aspect=w / h)
    for nc in (False, True):
        ref, orc = Reference(w, h), Oracle(w, h)
        for o in (ref, orc):
            o.clear()
            o.set_mvp(m)
        for k in range(len(sc)):
            ref.rasterize(sc.packed[k], sc.packets[k], sc.ref[k, :4], sc.ref[k, 4:], nc)
            orc.rasterize(sc.packed[k], sc.packets[k], sc.ref[k, :4], sc.ref[k, 4:], nc)
        assert np.array_equal(ref.depth(), orc.depth())
        assert np.array_equal(ref.hiz(), orc.hiz())


def test_block_index_wrap_above_65535_blocks():
    """3840x2160 has 129,600 blocks: the reference's 16-bit product
    (Rasterizer.cpp:1054) is reproduced by the oracle's default mode."""
    v, i = _mesh("Castle")
    sc = reference_bake_scene(v, i)
    eye, d, up, fov, _, _ = MESHES["Castle"]
    m = scenes.view_projection(eye, d, up, fov_y=fov, aspect=3840 / 2160)
    ref, scratch, orc = Reference(3840, 2160), Reference(3840, 2160), Oracle(3840, 2160)
    ref.frame_plain_packed(scratch, sc, m)
    orc.frame_plain(sc, m)
    assert np.array_equal(ref.depth(), orc.depth())
    assert np.array_equal(ref.hiz(), orc.hiz())


def test_x86_tables_against_the_instruction():
    """RCPPS / RSQRTPS emulation rules on 2^24 sampled inputs per table."""
    src = os.path.join(os.path.dirname(api.__file__), "csrc", "gen_x86_tables.c")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "gen")
        subprocess.run(["gcc", "-O2", "-mavx2", src, "-o", exe], check=True)
        out = subprocess.run([exe, "--sample"], capture_output=True, text=True, check=True)
        header = open(os.path.join(os.path.dirname(src), "x86_tables.h")).read()
        assert out.stdout == header
        assert "mismatches 0" in out.stderr and "rsqrt mismatches 0" in out.stderr


def test_query_special_values_against_reference():
    """queryVisibility on boxes with infinite, huge, tiny and signed-zero
    coordinates (overflow to infinity and NaN from inf - inf inside the
    arithmetic): the oracle's x86 rules against the reference.  Boxes with NaN
    coordinates are left out here: which NaN an x86 add or multiply returns
    depends on its operand order, and the compiler may swap the operands of
    the reference's commutative intrinsics; the oracle and the GPU follow the
    source order (the first operand's NaN), and they agree on such boxes
    (tests/test_gpu_parity.py)."""
    from helpers import boxes_occluders, special_boxes
    scene = to_baked(boxes_occluders())
    mvp = scenes.view_projection((3.0, 2.0, -50.0), (0.0, -0.05, 1.0), aspect=640 / 360)
    ref, scratch, orc = Reference(640, 360), Reference(640, 360), Oracle(640, 360)
    ref.frame_plain_packed(scratch, scene, mvp)
    orc.frame_plain(scene, mvp)
    mins, maxs = special_boxes(8192, seed=61, nan=False)
    rvis, rnc = ref.query(mins, maxs)
    ovis, onc = orc.query(mins, maxs)
    assert np.array_equal(rvis, ovis) and np.array_equal(rnc, onc)
    assert rvis.sum() > 0 and (1 - rvis).sum() > 0


def _adversarial_mesh(kind: str, seed: int):
    rng = np.random.default_rng(seed)
    if kind == "grid":  # quads split either way, shuffled, some triangles wound the other way
        tris = []
        for y in range(9):
            for x in range(9):
                a, b, c, d = y * 10 + x, y * 10 + x + 1, (y + 1) * 10 + x + 1, (y + 1) * 10 + x
                tris += [(a, b, c), (a, c, d)] if rng.random() < 0.5 else [(a, b, d), (b, c, d)]
        v = np.zeros((100, 4), np.float32)
        v[:, 0], v[:, 2], v[:, 3] = np.arange(100) % 10, np.arange(100) // 10, 1
        v[:, 1] = np.round(rng.uniform(0, 0.8, 100) * 4) / 4
        tris = np.array(tris, np.uint32)
        rng.shuffle(tris)
        flip = rng.random(len(tris)) < 0.2
        tris[flip] = tris[flip][:, ::-1]
    else:  # non-manifold: edges shared by three or more triangles, duplicated triangles
        v = (np.round(rng.uniform(-5, 5, (12, 4)) * 4) / 4).astype(np.float32)
        v[:, 3] = 1
        tris = rng.integers(0, 12, (300, 3)).astype(np.uint32)
        tris = tris[(tris[:, 0] != tris[:, 1]) & (tris[:, 1] != tris[:, 2]) & (tris[:, 0] != tris[:, 2])]
        tris = np.concatenate([tris, tris[:40]])
    return v, np.ascontiguousarray(tris, np.uint32).ravel()


@pytest.mark.parametrize("kind", ["grid", "nonmanifold"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_decomposition_adversarial_meshes(kind, seed):
    """Shuffled triangle order, mixed windings, non-manifold edges and
    duplicated triangles: the same quads as the reference's decomposition."""
    v, i = _adversarial_mesh(kind, seed)
    L = bindings.ref_lib()
    out = np.zeros(4 * (i.size // 3), np.uint32)
    n = L.ref_decompose(bindings._ptr(i), i.size, bindings._ptr(v), len(v), bindings._ptr(out))
    assert np.array_equal(api.QuadDecomposition.decompose(i, v), out[:n])


def test_sah_tied_and_signed_zero_centres():
    """SAH on boxes whose centres tie (snapped) or are -0 and +0: the same
    batches as the reference (its stable sorts keep tied boxes in order)."""
    rng = np.random.default_rng(4)
    n = 6000
    lo = (np.round(rng.uniform(-50, 50, (n, 4)) / 8) * 8).astype(np.float32)
    hi = (lo + np.round(rng.uniform(0, 3, (n, 4)))).astype(np.float32)
    z = rng.integers(0, n, n // 10)
    lo[z[::2], 0] = hi[z[::2], 0] = -0.0
    lo[z[1::2], 0] = hi[z[1::2], 0] = 0.0
    boxes = np.ascontiguousarray(np.concatenate([lo, hi], axis=1), np.float32)
    L = bindings.ref_lib()
    flat, offs = np.zeros(n, np.uint32), np.zeros(n + 1, np.uint32)
    nb = L.ref_sah(bindings._ptr(boxes), n, 512, 8, bindings._ptr(flat), bindings._ptr(offs))
    mine = api.SurfaceAreaHeuristic.generateBatches(boxes, 512, 8)
    assert len(mine) == nb
    for b in range(nb):
        assert np.array_equal(mine[b], flat[offs[b]:offs[b + 1]])


def test_decomposition_random_meshes():
    """60 random small meshes (shared vertices, planar and non-planar, no
    repeated index within a triangle): the same quads as the reference."""
    L = bindings.ref_lib()
    for seed in range(60):
        rng = np.random.default_rng(1000 + seed)
        nv = int(rng.integers(4, 60))
        v = (np.round(rng.uniform(-3, 3, (nv, 4)) * 2) / 2).astype(np.float32)
        v[:, 3] = 1
        if seed % 2:
            v[:, 1] = 0  # planar: many mergeable pairs
        t = rng.integers(0, nv, (int(rng.integers(1, 200)), 3)).astype(np.uint32)
        t = t[(t[:, 0] != t[:, 1]) & (t[:, 1] != t[:, 2]) & (t[:, 0] != t[:, 2])]
        if not len(t):
            continue
        i = np.ascontiguousarray(t).ravel()
        out = np.zeros(4 * len(t), np.uint32)
        n = L.ref_decompose(bindings._ptr(i), i.size, bindings._ptr(v), nv, bindings._ptr(out))
        assert np.array_equal(api.QuadDecomposition.decompose(i, v), out[:n]), seed


def test_bake_random_and_special_vertex_sets():
    """100 random Occluder::bake inputs: degenerate quads, NaN / infinite /
    huge / subnormal / signed-zero coordinates, integral coordinates (ties in
    the bounds), a reference box of zero height: packed words, bounds and
    centre bit for bit as the reference's."""
    L = bindings.ref_lib()
    specials = np.array([np.nan, np.inf, -np.inf, -0.0, 0.0, 1e38, -1e38, 1e-40], np.float32)
    for seed in range(100):
        rng = np.random.default_rng(2000 + seed)
        nq = 8 * int(rng.integers(1, 40))
        v = rng.normal(0, 10, (4 * nq, 4)).astype(np.float32)
        v[:, 3] = 1
        mode = seed % 5
        if mode == 1:
            v[: 4 * (nq // 3)] = v[0]
        if mode == 2:
            k = rng.integers(0, len(v), 6)
            v[k, rng.integers(0, 3, 6)] = rng.choice(specials, 6)
        if mode == 3:
            v = np.round(v)
        lo = np.array([-20, -20, -20, 1], np.float32)
        hi = np.array([20, 20, 20, 1], np.float32)
        if mode == 4:
            hi[1] = lo[1]
        packed = np.zeros(len(v), np.uint32)
        bmin, bmax, ctr = (np.zeros(4, np.float32) for _ in range(3))
        pc = L.ref_bake(bindings._ptr(v), len(v), bindings._ptr(lo), bindings._ptr(hi), bindings._ptr(packed),
                        bindings._ptr(bmin), bindings._ptr(bmax), bindings._ptr(ctr))
        o = api.Occluder.bake(v, lo, hi)
        assert o.packetCount == pc and np.array_equal(o.packed[:8 * pc], packed[:8 * pc]), seed
        for mine, ref in ((o.boundsMin, bmin), (o.boundsMax, bmax), (o.center, ctr)):
            assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32)), seed


def test_gated_frame_loop_against_reference():
    """The oracle's restatement of Main.cpp's own frame loop (occluders front
    to back, each queried against the live buffer before it is drawn) against
    the reference's loop on its own bake (std::sort with the DPPS distance),
    on the city's street-level frames: same depth, hiZ and query bits."""
    from oracle.bindings import ReferenceScene
    c = scenes.city_scene()
    rs = ReferenceScene(c.vertices, c.indices)
    sc = reference_bake_scene(c.vertices, c.indices)
    mvps, eyes = scenes.camera_path(300, seed=7)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    ref, orc = Reference(1920, 1080), Oracle(1920, 1080)
    for f in (0, 77, 150, 299):
        rs.frame_gated(ref, mvps[f], eyes[f])
        orc.frame_gated(sc, mvps[f], eyes[f])
        assert np.array_equal(orc.depth(), ref.depth()), f
        assert np.array_equal(orc.hiz(), ref.hiz()), f
        v0, n0 = ref.query(mins, maxs)
        v1, n1 = orc.query(mins, maxs)
        assert np.array_equal(v0, v1) and np.array_equal(n0, n1), f
    rs.close()
