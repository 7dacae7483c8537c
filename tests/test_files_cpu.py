"""Host-side files: the reference demo's mesh files and the baked occluder
file (round trip bit for bit, refusal of damaged files), through the Python
mirror and through the C++ facade.  No GPU."""
import os
import subprocess

import numpy as np
import pytest

from rasterizer_gb300 import api, scenes
from rasterizer_gb300._lib import OccError

from helpers import boxes_occluders

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OCC_ERR_IO = -6


def _same(a: api.Occluder, b: api.Occluder) -> bool:
    return (a.packetCount == b.packetCount and np.array_equal(a.packed[:8 * a.packetCount], b.packed)
            and all(np.array_equal(getattr(a, f).view(np.uint32), getattr(b, f).view(np.uint32))
                    for f in ("refMin", "refMax", "boundsMin", "boundsMax", "center")))


def test_baked_file_round_trip(tmp_path):
    occ = boxes_occluders()
    path = str(tmp_path / "boxes.occ")
    api.save_occluders(path, occ)
    assert not os.path.exists(path + ".part")
    back = api.load_occluders(path)
    assert len(back) == len(occ) and all(_same(a, b) for a, b in zip(occ, back))
    # a loaded scene bakes nothing: the file holds exactly the packed words and bounds
    words = sum(8 * o.packetCount for o in occ)
    assert os.path.getsize(path) == 24 + 96 * len(occ) + 4 * words + 8


def test_baked_file_empty_scene(tmp_path):
    path = str(tmp_path / "empty.occ")
    api.save_occluders(path, [])
    assert api.load_occluders(path) == []


@pytest.mark.parametrize("damage", ["flip", "truncate", "magic", "version", "extend"])
def test_baked_file_damaged_is_refused(tmp_path, damage):
    occ = boxes_occluders()
    path = str(tmp_path / "boxes.occ")
    api.save_occluders(path, occ)
    raw = bytearray(open(path, "rb").read())
    if damage == "flip":
        raw[len(raw) // 2] ^= 0x10
    elif damage == "truncate":
        raw = raw[:-9]
    elif damage == "magic":
        raw[0:8] = b"NOTOCCLU"
    elif damage == "version":
        raw[8] = 2
    else:
        raw += b"\0" * 4
    open(path, "wb").write(bytes(raw))
    with pytest.raises(OccError) as e:
        api.load_occluders(path)
    assert e.value.status == OCC_ERR_IO


def test_missing_file_is_refused(tmp_path):
    with pytest.raises(OccError):
        api.load_occluders(str(tmp_path / "none.occ"))
    with pytest.raises(OccError):
        api.load_mesh_bin(str(tmp_path))


def test_mesh_bin_round_trip(tmp_path):
    mesh = scenes.boxes_scene()
    v = np.ascontiguousarray(mesh.vertices, np.float32).reshape(-1, 4)
    i = np.ascontiguousarray(mesh.indices, np.uint32)
    v.tofile(str(tmp_path / "VertexBuffer.bin"))
    i.tofile(str(tmp_path / "IndexBuffer.bin"))
    lv, li = api.load_mesh_bin(str(tmp_path))
    assert np.array_equal(lv.view(np.uint32), v.view(np.uint32)) and np.array_equal(li, i)
    # the loaded mesh bakes to the same occluders
    a, b = api.bake_scene(v, i), api.bake_scene(lv, li)
    assert len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))


def test_mesh_bin_ragged_is_refused(tmp_path):
    np.zeros((4, 4), np.float32).tofile(str(tmp_path / "VertexBuffer.bin"))
    open(str(tmp_path / "IndexBuffer.bin"), "wb").write(b"\0" * 7)
    with pytest.raises(OccError):
        api.load_mesh_bin(str(tmp_path))


FACADE_FILES = r"""
#include "rasterizer_gb300/Rasterizer.hpp"
#include <cstdio>
// Host only: mesh files -> the demo's scene preparation -> file -> load.
int main(int argc, char** argv) {
  std::vector<gb300::Vec4> v;
  std::vector<uint32_t> idx;
  gb300::loadMeshBin(argv[1], v, idx);
  auto occ = gb300::bakeScene(v, idx);
  gb300::saveOccluders(argv[2], occ);
  auto back = gb300::loadOccluders(argv[2]);
  if (back.size() != occ.size()) return 2;
  for (size_t k = 0; k < occ.size(); ++k)
    if (back[k]->m_packetCount != occ[k]->m_packetCount || back[k]->m_vertexData != occ[k]->m_vertexData ||
        std::memcmp(back[k]->m_boundsMin.v, occ[k]->m_boundsMin.v, 16) || std::memcmp(back[k]->m_center.v, occ[k]->m_center.v, 16))
      return 3;
  // the same occluders as baking in steps: print the words for the caller to compare
  for (auto& o : occ)
    for (uint32_t w : o->m_vertexData) std::printf("%u\n", w);
  return 0;
}
"""


def test_cpp_facade_files(tmp_path):
    so = os.path.join(ROOT, "rasterizer_gb300", "lib", "librasterizer_gb300.so")
    if not os.path.exists(so):
        pytest.skip("library not built")
    mesh = scenes.boxes_scene()
    np.ascontiguousarray(mesh.vertices, np.float32).reshape(-1, 4).tofile(str(tmp_path / "VertexBuffer.bin"))
    np.ascontiguousarray(mesh.indices, np.uint32).tofile(str(tmp_path / "IndexBuffer.bin"))
    src, exe = str(tmp_path / "t.cpp"), str(tmp_path / "t")
    open(src, "w").write(FACADE_FILES)
    subprocess.run(["g++", "-std=c++17", "-O0", "-I" + os.path.join(ROOT, "include"), src, "-o", exe, so,
                    "-Wl,-rpath," + os.path.dirname(so)], check=True)
    r = subprocess.run([exe, str(tmp_path), str(tmp_path / "scene.occ")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    words = np.array([int(x) for x in r.stdout.split()], np.uint32)
    want = np.concatenate([o.packed[:8 * o.packetCount] for o in api.bake_scene(mesh.vertices, mesh.indices)])
    assert np.array_equal(words, want)


def test_scene_bake_in_one_call_equals_the_steps():
    """occ_scene_bake (the demo's preparation natively) gives the bytes of
    decompose -> pad -> boxes -> SAH -> Occluder::bake per batch; empty
    meshes give no occluders; bad indices and short buffers are refused."""
    import ctypes as C
    from rasterizer_gb300._lib import lib
    for mesh in (scenes.boxes_scene(), scenes.city_scene(grid=16, target_tris=20_000)):
        sets, lo, hi = api.scene_batches(mesh.vertices, mesh.indices)
        want = [api.Occluder.bake(s, lo, hi) for s in sets]
        got = api.bake_scene(mesh.vertices, mesh.indices)
        assert len(got) == len(want) and all(_same(a, b) for a, b in zip(got, want))
    assert api.bake_scene(np.zeros((0, 4), np.float32), np.zeros(0, np.uint32)) == []
    v = np.zeros((4, 4), np.float32)
    n, w = C.c_uint32(), C.c_uint64()
    bad = np.array([0, 1, 9], np.uint32)
    assert lib().occ_scene_bake(v.ctypes.data, 4, bad.ctypes.data, 3, 512, 8, 0, 0, C.byref(n), C.byref(w),
                                None, None, None) == -1
    mesh = scenes.boxes_scene()
    vv = np.ascontiguousarray(mesh.vertices, np.float32).reshape(-1, 4)
    ii = np.ascontiguousarray(mesh.indices, np.uint32)
    assert lib().occ_scene_bake(vv.ctypes.data, len(vv), ii.ctypes.data, ii.size, 512, 8, 0, 0, C.byref(n),
                                C.byref(w), None, None, None) == 0 and n.value >= 1
    counts, packed, bounds = np.zeros(1, np.uint32), np.zeros(8, np.uint32), np.zeros(20, np.float32)
    assert lib().occ_scene_bake(vv.ctypes.data, len(vv), ii.ctypes.data, ii.size, 512, 8, 1, 8, C.byref(n),
                                C.byref(w), counts.ctypes.data, packed.ctypes.data, bounds.ctypes.data) == -4
