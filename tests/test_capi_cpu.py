"""C ABI checks that need no GPU: the library loads, exports every function
include/rasterizer_gb300.h declares, validates arguments, and its host-side
routines (bake, tables) run."""
import ctypes as C
import os
import re
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from rasterizer_gb300 import _lib, api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rasterizer_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(occ_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    names = declared_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python bindings declare a signature for each of them
    assert not [n for n in names if n not in _lib.SIGNATURES]


def test_version_and_tables():
    lib = _lib.lib()
    assert lib.occ_version() == 1
    t = api.coverage_table()
    # for each slope the first offset entry is all ones, the last all zero (Rasterizer.cpp:592-602)
    slopes = set(i >> 6 for i in range(4096) if t[i] != 0)
    for s in slopes:
        assert t[s << 6] == -1
        assert t[(s << 6) | 63] == 0


def test_bake_argument_validation():
    lib = _lib.lib()
    idx = np.arange(4, dtype=np.uint32)
    v = np.zeros((4, 4), np.float32)
    out = np.zeros(16, np.uint32)
    n = C.c_uint32()
    assert lib.occ_quad_decompose(idx.ctypes.data, 4, v.ctypes.data, 4, out.ctypes.data, C.byref(n)) == -1
    idx3 = np.array([0, 1, 9], np.uint32)  # vertex index out of range
    assert lib.occ_quad_decompose(idx3.ctypes.data, 3, v.ctypes.data, 4, out.ctypes.data, C.byref(n)) == -1
    with pytest.raises(ValueError):
        api.Occluder.bake(np.zeros((15, 4), np.float32), np.zeros(4), np.ones(4))
    # 16 vertices pass the reference's assert but its packing reads 32
    with pytest.raises(ValueError):
        api.Occluder.bake(np.zeros((16, 4), np.float32), np.zeros(4), np.ones(4))
    packed, pc = np.zeros(16, np.uint32), C.c_uint32()
    z, o = np.zeros(4, np.float32), np.ones(4, np.float32)
    assert lib.occ_occluder_bake(np.zeros((16, 4), np.float32).ctypes.data, 16, z.ctypes.data, o.ctypes.data,
                                 packed.ctypes.data, C.byref(pc), z.ctypes.data, z.ctypes.data, z.ctypes.data) == -1


def test_sah_small_inputs_form_one_batch():
    """The reference's split search needs more than two granules (its unsigned
    loop bound); 16 quads or fewer stay one batch."""
    boxes = np.zeros((16, 8), np.float32)
    boxes[:, 4:] = 1
    b = api.SurfaceAreaHeuristic.generateBatches(boxes, 512, 8)
    assert len(b) == 1 and np.array_equal(b[0], np.arange(16))


def test_rasterizer_size_validation_is_host_side():
    with pytest.raises(ValueError):
        api.Rasterizer(None, 100, 64)  # not a multiple of 8: rejected before touching a GPU


def test_cpp_facade_compiles():
    src = '#include "rasterizer_gb300/Rasterizer.hpp"\nint main() { return 0; }\n'
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        open(p, "w").write(src)
        subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"), p], check=True)


FACADE_PROGRAM = r"""
#include "rasterizer_gb300/Rasterizer.hpp"
// The demo's frame loop with the learned selector, through the facade only
// (built and linked here; it needs a GPU to run).
int run(int argc) {
  gb300::Context ctx(0);
  gb300::Rasterizer raster(ctx, 1920, 1080);
  std::vector<gb300::Vec4> verts(32, gb300::Vec4{{0, 0, 0, 1}});
  auto occ = gb300::Occluder::bake(verts, gb300::Vec4{{0, 0, 0, 1}}, gb300::Vec4{{1, 1, 1, 1}});
  float mvp[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0};
  gb300::Batch::View v{&raster, mvp, {occ.get()}, {OCC_GATED}, {gb300::Vec4{{0, 0, 5, 1}}}, {gb300::Vec4{{1, 1, 6, 1}}}};
  gb300::Batch batch(ctx, {v});
  gb300::OccluderSelector sel(ctx, 1);
  batch.setSelection(&sel, 0.35f);
  batch.autotune(2);
  batch.launch();
  std::vector<uint32_t> vis, nc;
  batch.check_capacity();
  batch.results(0, vis, nc);
  raster.clear();
  raster.setModelViewProjection(mvp);
  bool needsClipping = false;
  if (raster.queryVisibility(occ->m_boundsMin, occ->m_boundsMax, needsClipping))
    needsClipping ? raster.rasterize<true>(*occ) : raster.rasterize<false>(*occ);
  return (int)vis.size() + argc;
}
int main(int argc, char**) { return argc > 100 ? run(argc) : 0; }
"""


def test_cpp_facade_links_against_the_library():
    """A program using the facade (batch, selector, the reference's calls)
    compiles and links against librasterizer_gb300; run with no argument it
    does not touch a GPU."""
    import rasterizer_gb300._lib as L
    so = L.lib_path() if hasattr(L, "lib_path") else os.path.join(ROOT, "rasterizer_gb300", "lib", "librasterizer_gb300.so")
    if not os.path.exists(so):
        pytest.skip("library not built")
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        open(p, "w").write(FACADE_PROGRAM)
        subprocess.run(["g++", "-std=c++17", "-O0", "-I" + os.path.join(ROOT, "include"), p, "-o", exe, so,
                        "-Wl,-rpath," + os.path.dirname(so)], check=True)
        assert subprocess.run([exe]).returncode == 0


def test_decomposition_of_triangles_with_a_repeated_vertex_terminates():
    """A triangle with a repeated vertex holds an edge and its reverse; the
    reference makes it its own neighbour and its matching can then loop
    forever on such input.  The library never pairs a triangle with itself:
    the call returns, and every triangle is emitted (in a pair or alone)."""
    code = (
        "import numpy as np\n"
        "from rasterizer_gb300 import api\n"
        "rng = np.random.default_rng(1)\n"
        "v = (np.round(rng.uniform(-5, 5, (200, 4)) * 4) / 4).astype(np.float32); v[:, 3] = 1\n"
        "v[5] = v[4]; v[6] = (v[4] + v[7]) / 2\n"
        "t = rng.integers(0, 10, (200, 3)).astype(np.uint32)\n"
        "for tris in (t, np.array([[8, 1, 8], [8, 5, 1]], np.uint32)):\n"
        "    q = api.QuadDecomposition.decompose(tris.ravel(), v).reshape(-1, 4)\n"
        "    assert (len(tris) + 1) // 2 <= len(q) <= len(tris), (len(tris), len(q))\n"
        "print('ok')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr
