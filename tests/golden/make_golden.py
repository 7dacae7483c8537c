"""Generates tests/golden/golden.json and golden_small.npz from the reference itself.

Runs on x86-64 only, with the reference's sources compiled by oracle/Makefile
(oracle/_ref/libref.so).  Every number here comes from the reference's own
code: its scene preparation (Main.cpp:86-128) and its Rasterizer
(Rasterizer.cpp), driven by the seeded synthetic inputs of
rasterizer_gb300.scenes.  The tests check the portable oracle and the
library's host bake against these fixtures on any host (x86-64 or aarch64).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.bindings import Reference, reference_bake_scene, save_baked_scene  # noqa: E402
from rasterizer_gb300 import scenes  # noqa: E402

# fixture cases: (name, scene builder, resolution, camera list, query spec)
CITY_FRAMES = (0, 60, 120, 180, 240, 299)


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:24]


def scene_digest(sc) -> str:
    return digest(*sc.packed, sc.packets, sc.ref, sc.bounds, sc.centers)


def run_frames(sc, w, h, mvps, mins, maxs):
    ref, scratch = Reference(w, h), Reference(w, h)
    out = []
    for m in mvps:
        flags = ref.frame_plain_packed(scratch, sc, m)
        vis, nc = ref.query(mins, maxs)
        depth, hiz = ref.depth(), ref.hiz()
        out.append({"flags": digest(flags), "depth": digest(depth), "hiz": digest(hiz),
                    "visible": digest(vis), "needsClipping": digest(nc), "readback": digest(ref.read_back()),
                    "visible_count": int(vis.sum()), "near_clipped": int(((flags & 3) == 3).sum()),
                    "drawn": int((flags & 1).sum())})
    return out


def main():
    g = {"generator": "tests/golden/make_golden.py (reference sources compiled by oracle/Makefile, x86-64)"}
    table = Reference(8, 8).table()
    g["coverage_table"] = digest(table)

    m = scenes.boxes_scene()
    sc = reference_bake_scene(m.vertices, m.indices)
    mins, maxs = scenes.query_boxes(4096, seed=43)
    g["boxes"] = {"mesh": m.digest(), "triangles": m.triangles, "occluders": len(sc), "quads": sc.quads,
                  "bake": scene_digest(sc),
                  "frames": run_frames(sc, 1920, 1080, [scenes.boxes_camera()], mins, maxs)}

    c = scenes.city_scene()
    sc = reference_bake_scene(c.vertices, c.indices)
    mvps, _ = scenes.camera_path(300, seed=7)
    mins, maxs = scenes.query_boxes(20000, seed=44, footprint=300.0, lognormal=(0.0, 1.0), y_range=(0.0, 20.0))
    g["city"] = {"mesh": c.digest(), "triangles": c.triangles, "occluders": len(sc), "quads": sc.quads,
                 "bake": scene_digest(sc), "frame_indices": list(CITY_FRAMES),
                 "frames": run_frames(sc, 1920, 1080, [mvps[f] for f in CITY_FRAMES], mins, maxs)}
    # the city's occluders as the reference bakes them, for the benchmark's CPU
    # arms (any host, no native library of this project involved)
    save_baked_scene(os.path.join(HERE, "city_occluders.npz"), sc)

    # one small frame kept raw: the boxes scene at 320x200 seen from above the footprint
    sc = reference_bake_scene(m.vertices, m.indices)
    mvp = scenes.view_projection((10.0, 25.0, -45.0), (-0.1, -0.45, 1.0), aspect=320 / 200)
    ref, scratch = Reference(320, 200), Reference(320, 200)
    flags = ref.frame_plain_packed(scratch, sc, mvp)
    qm, qM = scenes.query_boxes(1024, seed=45)
    vis, nc = ref.query(qm, qM)
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), mvp=mvp, depth=ref.depth(), hiz=ref.hiz(),
                        flags=flags, visible=vis, needsClipping=nc, readback=ref.read_back(), table=table)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    print("wrote golden.json and golden_small.npz")


if __name__ == "__main__":
    main()
