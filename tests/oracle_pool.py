"""Oracle frames in worker processes (test infrastructure): whole
configurations are checked against the oracle view by view, each view an
independent task.  Workers are spawned (never forked from a process that
holds a CUDA context) and load the baked scene from an npz file."""
from __future__ import annotations

import hashlib
import multiprocessing as mp
import os

import numpy as np

_STATE = {}


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:24]


def _init(scene_path: str):
    from oracle.bindings import Oracle, load_baked_scene
    _STATE["scene"] = load_baked_scene(scene_path)
    _STATE["table"] = Oracle(8, 8).table()  # built once per worker


def view_task(task: dict) -> dict:
    """One view: the plain all-occluder loop over `order` (or the whole scene),
    then the queries.  task: key, width, height, mvp, order, mins, maxs, and
    optionally depth / hiz (the state to start from, stale depth included)
    and frames (several matrices drawn one after the other, digests per frame)."""
    from oracle.bindings import Oracle
    sc = _STATE["scene"]
    orc = Oracle(task["width"], task["height"], _STATE["table"])
    orc.set_block_index_wrap(False)  # the library always uses the full block index
    if task.get("depth") is not None:
        orc.write_depth(task["depth"])
        orc.write_hiz(task["hiz"])
    out = []
    for m in task.get("frames", [task.get("mvp")]):
        orc.frame_plain(sc, m, order=task.get("order"))
        vis, nc = orc.query(task["mins"], task["maxs"])
        out.append({"depth": digest(orc.depth()), "hiz": digest(orc.hiz()), "visible": digest(vis),
                    "needsClipping": digest(nc)})
    orc.close()
    return {"key": task["key"], "frames": out}


def pool(scene_path: str, processes: int | None = None):
    n = processes or max(1, min(16, os.cpu_count() or 1))
    return mp.get_context("spawn").Pool(n, initializer=_init, initargs=(scene_path,))
