"""Loads librasterizer_gb300.so (built in-tree) and declares its C ABI.

There is no fallback: if the library is missing or cannot be loaded, import
fails with the reason.  The GPU work happens only inside the library.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int
FP = C.POINTER(C.c_float)

_lib = None


class OccError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where} failed ({status}): {message}")
        self.status = status


# name -> (restype, argtypes); mirrors include/rasterizer_gb300.h
SIGNATURES = {
    "occ_last_error": (C.c_char_p, []),
    "occ_version": (I32, []),
    "occ_ctx_create": (I32, [I32, C.POINTER(P)]),
    "occ_ctx_destroy": (I32, [P]),
    "occ_ctx_synchronize": (I32, [P]),
    "occ_ctx_stream": (P, [P]),
    "occ_occluder_upload": (I32, [P, P, U32, P, P, P, P, C.POINTER(U32)]),
    "occ_occluder_count": (I32, [P, C.POINTER(U32)]),
    "occ_raster_create": (I32, [P, U32, U32, C.POINTER(P)]),
    "occ_raster_destroy": (I32, [P]),
    "occ_raster_set_mvp": (I32, [P, P]),
    "occ_raster_clear": (I32, [P]),
    "occ_raster_rasterize": (I32, [P, U32, I32]),
    "occ_raster_rasterize_many": (I32, [P, U32, P, P]),
    "occ_raster_flush": (I32, [P]),
    "occ_raster_command_flags": (I32, [P, U32, P]),
    "occ_raster_query_visibility": (I32, [P, P, P, C.POINTER(I32), C.POINTER(I32)]),
    "occ_raster_query_batch": (I32, [P, U32, P, P, P, P]),
    "occ_raster_query_batch_device": (I32, [P, U32, P, P, P, P]),
    "occ_raster_query_batch_noalloc": (I32, [P, U32, P, P, P, P]),
    "occ_raster_query2d": (I32, [P, U32, U32, U32, U32, U32, C.POINTER(I32)]),
    "occ_raster_read_back_depth": (I32, [P, P]),
    "occ_raster_read_back": (I32, [P, I32, P]),
    "occ_raster_read_depth_raw": (I32, [P, P]),
    "occ_raster_read_hiz": (I32, [P, P, C.POINTER(U32)]),
    "occ_raster_write_depth_raw": (I32, [P, P]),
    "occ_raster_write_hiz": (I32, [P, P]),
    "occ_raster_size": (I32, [P, C.POINTER(U32), C.POINTER(U32)]),
    "occ_batch_execute": (I32, [P, U32, P]),
    "occ_batch_prepare": (I32, [P, U32, P, C.POINTER(P)]),
    "occ_batch_set_mvp": (I32, [P, U32, P]),
    "occ_batch_launch": (I32, [P]),
    "occ_batch_results": (I32, [P, U32, P, P]),
    "occ_batch_check": (I32, [P]),
    "occ_batch_profile": (I32, [P, U32, P]),
    "occ_batch_destroy": (I32, [P]),
    "occ_batch_set_selection": (I32, [P, P, C.c_float, I32]),
    "occ_batch_read_selection": (I32, [P, U32, P, P, P, P, P]),
    "occ_batch_set_zero_depth": (I32, [P, I32]),
    "occ_batch_set_second_pass": (I32, [P, I32]),
    "occ_batch_set_cull_labels": (I32, [P, I32]),
    "occ_batch_read_cull_labels": (I32, [P, U32, P]),
    "occ_batch_stats": (I32, [P, P]),
    "occ_batch_set_mvps": (I32, [P, U32, U32, P]),
    "occ_batch_result_words": (I32, [P, C.POINTER(U32)]),
    "occ_batch_results_all": (I32, [P, P, P, P]),
    "occ_batch_results_all_async": (I32, [P, P, P]),
    "occ_batch_set_queries": (I32, [P, U32, U32, P, P]),
    "occ_batch_autotune": (I32, [P, U32, P, P, P]),
    "occ_batch_set_tuning": (I32, [P, P]),
    "occ_mlp_param_count": (I32, []),
    "occ_mlp_create": (I32, [P, U32, C.POINTER(P)]),
    "occ_mlp_destroy": (I32, [P]),
    "occ_mlp_get_params": (I32, [P, P]),
    "occ_mlp_get_state": (I32, [P, P, P, P, C.POINTER(U32)]),
    "occ_mlp_set_state": (I32, [P, P, P, P, U32]),
    "occ_mlp_set_params": (I32, [P, P]),
    "occ_mlp_forward": (I32, [P, U32, P, P]),
    "occ_mlp_gradients": (I32, [P, U32, P, P, C.POINTER(C.c_float), P]),
    "occ_mlp_train_step": (I32, [P, U32, P, P, C.c_float, C.POINTER(C.c_float)]),
    "occ_mlp_gradients_listwise": (I32, [P, U32, P, P, U32, P, C.POINTER(C.c_float), P]),
    "occ_mlp_train_step_listwise": (I32, [P, U32, P, P, U32, P, C.c_float, C.POINTER(C.c_float)]),
    "occ_quad_decompose": (I32, [P, U32, P, U32, P, C.POINTER(U32)]),
    "occ_sah_generate_batches": (I32, [P, U32, U32, U32, P, P, C.POINTER(U32)]),
    "occ_sah_generate_batches_device": (I32, [P, P, U32, U32, U32, P, P, C.POINTER(U32)]),
    "occ_occluder_bake": (I32, [P, U32, P, P, P, C.POINTER(U32), P, P, P]),
    "occ_occluders_bake_device": (I32, [P, U32, P, P, P, P, P]),
    "occ_scene_bake": (I32, [P, U32, P, U32, U32, U32, U32, C.c_uint64, C.POINTER(U32), C.POINTER(C.c_uint64), P, P, P]),
    "occ_occluder_upload_device": (I32, [P, P, U32, P, C.POINTER(U32)]),
    "occ_mesh_load_bin": (I32, [C.c_char_p, C.c_char_p, P, C.POINTER(U32), P, C.POINTER(U32)]),
    "occ_occluders_save": (I32, [C.c_char_p, U32, P, P, P]),
    "occ_occluders_file_info": (I32, [C.c_char_p, C.POINTER(U32), C.POINTER(C.c_uint64)]),
    "occ_occluders_load": (I32, [C.c_char_p, U32, C.c_uint64, P, P, P]),
    "occ_build_coverage_table": (I32, [P]),
    "occ_coverage_table": (I32, [P]),
}


class ViewWork(C.Structure):
    """occ_view_work"""
    _fields_ = [
        ("raster", P),
        ("mvp", P),
        ("clear", I32),
        ("numOccluders", U32),
        ("occluders", P),
        ("flags", P),
        ("numQueries", U32),
        ("queryMins", P),
        ("queryMaxs", P),
        ("visibleBits", P),
        ("needsClippingBits", P),
    ]


def library_path() -> str:
    return _build.LIB


def lib():
    """The loaded library (built on first use if the sources are newer)."""
    global _lib
    if _lib is None:
        path = _build.build()
        if not os.path.exists(path):
            raise ImportError(f"librasterizer_gb300.so missing at {path}")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != 0:
        msg = lib().occ_last_error()
        raise OccError(status, where, msg.decode() if msg else "")
