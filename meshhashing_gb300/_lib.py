"""Loader of the in-tree CUDA library (libmeshhash.so) and its C signatures.

There is no fallback: if the library is missing or cannot be loaded, every
entry point raises.  ``SYMBOLS`` lists the extern "C" functions declared in
include/meshhash.h.
"""
from __future__ import annotations

import ctypes as C
import os

from ._abi import MhBatchTuning, MhParams, MhStats

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmeshhash.so")

vp = C.c_void_p
i32p = C.POINTER(C.c_int32)
f32p = C.POINTER(C.c_float)
u8p = C.POINTER(C.c_uint8)
u16p = C.POINTER(C.c_uint16)
i32 = C.c_int
MHV = C.c_void_p  # opaque mh_volume*

SIGNATURES = {
    "mh_default_params": (i32, [C.POINTER(MhParams)]),
    "mh_volume_create": (i32, [C.POINTER(MhParams), C.POINTER(MHV)]),
    "mh_volume_destroy": (i32, [MHV]),
    "mh_volume_reset": (i32, [MHV, vp]),
    "mh_frame_set": (i32, [MHV, vp, i32, f32p, vp]),
    "mh_frame_set_u16": (i32, [MHV, vp, i32, f32p, vp]),
    "mh_allocate": (i32, [MHV, vp]),
    "mh_collect_frustum": (i32, [MHV, vp]),
    "mh_collect_all": (i32, [MHV, vp]),
    "mh_integrate_simple": (i32, [MHV, vp]),
    "mh_predict_inlier": (i32, [MHV, vp]),
    "mh_integrate_psdf": (i32, [MHV, vp]),
    "mh_mesh": (i32, [MHV, vp]),
    "mh_gc_low_surfel": (i32, [MHV, vp]),
    "mh_gc_recycle": (i32, [MHV, vp]),
    "mh_gc_starve": (i32, [MHV, vp]),
    "mh_gc_collect_garbage": (i32, [MHV, vp]),
    "mh_raycast": (i32, [MHV, f32p, vp, vp, vp, i32, vp]),
    "mh_denoise_tv": (i32, [MHV, C.c_float, i32, vp]),
    "mh_integrate_frame": (i32, [MHV, vp, i32, f32p, i32, C.c_float, vp, vp, vp, i32, vp]),
    "mh_stats_get": (i32, [MHV, C.POINTER(MhStats), vp]),
    "mh_clear_error": (i32, [MHV, vp]),
    "mh_dump_blocks": (i32, [MHV, i32, i32p, f32p, f32p, f32p, f32p, i32p]),
    "mh_load_blocks": (i32, [MHV, i32, i32p, f32p, f32p, f32p, f32p]),
    "mh_dump_candidates": (i32, [MHV, i32, i32p, i32p]),
    "mh_set_candidates": (i32, [MHV, i32, i32p]),
    "mh_dump_inlier": (i32, [MHV, f32p]),
    "mh_dump_depth": (i32, [MHV, f32p]),
    "mh_dump_mesh": (i32, [MHV, i32, i32p, f32p, i32, i32p, i32p, i32p]),
    "mh_dump_cubes": (i32, [MHV, i32, i32p, u8p]),
    "mh_dump_block_meta": (i32, [MHV, i32, i32p, i32p, i32p, i32p]),
    "mh_dump_flags": (i32, [MHV, i32, u8p, i32p]),
    "mh_dump_nonneg_counts": (i32, [MHV, i32, i32p, i32p]),
    "mh_raycast_footprint": (i32, [MHV, f32p, i32p, vp]),
    "mh_hash_bucket": (C.c_uint32, [C.c_int32, C.c_int32, C.c_int32, C.c_uint32]),
    "mh_bytes_model": (i32, [MHV, C.POINTER(C.c_double)]),
    "mh_profile_enable": (i32, [MHV, i32]),
    "mh_profile_read": (i32, [MHV, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "mh_launch_count": (C.c_uint64, []),
    "mh_denoise_tv_static": (i32, [vp, vp, i32, i32, C.c_float, i32, vp]),
    "mh_raycast_backward": (i32, [MHV, f32p, vp, vp, vp, C.POINTER(C.c_double), vp]),
    "mh_raycast_normal_equations": (i32, [MHV, f32p, vp, C.c_float, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.POINTER(C.c_int32), vp]),
    "mh_refine_pose": (i32, [MHV, vp, f32p, i32, C.c_float, C.POINTER(C.c_double), C.POINTER(C.c_int32), vp]),
    "mh_dump_block_field": (i32, [MHV, vp, i32, i32p, f32p, i32p]),
    "mh_point_to_psdf_normal_equations": (i32, [MHV, f32p, i32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                C.POINTER(C.c_double), i32p, vp]),
    "mh_track_point_to_psdf": (i32, [MHV, f32p, i32, C.c_float, i32, C.POINTER(C.c_double), i32p, vp]),
    "mh_mesh_compact": (i32, [MHV, i32, vp, vp, i32, vp, i32p, i32p, i32, vp]),
    "mh_write_ply": (i32, [MHV, C.c_char_p]),
    "mh_write_obj": (i32, [MHV, C.c_char_p]),
    "mh_save_volume": (i32, [MHV, C.c_char_p]),
    "mh_load_volume": (i32, [MHV, C.c_char_p, i32p]),
    "mh_huber_tv_init": (i32, [MHV, vp]),
    "mh_huber_tv_iterate": (i32, [MHV, C.c_float, C.c_float, C.c_float, i32, C.POINTER(C.c_double), vp]),
    "mh_batch_create": (i32, [C.POINTER(MHV), i32, i32, C.POINTER(vp)]),
    "mh_batch_destroy": (i32, [vp]),
    "mh_batch_step": (i32, [vp, C.POINTER(vp), i32, f32p, i32p, i32, C.c_float, i32, vp]),
    "mh_batch_outputs": (i32, [vp, i32, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "mh_batch_dump_raycast": (i32, [vp, i32, f32p, f32p, f32p]),
    "mh_batch_get_tuning": (i32, [vp, C.POINTER(MhBatchTuning)]),
    "mh_batch_set_tuning": (i32, [vp, C.POINTER(MhBatchTuning)]),
    "mh_batch_autotune": (i32, [vp, i32]),
    "mh_batch_tuning_times": (i32, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mh_batch_stage_times": (i32, [vp, C.POINTER(C.c_double)]),
}
SYMBOLS = sorted(SIGNATURES)

_lib = None


class MeshHashError(RuntimeError):
    def __init__(self, fn, code):
        from ._abi import STATUS_NAMES
        super().__init__(f"{fn} failed: {STATUS_NAMES.get(code, code)}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load libmeshhash.so (build it first with meshhashing_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build the CUDA library first "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(fn_name: str, code: int):
    if code != 0:
        raise MeshHashError(fn_name, code)
