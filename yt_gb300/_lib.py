"""ctypes binding of libytgb.so (the C ABI declared in include/ytgb.h).

The structures below mirror ``ytgb_brick``, ``ytgb_view``, ``ytgb_tf`` and
``ytgb_render_args`` field for field.  The library is loaded from the package
tree (``yt_gb300/lib/libytgb.so``); when it is missing or fails to load,
every entry point raises: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libytgb.so"

OK, ERR_INVALID, ERR_CUDA, ERR_DEVICE = 0, -1, -2, -3
VOLUME_RENDER, PROJECTION, INTERPOLATED_PROJECTION, MIP, LIGHT_SOURCE = 0, 1, 2, 3, 4
LENS_PLANE_PARALLEL, LENS_PER_PIXEL, LENS_PERSPECTIVE = 0, 1, 2
EXTENT_PLANE_PARALLEL, EXTENT_PERSPECTIVE, EXTENT_NULL = 0, 1, 2
FLAG_NO_COMPENSATION = 1
FLAG_TILE_SHIFT = 8
NOALLOC_MAX_ENTRIES = 128  # YTGB_NOALLOC_MAX_ENTRIES
VARIANT_CTF, VARIANT_RANGE64 = 1, 2  # YTGB_VARIANT_*
FNV_OFFSET = 1469598103934665603

_dp = C.POINTER(C.c_double)


class Brick(C.Structure):
    _fields_ = [
        ("left_edge", C.c_double * 3),
        ("right_edge", C.c_double * 3),
        ("dds", C.c_double * 3),
        ("idds", C.c_double * 3),
        ("snap", C.c_double * 3),
        ("dims", C.c_int32 * 3),
        ("n_fields", C.c_int32),
        ("data_offset", C.c_int64),
        ("field_stride", C.c_int64),
        ("mask_offset", C.c_int64),
        ("bounds_offset", C.c_int64),
        ("lef", C.c_float * 3),
        ("ref", C.c_float * 3),
        ("iddsf", C.c_float * 3),
        ("pad", C.c_int32 * 5),
    ]


class View(C.Structure):
    _fields_ = [
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("lens", C.c_int32),
        ("extent", C.c_int32),
        ("vp_pos", C.c_double * 12),
        ("vp_dir", C.c_double * 3),
        ("center", C.c_double * 3),
        ("bounds", C.c_double * 4),
        ("x_vec", C.c_double * 3),
        ("y_vec", C.c_double * 3),
        ("width", C.c_double * 3),
        ("camera_data", C.c_double * 15),
        ("pdx", C.c_double),
        ("pdy", C.c_double),
        ("ray_scale", C.c_double),
        ("lin_step", C.c_double * 2),
        ("normal_w2", C.c_double * 3),
        ("px_pos", C.c_void_p),
        ("px_dir", C.c_void_p),
    ]


class TF(C.Structure):
    _fields_ = [
        ("n_fits", C.c_int32),
        ("grey_opacity", C.c_int32),
        ("nbins_max", C.c_int32),
        ("ctf_fast", C.c_int32),
        ("field_table_ids", C.c_int32 * 6),
        ("field_id", C.c_int32 * 6),
        ("weight_field_id", C.c_int32 * 6),
        ("weight_table_id", C.c_int32 * 6),
        ("nbins", C.c_int32 * 6),
        ("lo_excl", C.c_float * 6),
        ("hi_excl", C.c_float * 6),
        ("b0", C.c_float * 6),
        ("idbin", C.c_float * 6),
        ("bound64", (C.c_double * 2) * 6),
    ]


class RenderArgs(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("n_samples", C.c_int32),
        ("n_order", C.c_int32),
        ("flags", C.c_uint32),
        ("view", View),
        ("bricks", C.c_void_p),
        ("order", C.c_void_p),
        ("rects", C.c_void_p),
        ("data", C.c_void_p),
        ("masks", C.c_void_p),
        ("bounds", C.c_void_p),
        ("tf", TF),
        ("tf_tables", C.c_void_p),
        ("image", C.c_void_p),
        ("zbuffer", C.c_void_p),
        ("counters", C.c_void_p),
        ("error", C.c_void_p),
        ("data_lo", C.c_void_p),
        ("light_dir", C.c_float * 3),
        ("light_rgba", C.c_float * 4),
        ("range_eps", C.c_float),
    ]


class ONode(C.Structure):
    _fields_ = [("child", C.c_int32 * 8), ("key", C.c_int32), ("flags", C.c_int32)]


class OctreeArgs(C.Structure):
    _fields_ = [
        ("nodes", C.c_void_p),
        ("verts", C.c_void_p),
        ("edges", C.c_void_p),
        ("n_nodes", C.c_int32),
        ("n_cells", C.c_int32),
        ("depth", C.c_int32),
        ("pad", C.c_int32),
        ("dle", C.c_double * 3),
        ("dre", C.c_double * 3),
        ("edges_f", C.c_void_p),
    ]


class OffaxisArgs(C.Structure):
    _fields_ = [
        ("xp", C.c_void_p),
        ("dxp", C.c_void_p),
        ("qty", C.c_void_p),
        ("weight", C.c_void_p),
        ("stamp", C.c_void_p),
        ("buffer", C.c_void_p),
        ("buffer_weight", C.c_void_p),
        ("rot", C.c_double * 6),
        ("n", C.c_int64),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nsx", C.c_int32),
        ("nsy", C.c_int32),
        ("max_depth", C.c_int32),
        ("pad", C.c_int32),
    ]


class BatchEntry(C.Structure):
    _fields_ = [
        ("args", RenderArgs),
        ("tile_begin", C.c_int32),
        ("tiles_y", C.c_int32),
        ("tiles", C.c_int32),
        ("pad", C.c_int32),
    ]


class YtgbError(RuntimeError):
    pass


_lib = None
_lock = threading.Lock()

# every exported symbol of include/ytgb.h with (restype, argtypes)
SIGNATURES = {
    "ytgb_abi_version": (C.c_int, []),
    "ytgb_last_error": (C.c_char_p, []),
    "ytgb_check_error": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ytgb_brick_rects": (C.c_int, [C.POINTER(View), C.POINTER(Brick), C.c_int32, C.c_void_p, C.c_int32,
                                   C.c_void_p]),
    "ytgb_tf_pack": (C.c_int, [C.c_int32, C.POINTER(_dp), C.POINTER(C.c_int32), _dp, C.POINTER(C.c_int32),
                               C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32,
                               C.POINTER(TF), C.c_void_p]),
    "ytgb_render": (C.c_int, [C.POINTER(RenderArgs), C.c_void_p]),
    "ytgb_trace": (C.c_int, [C.POINTER(RenderArgs), C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_batch_plan": (C.c_int, [C.POINTER(BatchEntry), C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int32)]),
    "ytgb_batch_render": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_void_p, C.c_int32, C.c_void_p]),
    "ytgb_batch_render_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                            C.c_int32, C.c_int32, C.c_void_p]),
    "ytgb_vertex_bricks": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                     C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_pack_fields_split": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                         C.c_int32]),
    "ytgb_octree_build": (C.c_void_p, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_int64]),
    "ytgb_octree_num_nodes": (C.c_int64, [C.c_void_p]),
    "ytgb_octree_nodes": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ytgb_octree_destroy": (None, [C.c_void_p]),
    "ytgb_render_octree": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_offaxis_cells": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_offaxis_depths": (C.c_int, [C.c_void_p] * 4 + [C.c_int32] * 3 + [C.c_void_p, C.c_void_p]),
    "ytgb_gather_fields": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                     C.c_int64, C.c_void_p]),
    "ytgb_device_reads_host": (C.c_int, [C.c_void_p]),
    "ytgb_gather_masks": (C.c_int, [C.c_void_p] * 4 + [C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32,
                                                        C.c_void_p]),
    "ytgb_brick_layout": (C.c_int, [C.c_int64] + [C.c_void_p] * 7 + [C.c_int64, C.c_void_p]),
    "ytgb_trace_octree": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_pack_fields": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32]),
    "ytgb_pack_masks": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32,
                                  C.POINTER(C.c_int32)]),
    "ytgb_host_copy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32]),
    "ytgb_host_prefault": (C.c_int, [C.c_void_p, C.c_int64]),
    "ytgb_host_is_uniform": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_int32, C.POINTER(C.c_int32)]),
    "ytgb_kdtree_build": (C.c_void_p, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_kdtree_destroy": (None, [C.c_void_p]),
    "ytgb_kdtree_num_leaves": (C.c_int32, [C.c_void_p]),
    "ytgb_kdtree_leaves": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_kdtree_viewpoint_order": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "ytgb_kdtree_viewpoint_orders": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
}


def lib() -> C.CDLL:
    """Load libytgb.so (raising if it is absent: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise YtgbError(
                    f"{LIB_PATH} is missing: build it with `python -m yt_gb300.build` "
                    "(the CUDA renderer has no CPU fallback)")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            if L.ytgb_abi_version() != 4:
                raise YtgbError("libytgb ABI version mismatch")
            _lib = L
    return _lib


def render_variant(a) -> int:
    """The kernel variant (YTGB_VARIANT_* bits) a RenderArgs calls for: the
    ColorTransferFunction layout, and float64 range decisions where the
    arena's rounding errors (data_lo) and range_eps > 0 are given -- except
    for a ColorTransferFunction whose table excludes every value."""
    v = 0
    if a.kind == VOLUME_RENDER and a.tf.ctf_fast:
        v |= VARIANT_CTF
    if (a.kind in (VOLUME_RENDER, LIGHT_SOURCE) and a.data_lo and a.range_eps > 0.0
            and (not v & VARIANT_CTF or a.tf.lo_excl[0] <= a.tf.hi_excl[0])):
        v |= VARIANT_RANGE64
    return v


def check(status: int, what: str) -> None:
    if status != OK:
        msg = lib().ytgb_last_error().decode(errors="replace")
        raise YtgbError(f"{what} failed ({status}): {msg}")
