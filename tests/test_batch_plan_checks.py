"""Host-side checks of the batch entry points, without a GPU.

``ytgb_batch_render_noalloc`` receives the planned entry table in host
memory, so it checks the table against its launch arguments before anything
reaches the device: a sampler kind or table layout that differs from the
entries', shared memory below what the entries' tables take, a tile shape or
total the entries were not planned for.  Each is rejected with
YTGB_ERR_INVALID and no CUDA call (these cases run on a machine without a
GPU).  The table's device pointers are never dereferenced by the host, so
placeholder addresses stand in for them.
"""
import ctypes as C

import numpy as np

from yt_gb300 import _lib, workloads
from yt_gb300.camera import Camera
from yt_gb300.transfer_functions import pack

FAKE = 1 << 20  # a 16-byte aligned placeholder device address


def planned(tile_shape=1, sizes=((40, 24), (64, 64), (17, 90))):
    w = workloads.uniform_vr(n=8, res=8)
    tf = pack(w.tf)
    entries = (_lib.BatchEntry * len(sizes))()
    for k, res in enumerate(sizes):
        cam = Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), 1.5, res, lens_type="perspective")
        a = entries[k].args
        a.kind = _lib.VOLUME_RENDER
        a.n_samples = 1
        a.n_order = 1
        a.flags = tile_shape << _lib.FLAG_TILE_SHIFT
        a.view = cam.device_view()
        a.bricks = a.order = a.rects = a.data = a.bounds = a.tf_tables = a.image = FAKE
        a.tf = tf.header
    total, smem = C.c_int32(), C.c_int32()
    L = _lib.lib()
    assert L.ytgb_batch_plan(entries, len(sizes), tile_shape, C.byref(total), C.byref(smem)) == _lib.OK
    return entries, len(sizes), total.value, smem.value, int(tf.header.ctf_fast)


def noalloc(entries, n, kind, ctf, tile_shape, total, smem):
    L = _lib.lib()
    st = L.ytgb_batch_render_noalloc(entries, n, kind, ctf, tile_shape, total, smem, 0, None)
    return st, L.ytgb_last_error().decode()


def test_plan_numbering():
    entries, n, total, smem, ctf = planned(tile_shape=1)
    assert ctf == 1 and smem == 3 * 256 * 16
    # tile shape 1: 16 rows x 8 columns per tile
    expect = [((40 + 15) // 16) * ((24 + 7) // 8), ((64 + 15) // 16) * ((64 + 7) // 8),
              ((17 + 15) // 16) * ((90 + 7) // 8)]
    assert [entries[k].tiles for k in range(n)] == expect
    assert [entries[k].tile_begin for k in range(n)] == list(np.cumsum([0] + expect[:-1]))
    assert total == sum(expect)


def test_noalloc_rejects_mismatched_kind_and_layout():
    entries, n, total, smem, ctf = planned()
    st, msg = noalloc(entries, n, _lib.PROJECTION, 0, 1, total, 0)
    assert st == _lib.ERR_INVALID and "sampler kind" in msg
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, 0, 1, total, smem)
    assert st == _lib.ERR_INVALID and "variant" in msg


def test_range_decisions_are_one_variant():
    """Entries with the arena's rounding errors (data_lo, range_eps > 0) take
    the float64 range-decision kernels: a batch may not mix them with
    entries without, and the launch's variant must say which."""
    entries, n, total, smem, ctf = planned()
    entries[0].args.data_lo = FAKE
    entries[0].args.range_eps = 1e-7
    L = _lib.lib()
    t, sm = C.c_int32(), C.c_int32()
    assert L.ytgb_batch_plan(entries, n, 1, C.byref(t), C.byref(sm)) == _lib.ERR_INVALID
    assert "range decisions" in L.ytgb_last_error().decode()
    for k in range(n):
        entries[k].args.data_lo = FAKE
        entries[k].args.range_eps = 1e-7
    assert L.ytgb_batch_plan(entries, n, 1, C.byref(t), C.byref(sm)) == _lib.OK
    assert _lib.render_variant(entries[0].args) == _lib.VARIANT_CTF | _lib.VARIANT_RANGE64
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 1, total, smem)
    assert st == _lib.ERR_INVALID and "variant" in msg
    entries[1].args.range_eps = float("nan")
    assert L.ytgb_batch_plan(entries, n, 1, C.byref(t), C.byref(sm)) == _lib.ERR_INVALID
    assert "range_eps" in L.ytgb_last_error().decode()


def test_noalloc_rejects_short_shared_memory():
    entries, n, total, smem, ctf = planned()
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 1, total, smem - 16)
    assert st == _lib.ERR_INVALID and "smem_bytes" in msg


def test_noalloc_rejects_other_tiling():
    entries, n, total, smem, ctf = planned(tile_shape=1)
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 0, total, smem)
    assert st == _lib.ERR_INVALID and "tile shape" in msg
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 1, total + 1, smem)
    assert st == _lib.ERR_INVALID and "total_tiles" in msg
    entries[1].tile_begin += 1
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 1, total, smem)
    assert st == _lib.ERR_INVALID and "tile shape" in msg


def test_noalloc_rejects_invalid_entry_arguments():
    entries, n, total, smem, ctf = planned()
    entries[2].args.image = None
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 1, total, smem)
    assert st == _lib.ERR_INVALID and "missing image" in msg


def test_plan_asks_for_shared_memory_only_for_one_shared_table():
    """Entries that read different transfer functions are planned for the
    global-memory table path (smem_bytes 0); staging one shared table
    (smem_bytes > 0) is then rejected by the no-alloc entry point."""
    entries, n, total, smem, ctf = planned()
    entries[1].args.tf_tables = FAKE + 4096
    t, sm = C.c_int32(), C.c_int32()
    assert _lib.lib().ytgb_batch_plan(entries, n, 1, C.byref(t), C.byref(sm)) == _lib.OK
    assert sm.value == 0 and t.value == total
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 1, total, smem)
    assert st == _lib.ERR_INVALID and "different" in msg


def test_noalloc_rejects_views_without_derived_constants():
    """ytgb_batch_plan derives each view's per-view ray constants (the
    perspective lens's linspace steps and normal * width); a table that did
    not go through it is rejected before anything is queued."""
    entries, n, total, smem, ctf = planned()
    assert entries[0].args.view.lin_step[0] > 0
    entries[1].args.view.lin_step[0] = 0.0
    st, msg = noalloc(entries, n, _lib.VOLUME_RENDER, ctf, 1, total, smem)
    assert st == _lib.ERR_INVALID and "derived view constants" in msg


def test_render_variant_cases():
    """The kernel variant a render's arguments call for (``render_variant``,
    the host mirror of the library's): the ColorTransferFunction layout for
    volume rendering only; float64 range decisions with data_lo and a
    positive range_eps, for volume rendering and the light source, but not
    for a ColorTransferFunction whose table excludes every value."""
    from yt_gb300.transfer_functions import ProjectionTransferFunction

    w = workloads.uniform_vr(n=8, res=8)
    a = _lib.RenderArgs()
    a.kind = _lib.VOLUME_RENDER
    a.tf = pack(w.tf).header
    assert _lib.render_variant(a) == _lib.VARIANT_CTF
    a.data_lo, a.range_eps = FAKE, 1e-7
    assert _lib.render_variant(a) == _lib.VARIANT_CTF | _lib.VARIANT_RANGE64
    a.range_eps = 0.0
    assert _lib.render_variant(a) == _lib.VARIANT_CTF
    a.kind, a.range_eps = _lib.LIGHT_SOURCE, 1e-7
    assert _lib.render_variant(a) == _lib.VARIANT_RANGE64
    a.kind = _lib.PROJECTION
    assert _lib.render_variant(a) == 0
    # a table that excludes every value (all-zero table, bounds beyond float32)
    a.kind = _lib.VOLUME_RENDER
    a.tf = pack(ProjectionTransferFunction()).header
    assert a.tf.lo_excl[0] > a.tf.hi_excl[0]
    assert _lib.render_variant(a) & _lib.VARIANT_RANGE64 == (0 if a.tf.ctf_fast else _lib.VARIANT_RANGE64)
