"""Device-resident bricks and the one-launch render call.

A :class:`BrickSet` is yt's list of ``PartitionedGrid`` bricks laid out for
HBM: one float32 arena holding every brick's fields back to back (each field
16-byte aligned, C order exactly as the brick's numpy array), an optional
uint8 mask arena, and an array of ``ytgb_brick`` descriptors -- the float64
edges, dds/idds and dims of yt's ``VolumeContainer``
(``yt/utilities/lib/volume_container.pxd:13-33``).  It stays resident across
renders, so a render only uploads its view (the ray generation parameters,
the kd order and the per-brick pixel rectangles).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np
import torch

from . import _lib


def _align4(n: int) -> int:
    return (n + 3) & ~3


def _pinned(shape, dtype, device) -> torch.Tensor:
    t = torch.empty(shape, dtype=dtype)
    if torch.device(device).type == "cuda":
        t = t.pin_memory()
    return t


class BrickSet:
    """Bricks ``(data, mask, left_edge, right_edge, dims)`` resident on ``device``.

    ``data`` is a list of float64 arrays (one per field, any shape; the
    samplers index them exactly as yt does), ``mask`` a uint8 array of
    ``dims`` or None (all ones)."""

    def __init__(self, bricks: Sequence, device="cuda"):
        self.device = torch.device(device)
        n = len(bricks)
        self.n = n
        self.host = (_lib.Brick * max(n, 1))()
        offs = []
        total = 0
        mtotal = 0
        need_mask = False
        self.min_elems = np.zeros(max(n, 1), dtype=np.int64)
        self.cells = np.zeros(max(n, 1), dtype=np.int64)
        self.verts = np.zeros(max(n, 1), dtype=np.int64)
        for k, (data, mask, _le, _re, dims) in enumerate(bricks):
            dims_i = [int(x) for x in dims]
            if len(dims_i) != 3 or min(dims_i) <= 0:
                raise ValueError(f"brick {k}: dims must be 3 positive integers, got {dims_i}")
            if not 1 <= len(data) <= 6:
                raise ValueError(f"brick {k}: 1 to 6 fields supported, got {len(data)}")
            if mask is not None and int(np.asarray(mask).size) != int(np.prod(dims_i)):
                raise ValueError(f"brick {k}: mask must have prod(dims) entries")
            sizes = [int(np.asarray(d).size) for d in data]
            self.min_elems[k] = min(sizes)
            self.cells[k] = int(np.prod(dims_i))
            self.verts[k] = int(np.prod([d + 1 for d in dims_i]))
            stride = _align4(max(sizes) if sizes else 0)
            offs.append((total, stride, mtotal))
            total += stride * len(data)
            if mask is not None and not bool(np.all(np.asarray(mask) == 1)):
                need_mask = True
            mtotal += int(np.prod([int(x) for x in dims]))
        # cell-boundary tables: for each brick and axis, k*dds + le for
        # k = 0..dims (the float64 values walk_volume forms for tmax,
        # grid_traversal.pyx:106-108); numpy's elementwise multiply and add
        # round exactly like the reference's C expression
        nb_total = sum(sum(int(x) + 1 for x in b[4]) for b in bricks)
        bounds = np.empty(max(nb_total, 1), dtype=np.float64)
        buf = _pinned((max(total, 4),), torch.float32, self.device)
        bnp = buf.numpy()
        mbuf = _pinned((max(mtotal, 1),), torch.uint8, self.device) if need_mask else None
        boff = 0
        for k, (data, mask, le, re, dims) in enumerate(bricks):
            off, stride, moff = offs[k]
            b = self.host[k]
            dims = [int(x) for x in dims]
            b.bounds_offset = boff
            for i in range(3):
                b.left_edge[i] = float(le[i])
                b.right_edge[i] = float(re[i])
                b.dims[i] = dims[i]
                # PartitionedGrid.__cinit__ (partitioned_grid.pyx:54-55)
                b.dds[i] = (b.right_edge[i] - b.left_edge[i]) / dims[i]
                b.idds[i] = 1.0 / b.dds[i]
                b.snap[i] = 1e-10 * b.dds[i]
                b.lef[i] = b.left_edge[i]
                b.ref[i] = b.right_edge[i]
                b.iddsf[i] = b.idds[i]
                bounds[boff: boff + dims[i] + 1] = np.arange(dims[i] + 1, dtype=np.float64) * b.dds[i] + b.left_edge[i]
                boff += dims[i] + 1
            b.n_fields = len(data)
            b.data_offset = off
            b.field_stride = stride
            for f, d in enumerate(data):
                a = np.asarray(d).ravel()
                bnp[off + f * stride: off + f * stride + a.size] = a
            if need_mask and mask is not None:
                mnp = mbuf.numpy()
                m = np.asarray(mask, dtype=np.uint8).ravel()
                mnp[moff: moff + m.size] = m
                b.mask_offset = moff
            else:
                b.mask_offset = -1
        self.data = buf.to(self.device, non_blocking=True)
        self.bounds = torch.from_numpy(bounds).to(self.device)
        self.masks = mbuf.to(self.device, non_blocking=True) if mbuf is not None else None
        raw = np.frombuffer(self.host, dtype=np.uint8, count=C.sizeof(_lib.Brick) * max(n, 1)).copy()
        self.desc = torch.from_numpy(raw).to(self.device)
        self.nbytes = int(self.data.numel() * 4)

    def rects(self, view: _lib.View, order: np.ndarray) -> np.ndarray:
        """Per-order-entry pixel rectangles (ytgb_brick_rects)."""
        order = np.ascontiguousarray(order, dtype=np.int32)
        out = np.empty((order.size, 4), dtype=np.int32)
        st = _lib.lib().ytgb_brick_rects(C.byref(view), self.host, self.n, order.ctypes.data, order.size,
                                         out.ctypes.data)
        _lib.check(st, "ytgb_brick_rects")
        return out


def _ptr(t):
    return None if t is None else t.data_ptr()


def check_inputs(bricks: BrickSet, view: _lib.View, order, kind, image=None, zbuffer=None, px_pos=None,
                 px_dir=None):
    """Reject inputs the kernel would index out of bounds: the vertex-centred
    samplers read (dims+1)^3 values per field, the projection samplers
    dims^3 (image_samplers.pyx:341, :384-385, :465-466)."""
    if order.size and (order.min() < 0 or order.max() >= bricks.n):
        raise ValueError("order entry out of range")
    used = np.unique(order) if order.size else order
    need = bricks.verts if kind in (_lib.VOLUME_RENDER, _lib.INTERPOLATED_PROJECTION) else bricks.cells
    short = used[bricks.min_elems[used] < need[used]] if used.size else used
    if short.size:
        k = int(short[0])
        raise ValueError(f"brick {k} has {bricks.min_elems[k]} values per field; this sampler reads {need[k]}")
    nx, ny = view.nx, view.ny
    if image is not None and tuple(image.shape) != (nx, ny, 4) or (image is not None and (
            image.dtype != torch.float64 or not image.is_contiguous())):
        raise ValueError(f"image must be a contiguous float64 ({nx}, {ny}, 4) tensor")
    if zbuffer is not None and (zbuffer.numel() != nx * ny or zbuffer.dtype != torch.float64
                                or not zbuffer.is_contiguous()):
        raise ValueError("zbuffer must be a contiguous float64 (nx, ny) tensor")
    if view.lens == _lib.LENS_PER_PIXEL:
        for t in (px_pos, px_dir):
            if t is None or t.numel() != nx * ny * 3 or t.dtype != torch.float64 or not t.is_contiguous():
                raise ValueError("per-pixel lens needs contiguous float64 (nx, ny, 3) positions and directions")


def render(bricks: BrickSet, view: _lib.View, order: np.ndarray, kind: int, image: torch.Tensor,
           tf=None, zbuffer: torch.Tensor | None = None, n_samples: int = 1, flags: int = 0,
           counters: torch.Tensor | None = None, error: torch.Tensor | None = None,
           px_pos: torch.Tensor | None = None, px_dir: torch.Tensor | None = None,
           stream: torch.cuda.Stream | None = None, rects: np.ndarray | None = None,
           keep: list | None = None) -> None:
    """Launch ytgb_render for one view.  ``image`` is a (nx, ny, 4) float64
    device tensor updated in place; ``tf`` a PackedTF for volume rendering.
    Device temporaries that must outlive the asynchronous launch are appended
    to ``keep`` when given."""
    dev = bricks.device
    order = np.ascontiguousarray(order, dtype=np.int32)
    check_inputs(bricks, view, order, kind, image, zbuffer, px_pos, px_dir)
    if rects is None:
        rects = bricks.rects(view, order)
    tab = np.empty(order.size * 5, dtype=np.int32)
    tab[: order.size * 4] = rects.ravel()
    tab[order.size * 4:] = order
    if stream is None:
        stream = torch.cuda.current_stream(dev)
    with torch.cuda.stream(stream):
        tab_d = torch.from_numpy(tab).pin_memory().to(dev, non_blocking=True)
    args = _lib.RenderArgs()
    args.kind = int(kind)
    args.n_samples = int(n_samples)
    args.n_order = int(order.size)
    args.flags = int(flags)
    args.view = view
    if px_pos is not None:
        args.view.px_pos = px_pos.data_ptr()
        args.view.px_dir = px_dir.data_ptr()
    args.bricks = bricks.desc.data_ptr()
    args.rects = tab_d.data_ptr()
    args.order = tab_d.data_ptr() + 4 * 4 * order.size
    args.data = bricks.data.data_ptr()
    args.masks = _ptr(bricks.masks)
    args.bounds = bricks.bounds.data_ptr()
    if tf is not None:
        args.tf = tf.header
        args.tf_tables = tf.device_tables(dev).data_ptr()
    args.image = image.data_ptr()
    args.zbuffer = _ptr(zbuffer)
    args.counters = _ptr(counters)
    args.error = _ptr(error)
    st = _lib.lib().ytgb_render(C.byref(args), C.c_void_p(stream.cuda_stream))
    _lib.check(st, "ytgb_render")
    if keep is not None:
        keep.append(tab_d)
    else:
        # the launch reads tab_d asynchronously: keep it alive until done
        stream.synchronize()


def trace(bricks: BrickSet, view: _lib.View, order: np.ndarray, zbuffer=None, px_pos=None, px_dir=None):
    """Per-pixel traversal hash and visit count (ytgb_trace)."""
    dev = bricks.device
    order = np.ascontiguousarray(order, dtype=np.int32)
    rects = bricks.rects(view, order)
    tab = np.concatenate([rects.ravel(), order]).astype(np.int32)
    tab_d = torch.from_numpy(tab).to(dev)
    nx, ny = view.nx, view.ny
    hashes = torch.full((nx * ny,), _lib.FNV_OFFSET, dtype=torch.int64, device=dev)
    counts = torch.zeros(nx * ny, dtype=torch.int64, device=dev)
    args = _lib.RenderArgs()
    args.kind = 0
    args.n_samples = 1
    args.n_order = int(order.size)
    args.view = view
    if px_pos is not None:
        args.view.px_pos = px_pos.data_ptr()
        args.view.px_dir = px_dir.data_ptr()
    args.bricks = bricks.desc.data_ptr()
    args.rects = tab_d.data_ptr()
    args.order = tab_d.data_ptr() + 16 * order.size
    args.data = bricks.data.data_ptr()
    args.bounds = bricks.bounds.data_ptr()
    args.zbuffer = _ptr(zbuffer)
    stream = torch.cuda.current_stream(dev)
    st = _lib.lib().ytgb_trace(C.byref(args), hashes.data_ptr(), counts.data_ptr(), C.c_void_p(stream.cuda_stream))
    _lib.check(st, "ytgb_trace")
    stream.synchronize()
    h = hashes.cpu().numpy().view(np.uint64).reshape(nx, ny)
    return h, counts.cpu().numpy().reshape(nx, ny)
