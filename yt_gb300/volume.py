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


def _pinned(shape, dtype, device) -> torch.Tensor:
    # page-locked host memory from torch's caching host allocator (reused
    # across calls) when the destination is a GPU
    return torch.empty(shape, dtype=dtype, pin_memory=torch.device(device).type == "cuda")


def brick_parts(pg):
    """(data, mask, left_edge, right_edge, dims) of a PartitionedGrid -- yt's
    own Cython object or :class:`yt_gb300.partitioned_grid.PartitionedGrid`.
    dims come from the mask, which has one entry per cell."""
    mask = pg.source_mask
    if not isinstance(mask, np.ndarray):
        mask = np.asarray(mask)
    return list(pg.my_data), mask, pg.LeftEdge, pg.RightEdge, mask.shape


_MARSHAL: list = []


def _marshal():
    """The native brick scanner (``_ytgb_marshal``, built with libytgb), or
    None where it is not built: the Python scan then does the same work."""
    if not _MARSHAL:
        mod = None
        try:
            import importlib.util

            from .build import MARSHAL

            if MARSHAL.exists():
                spec = importlib.util.spec_from_file_location("_ytgb_marshal", MARSHAL)
                mod = importlib.util.module_from_spec(spec)
                spec.loader.exec_module(mod)
        except ImportError:
            mod = None
        _MARSHAL.append(mod)
    return _MARSHAL[0]


def _scan(bricks, n, dims, le, re, nfields):
    """Brick scan by ``_ytgb_marshal.scan``: (field addresses, field sizes,
    masked bricks, their mask addresses, their mask sizes), filling dims, le,
    re and nfields; None when the module is missing or a brick needs
    converting (the Python scan handles those)."""
    mod = _marshal()
    if mod is None or n == 0:
        return None
    cap = 6 * n
    fptr = np.empty(cap, dtype=np.uintp)
    fsize = np.empty(cap, dtype=np.int64)
    mptr = np.empty(n, dtype=np.uintp)
    msz = np.empty(n, dtype=np.int64)
    got = mod.scan(bricks, cap, fptr.ctypes.data, fsize.ctypes.data, nfields.ctypes.data, dims.ctypes.data,
                   le.ctypes.data, re.ctypes.data, mptr.ctypes.data, msz.ctypes.data)
    if got is False:
        return None
    mk = np.nonzero(msz >= 0)[0]
    return fptr[:got], fsize[:got], mk, mptr[mk], msz[mk]


_READS_HOST: dict = {}


def device_reads_host(device) -> bool:
    """Whether ``device`` reads pageable host memory coherently (a Grace CPU
    and its GPU joined by NVLink-C2C): bricks are then gathered from the
    caller's host arrays by the device (``ytgb_gather_fields``) instead of
    packed on the host and copied.  ``YTGB_HOST_PACK=1`` forces the host
    pack."""
    import os

    dev = torch.device(device)
    if dev.type != "cuda" or os.environ.get("YTGB_HOST_PACK") == "1":
        return False
    idx = dev.index if dev.index is not None else torch.cuda.current_device()
    if idx not in _READS_HOST:
        out = C.c_int32()
        with torch.cuda.device(idx):
            _lib.check(_lib.lib().ytgb_device_reads_host(C.byref(out)), "ytgb_device_reads_host")
        _READS_HOST[idx] = bool(out.value)
    return _READS_HOST[idx]


def _address(a: np.ndarray) -> int:
    """Data address of a C-contiguous array (through the buffer protocol,
    which is cheaper than ``a.ctypes.data``; read-only arrays take the slow
    path)."""
    try:
        return C.addressof(C.c_char.from_buffer(a))
    except (TypeError, ValueError):
        return a.ctypes.data


# numpy view of ytgb_brick (include/ytgb.h), field for field
BRICK_DTYPE = np.dtype({
    "names": ["left_edge", "right_edge", "dds", "idds", "snap", "dims", "n_fields", "data_offset", "field_stride",
              "mask_offset", "bounds_offset", "lef", "ref", "iddsf", "pad"],
    "formats": [("<f8", 3), ("<f8", 3), ("<f8", 3), ("<f8", 3), ("<f8", 3), ("<i4", 3), "<i4", "<i8", "<i8", "<i8",
                "<i8", ("<f4", 3), ("<f4", 3), ("<f4", 3), ("<i4", 5)],
    "offsets": [0, 24, 48, 72, 96, 120, 132, 136, 144, 152, 160, 168, 180, 192, 204],
    "itemsize": 224,
})
assert BRICK_DTYPE.itemsize == C.sizeof(_lib.Brick)


class BrickSet:
    """Bricks ``(data, mask, left_edge, right_edge, dims)`` resident on ``device``
    (PartitionedGrid objects are taken as well).

    On a GPU that reads pageable host memory (``direct``, by default where
    available) the device gathers the float64 fields itself; ``sync=False``
    then returns with that gather in flight on the current stream, and the
    caller keeps the bricks' arrays unchanged until the stream has passed
    it.

    ``data`` is a list of float64 arrays (one per field, any shape; the
    samplers index them exactly as yt does), ``mask`` a uint8 array of
    ``dims`` or None (all ones)."""

    def __init__(self, bricks: Sequence, device="cuda", with_lo=False, direct=None, sync=True):
        self.device = torch.device(device)
        direct = device_reads_host(self.device) if direct is None else bool(direct)
        self.direct = direct
        n = len(bricks)
        self.n = n
        m = max(n, 1)
        dims = np.ones((m, 3), dtype=np.int64)
        le = np.zeros((m, 3))
        re = np.ones((m, 3))
        nfields = np.zeros(m, dtype=np.int64)
        scanned = _scan(bricks, n, dims, le, re, nfields)
        if scanned is not None:
            src, fsize, mk_brick, mptr, mk_size = scanned
        else:
            src, fsize, mk_brick, mptr, mk_size = self._scan_python(bricks, n, dims, le, re, nfields)
        bad = np.nonzero((dims[:n] <= 0).any(axis=1) | (nfields[:n] < 1) | (nfields[:n] > 6))[0]
        if bad.size:
            k = int(bad[0])
            raise ValueError(f"brick {k}: dims must be 3 positive integers and 1 to 6 fields are supported "
                             f"(dims {dims[k].tolist()}, {int(nfields[k])} fields)")
        if mk_brick.size:
            wrong = np.nonzero(mk_size != dims[mk_brick].prod(axis=1))[0]
            if wrong.size:
                raise ValueError(f"brick {int(mk_brick[wrong[0]])}: mask must have prod(dims) entries")
        fstart = np.concatenate([[0], np.cumsum(nfields[:n])]).astype(np.int64)
        sizes_min = np.minimum.reduceat(fsize, fstart[:-1]) if n else fsize
        sizes_max = np.maximum.reduceat(fsize, fstart[:-1]) if n else fsize
        desc, stride, data_off, total, bounds = self._layout(dims, le, re, nfields, sizes_min, sizes_max)
        L = _lib.lib()
        fbrick = np.repeat(np.arange(n), nfields[:n])
        dst_f = (data_off[fbrick] + (np.arange(len(src)) - fstart[fbrick]) * stride[fbrick]).astype(np.int64)
        arena_len = max(total, 4)
        # masks: kept only when some cell is masked out
        mstart = np.concatenate([[0], np.cumsum(self.cells[:n])]).astype(np.int64)
        desc["mask_offset"][:] = -1
        mbuf = None
        mask_gather = None
        if mk_brick.size and direct:
            # the device copies the masks and marks the bricks that need one
            mask_gather = (np.ascontiguousarray(mptr, dtype=np.uintp), np.ascontiguousarray(mk_size, dtype=np.int64),
                           np.ascontiguousarray(mstart[mk_brick]), np.ascontiguousarray(mk_brick, dtype=np.int32))
        elif mk_brick.size:
            msrc = np.ascontiguousarray(mptr, dtype=np.uintp)
            mcnt = np.ascontiguousarray(mk_size, dtype=np.int64)
            mdst = np.ascontiguousarray(mstart[mk_brick])
            ones = C.c_int32()
            _lib.check(L.ytgb_pack_masks(msrc.ctypes.data, mcnt.ctypes.data, mdst.ctypes.data, mk_brick.size, None,
                                         0, C.byref(ones)), "ytgb_pack_masks")
            if not ones.value:
                mbuf = _pinned((max(int(mstart[-1]), 1),), torch.uint8, self.device)
                _lib.check(L.ytgb_pack_masks(msrc.ctypes.data, mcnt.ctypes.data, mdst.ctypes.data, mk_brick.size,
                                             mbuf.data_ptr(), 0, C.byref(ones)), "ytgb_pack_masks")
                desc["mask_offset"][mk_brick] = mdst
        # (on the direct path the device sets the mask offsets of its copy;
        # the host copy, used for the pixel rectangles, keeps -1)
        self.desc_host = desc
        self.host = desc.ctypes.data_as(C.POINTER(_lib.Brick))
        # the small tables first: copies from pageable memory wait for the
        # stream, which is idle before the gather below
        self.bounds = torch.from_numpy(np.ascontiguousarray(bounds)).to(self.device)
        self.desc = torch.from_numpy(desc.view(np.uint8).copy()).to(self.device)
        self.masks = mbuf.to(self.device, non_blocking=True) if mbuf is not None else None
        if mask_gather is not None:
            msrc, mcnt, mdst, mbrick = mask_gather
            mlen = max(int(mstart[-1]), 1)
            self.masks = torch.empty((mlen,), dtype=torch.uint8, device=self.device)
            stream = torch.cuda.current_stream(self.device)
            _lib.check(L.ytgb_gather_masks(msrc.ctypes.data, mcnt.ctypes.data, mdst.ctypes.data, mbrick.ctypes.data,
                                           mbrick.size, self.masks.data_ptr(), mlen, self.desc.data_ptr(), n,
                                           C.c_void_p(stream.cuda_stream)), "ytgb_gather_masks")
        self._range_eps = None
        # with_lo: the padding between fields is zeroed, so that range_eps can
        # take the arena's largest value over the whole buffer
        alloc = torch.zeros if with_lo else torch.empty
        if direct:
            # the device reads the caller's float64 arrays over the CPU-GPU
            # link and writes the float32 arena itself
            buf = alloc((arena_len,), dtype=torch.float32, device=self.device)
            buf_lo = torch.empty((arena_len,), dtype=torch.float32, device=self.device) if with_lo else None
            stream = torch.cuda.current_stream(self.device)
            _lib.check(L.ytgb_gather_fields(src.ctypes.data, fsize.ctypes.data, dst_f.ctypes.data, len(src),
                                            buf.data_ptr(), buf_lo.data_ptr() if buf_lo is not None else None,
                                            arena_len, C.c_void_p(stream.cuda_stream)), "ytgb_gather_fields")
            self.data, self.data_lo = buf, buf_lo
            # the device reads the caller's arrays (and converted copies) and
            # the pointer lists asynchronously: with sync=False the caller
            # keeps the bricks unchanged until the stream has passed here
            self._gather_keep = (src, fsize, dst_f, mask_gather)
            if sync:
                stream.synchronize()
        else:
            # float64 -> float32 gather into the pinned arena, on all host cores
            buf = _pinned((arena_len,), torch.float32, self.device)
            buf_lo = _pinned((arena_len,), torch.float32, self.device) if with_lo else None
            if with_lo:
                buf.zero_()
                _lib.check(L.ytgb_pack_fields_split(src.ctypes.data, fsize.ctypes.data, dst_f.ctypes.data,
                                                    len(src), buf.data_ptr(), buf_lo.data_ptr(), 0),
                           "ytgb_pack_fields_split")
            else:
                _lib.check(L.ytgb_pack_fields(src.ctypes.data, fsize.ctypes.data, dst_f.ctypes.data, len(src),
                                              buf.data_ptr(), 0), "ytgb_pack_fields")
            self.data = buf.to(self.device, non_blocking=True)
            self.data_lo = buf_lo.to(self.device, non_blocking=True) if buf_lo is not None else None
        self.nbytes = int(self.data.numel() * 4)
        self.upload_bytes = int(self.data.numel() * 4 * (2 if with_lo else 1) + self.bounds.numel() * 8 +
                                self.desc.numel() + (self.masks.numel() if self.masks is not None else 0))

    @property
    def range_eps(self) -> float:
        """The scale of the float64 range decisions (``ytgb_render_args.
        range_eps``): M * 2^-24, M the largest finite |value| of the arena,
        computed from the device arena on first use (one synchronising
        reduction) and kept; 0 without ``data_lo`` (float32 decisions)."""
        if self.data_lo is None:
            return 0.0
        if self._range_eps is None:
            m = float(torch.nan_to_num(self.data.abs(), nan=0.0, posinf=0.0).max()) if self.data.numel() else 0.0
            self._range_eps = m * 2.0 ** -24
        return self._range_eps

    def data_changed(self):
        """Forget range_eps after the arena was (re)written in place."""
        self._range_eps = None

    def _scan_python(self, bricks, n, dims, le, re, nfields):
        """The brick scan in Python (any array types): field addresses and
        sizes, masked bricks with their mask addresses and sizes; fills dims,
        le, re and nfields.  Converted arrays are kept on the instance until
        the arena has been written."""
        f64 = np.dtype(np.float64)
        u8 = np.dtype(np.uint8)
        dims_l, le_l, re_l, nf_l = [], [], [], []
        keep = []                      # arrays whose addresses are taken
        fptr, fsz = [], []             # every field of every brick, in order
        mk_k, mptr, msz = [], [], []   # bricks with a mask
        addr = _address
        for k, item in enumerate(bricks):
            data, mask, le_k, re_k, dims_k = item if isinstance(item, tuple) else brick_parts(item)
            dims_l.append(dims_k)
            le_l.append(le_k)
            re_l.append(re_k)
            nf_l.append(len(data))
            for d in data:
                if not (type(d) is np.ndarray and d.dtype == f64 and d.flags.c_contiguous):
                    d = np.ascontiguousarray(d, dtype=np.float64)
                keep.append(d)
                fptr.append(addr(d))
                fsz.append(d.size)
            if mask is not None:
                mk = mask
                if not (type(mk) is np.ndarray and mk.dtype == u8 and mk.flags.c_contiguous):
                    mk = np.asarray(mk)
                    mk = np.ascontiguousarray(mk.view(np.uint8) if mk.dtype == np.bool_ else mk, dtype=np.uint8)
                keep.append(mk)
                mk_k.append(k)
                mptr.append(addr(mk))
                msz.append(mk.size)
        if n:
            try:
                dims[:n] = np.array(dims_l, dtype=np.int64).reshape(n, 3)
            except ValueError:
                raise ValueError("brick dims must be 3 positive integers") from None
            le[:n] = np.array(le_l, dtype=np.float64).reshape(n, -1)[:, :3]
            re[:n] = np.array(re_l, dtype=np.float64).reshape(n, -1)[:, :3]
            nfields[:n] = nf_l
        self._keep = keep
        return (np.array(fptr, dtype=np.uintp), np.array(fsz, dtype=np.int64), np.array(mk_k, dtype=np.int64),
                np.array(mptr, dtype=np.uintp), np.array(msz, dtype=np.int64))

    @classmethod
    def on_device(cls, dims, le, re, device="cuda", n_fields=1, with_lo=False):
        """Bricks of the given geometry whose vertex-centred fields are
        written on the device (``AMRKDTree.device_brickset``): descriptors and
        boundary tables as usual, a float32 arena of (dims+1)^3 values per
        field allocated on the device and left unfilled, no masks."""
        self = cls.__new__(cls)
        self.device = torch.device(device)
        d = np.ascontiguousarray(dims, dtype=np.int64).reshape(-1, 3)
        n = d.shape[0]
        self.n = n
        m = max(n, 1)
        if n and (d <= 0).any():
            raise ValueError("brick dims must be positive")
        dims_m = np.ones((m, 3), dtype=np.int64)
        le_m = np.zeros((m, 3))
        re_m = np.ones((m, 3))
        dims_m[:n] = d
        le_m[:n] = np.asarray(le, dtype=np.float64).reshape(n, 3)
        re_m[:n] = np.asarray(re, dtype=np.float64).reshape(n, 3)
        nfields = np.zeros(m, dtype=np.int64)
        nfields[:n] = n_fields
        verts = (d + 1).prod(axis=1)
        desc, stride, data_off, total, bounds = self._layout(dims_m, le_m, re_m, nfields, verts, verts)
        desc["mask_offset"][:] = -1
        self.desc_host = desc
        self.host = desc.ctypes.data_as(C.POINTER(_lib.Brick))
        self.data = (torch.zeros if with_lo else torch.empty)(max(total, 4), dtype=torch.float32, device=self.device)
        self.data_lo = torch.empty_like(self.data) if with_lo else None
        self._range_eps = None
        self.masks = None
        self.bounds = torch.from_numpy(np.ascontiguousarray(bounds)).to(self.device)
        self.desc = torch.from_numpy(desc.view(np.uint8).copy()).to(self.device)
        self.nbytes = int(self.data.numel() * 4)
        self.upload_bytes = int(self.bounds.numel() * 8 + self.desc.numel())
        return self

    def _layout(self, dims, le, re, nfields, sizes_min, sizes_max):
        """Descriptors, arena strides/offsets and cell-boundary tables of
        bricks with the given geometry and per-field element counts
        (``ytgb_brick_layout``: PartitionedGrid.__cinit__'s dds and idds,
        partitioned_grid.pyx:54-55, and the k*dds + le tables walk_volume
        forms, grid_traversal.pyx:106-108, in the same float64 operations)."""
        n, m = self.n, max(self.n, 1)
        desc = np.zeros(m, dtype=BRICK_DTYPE)
        self.cells = dims.prod(axis=1)
        self.verts = (dims + 1).prod(axis=1)
        self.min_elems = np.zeros(m, dtype=np.int64)
        self.min_elems[:n] = sizes_min
        nb_total = int((dims[:n] + 1).sum())
        bounds = np.zeros(max(nb_total, 1))
        total = C.c_int64(0)
        if n:
            smax = np.ascontiguousarray(sizes_max, dtype=np.int64)
            _lib.check(_lib.lib().ytgb_brick_layout(
                n, np.ascontiguousarray(dims[:n]).ctypes.data, np.ascontiguousarray(le[:n]).ctypes.data,
                np.ascontiguousarray(re[:n]).ctypes.data, np.ascontiguousarray(nfields[:n]).ctypes.data,
                smax.ctypes.data, desc.ctypes.data, bounds.ctypes.data, bounds.size, C.byref(total)),
                "ytgb_brick_layout")
        return desc, desc["field_stride"].copy(), desc["data_offset"].copy(), int(total.value), bounds

    def rects(self, view: _lib.View, order: np.ndarray) -> np.ndarray:
        """Per-order-entry pixel rectangles (ytgb_brick_rects)."""
        order = np.ascontiguousarray(order, dtype=np.int32)
        out = np.empty((order.size, 4), dtype=np.int32)
        st = _lib.lib().ytgb_brick_rects(C.byref(view), self.host, self.n, order.ctypes.data, order.size,
                                         out.ctypes.data)
        _lib.check(st, "ytgb_brick_rects")
        return out


def normalised_light(light_dir) -> np.ndarray:
    """LightSourceRenderSampler.__cinit__'s normalisation (image_samplers.pyx:
    530-532), in float64."""
    ld = np.asarray(light_dir, dtype=np.float64)
    return ld / np.sqrt(ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2])


def set_light(args, bricks, light):
    """Fill the light-source fields of a ytgb_render_args: ``light`` is
    (light_dir, light_rgba) or None for yt's defaults ((1,1,1), (1,1,1,1))."""
    ld, rgba = light if light is not None else ((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0))
    ld = normalised_light(ld)
    for i in range(3):
        args.light_dir[i] = float(ld[i])
    for i in range(4):
        args.light_rgba[i] = float(rgba[i])
    set_range(args, bricks)


def set_range(args, bricks):
    """The arena's float32 rounding errors and their scale, for the float64
    range decisions near a transfer-function bound (volume rendering and
    light source; none when the bricks carry no ``data_lo``)."""
    args.data_lo = _ptr(bricks.data_lo)
    args.range_eps = bricks.range_eps


def _ptr(t):
    if t is None:
        return None
    return t.ctypes.data if isinstance(t, np.ndarray) else t.data_ptr()


def _f64_contiguous(t, writeable=False) -> bool:
    if isinstance(t, np.ndarray):
        return t.dtype == np.float64 and t.flags.c_contiguous and (t.flags.writeable or not writeable)
    return t.dtype == torch.float64 and t.is_contiguous()


def _numel(t) -> int:
    return t.size if isinstance(t, np.ndarray) else t.numel()


def check_inputs(bricks: BrickSet, view: _lib.View, order, kind, image=None, zbuffer=None, px_pos=None,
                 px_dir=None):
    """Reject inputs the kernel would index out of bounds: the vertex-centred
    samplers read (dims+1)^3 values per field, the projection samplers
    dims^3 (image_samplers.pyx:341, :384-385, :465-466)."""
    if order.size and (order.min() < 0 or order.max() >= bricks.n):
        raise ValueError("order entry out of range")
    used = np.unique(order) if order.size else order
    need = (bricks.verts if kind in (_lib.VOLUME_RENDER, _lib.INTERPOLATED_PROJECTION, _lib.LIGHT_SOURCE)
            else bricks.cells)
    short = used[bricks.min_elems[used] < need[used]] if used.size else used
    if short.size:
        k = int(short[0])
        raise ValueError(f"brick {k} has {bricks.min_elems[k]} values per field; this sampler reads {need[k]}")
    nx, ny = view.nx, view.ny
    for t in (image, zbuffer):
        # host arrays: only where the device reads and writes them in place
        if isinstance(t, np.ndarray) and not device_reads_host(bricks.device):
            raise ValueError("host image and zbuffer arrays need a device that reads pageable host memory")
    if image is not None and tuple(image.shape) != (nx, ny, 4) or (image is not None and not _f64_contiguous(image, True)):
        raise ValueError(f"image must be a contiguous float64 ({nx}, {ny}, 4) tensor or array")
    if zbuffer is not None and (_numel(zbuffer) != nx * ny or not _f64_contiguous(zbuffer)):
        raise ValueError("zbuffer must be a contiguous float64 (nx, ny) tensor or array")
    if view.lens == _lib.LENS_PER_PIXEL:
        for t in (px_pos, px_dir):
            if isinstance(t, np.ndarray):
                if t.size != nx * ny * 3 or t.dtype != np.float64 or not t.flags.c_contiguous:
                    raise ValueError("per-pixel lens needs contiguous float64 (nx, ny, 3) positions and directions")
                if not device_reads_host(bricks.device):
                    raise ValueError("host per-pixel ray arrays need a device that reads pageable host memory")
            elif t is None or t.numel() != nx * ny * 3 or t.dtype != torch.float64 or not t.is_contiguous():
                raise ValueError("per-pixel lens needs contiguous float64 (nx, ny, 3) positions and directions")


def _table(rects: np.ndarray, order: np.ndarray) -> np.ndarray:
    tab = np.empty(order.size * 5, dtype=np.int32)
    tab[: order.size * 4] = np.asarray(rects, dtype=np.int32).ravel()
    tab[order.size * 4:] = order
    return tab


def _view_key(view: _lib.View) -> bytes:
    """The view's geometry as bytes: every field the pixel rectangles depend
    on (image size, lens, camera vectors, bounds, widths, camera data), not
    the per-pixel ray pointers."""
    return bytes(view)[: _lib.View.px_pos.offset]


class RenderTables:
    """The table one render reads -- each order entry's pixel rectangle (4
    int32), then the order -- on the device, with the host copies of the
    order and of the view geometry it was made for.  The kernel indexes the
    bricks by the device copy of the order and culls each brick to its
    stored rectangle, so render() accepts the table only for that same order
    and view: a camera that moved while the order stayed the same would
    otherwise cull bricks from pixels they now cover."""

    def __init__(self, table: torch.Tensor, order: np.ndarray, view_key: bytes):
        self.table = table
        self.order = order.copy()
        self.view_key = view_key


def render_tables(bricks: BrickSet, view: _lib.View, order: np.ndarray, rects: np.ndarray | None = None
                  ) -> RenderTables:
    """A :class:`RenderTables` for ``render(..., tables=)``, to keep resident
    across launches of the same view and order."""
    order = np.ascontiguousarray(order, dtype=np.int32)
    if order.size and (order.min() < 0 or order.max() >= bricks.n):
        raise ValueError("order entry out of range")
    if rects is None:
        rects = bricks.rects(view, order)
    if np.shape(rects) != (order.size, 4):
        raise ValueError("rects must hold 4 entries per order entry")
    return RenderTables(torch.from_numpy(_table(rects, order)).to(bricks.device), order, _view_key(view))


def render(bricks: BrickSet, view: _lib.View, order: np.ndarray, kind: int, image: torch.Tensor,
           tf=None, zbuffer: torch.Tensor | None = None, n_samples: int = 1, flags: int = 0,
           counters: torch.Tensor | None = None, error: torch.Tensor | None = None,
           px_pos: torch.Tensor | None = None, px_dir: torch.Tensor | None = None,
           stream: torch.cuda.Stream | None = None, rects: np.ndarray | None = None,
           keep: list | None = None, light=None, tables: RenderTables | None = None) -> None:
    """Launch ytgb_render for one view.  ``image`` is a (nx, ny, 4) float64
    device tensor updated in place -- or, on a device that reads and writes
    pageable host memory, a host array (likewise ``zbuffer``); ``tf`` a
    PackedTF for volume rendering; ``tables`` the resident table of
    :func:`render_tables` for this view and order (else it is built from
    ``rects`` and uploaded for this launch).
    Device temporaries that must outlive the asynchronous launch are appended
    to ``keep`` when given."""
    dev = bricks.device
    order = np.ascontiguousarray(order, dtype=np.int32)
    check_inputs(bricks, view, order, kind, image, zbuffer, px_pos, px_dir)
    if stream is None:
        stream = torch.cuda.current_stream(dev)
    if tables is None:
        if rects is None:
            rects = bricks.rects(view, order)
        with torch.cuda.stream(stream):
            tab_d = torch.from_numpy(_table(rects, order)).pin_memory().to(dev, non_blocking=True)
    else:
        t = tables.table if isinstance(tables, RenderTables) else None
        if (t is None or not np.array_equal(tables.order, order) or t.device.type != "cuda"
                or (dev.index is not None and t.device.index != dev.index)):
            raise ValueError(f"tables must come from render_tables for this order, on {dev}")
        if tables.view_key != _view_key(view):
            raise ValueError("tables were made for another view: their pixel rectangles do not fit this camera")
        tab_d = t
    args = _lib.RenderArgs()
    args.kind = int(kind)
    args.n_samples = int(n_samples)
    args.n_order = int(order.size)
    args.flags = int(flags)
    args.view = view
    if px_pos is not None:
        # device tensors, or host arrays the device reads in place
        args.view.px_pos = px_pos.ctypes.data if isinstance(px_pos, np.ndarray) else px_pos.data_ptr()
        args.view.px_dir = px_dir.ctypes.data if isinstance(px_dir, np.ndarray) else px_dir.data_ptr()
    args.bricks = bricks.desc.data_ptr()
    args.rects = tab_d.data_ptr()
    args.order = tab_d.data_ptr() + 4 * 4 * order.size
    args.data = bricks.data.data_ptr()
    args.masks = _ptr(bricks.masks)
    args.bounds = bricks.bounds.data_ptr()
    if tf is not None:
        args.tf = tf.header
        args.tf_tables = tf.device_tables(dev).data_ptr()
    args.image = _ptr(image)
    args.zbuffer = _ptr(zbuffer)
    if kind == _lib.LIGHT_SOURCE:
        set_light(args, bricks, light)
    elif kind == _lib.VOLUME_RENDER:
        set_range(args, bricks)
    args.counters = _ptr(counters)
    args.error = _ptr(error)
    st = _lib.lib().ytgb_render(C.byref(args), C.c_void_p(stream.cuda_stream))
    _lib.check(st, "ytgb_render")
    if keep is not None:
        keep.append(tab_d)
    elif tables is None:
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
