"""Octree volumes: yt's octree volume source on the device.

yt renders octree datasets (``OctreeVolumeSource``, render_source.py:619-693)
by building an ``_OctreeRayTracing`` over the data's cells
(``OctreeRayTracing``, octree_raytracing.py:19-41: each cell inserted at
``ipos = floor(centre * 2^depth)`` and its level, keyed by its index) and
handing the sampler one PartitionedGrid that packs 14 values per cell: the
8 vertex values, the left edge and the right edge.  The sampler's
``cast_through_octree`` (image_samplers.pyx:202-288) casts every pixel's ray
through the octree and samples each cell it meets.

:class:`Octree` has ``_OctreeRayTracing``'s constructor and ``add_nodes``,
built natively (``ytgb_octree_build``); :class:`OctreeVolume` keeps the
nodes and the cells resident on the device; :func:`render_octree` runs the
``ytgb_render_octree`` launch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

ONODE_DTYPE = np.dtype({"names": ["child", "key", "flags"], "formats": [("<i4", 8), "<i4", "<i4"],
                        "offsets": [0, 32, 36], "itemsize": 40})
assert ONODE_DTYPE.itemsize == C.sizeof(_lib.ONode)


class Octree:
    """``_OctreeRayTracing(LE, RE, depth)`` (_octree_raytracing.pyx:14-31)."""

    def __init__(self, LE, RE, depth):
        self.LE = np.ascontiguousarray(LE, dtype=np.float64).reshape(3)
        self.RE = np.ascontiguousarray(RE, dtype=np.float64).reshape(3)
        self.depth = int(depth)
        self._ipos = []
        self._lvl = []
        self._key = []
        self._nodes = None

    def add_nodes(self, ipos_view, lvl_view, key):
        """Insert cells (``_OctreeRayTracing.add_nodes``): later insertions
        into an existing terminal node overwrite its key, as the reference's
        do."""
        self._ipos.append(np.ascontiguousarray(ipos_view, dtype=np.int32).reshape(-1, 3))
        self._lvl.append(np.ascontiguousarray(lvl_view, dtype=np.int32).ravel())
        self._key.append(np.ascontiguousarray(key, dtype=np.int32).ravel())
        self._nodes = None

    def nodes(self) -> np.ndarray:
        """The nodes in creation order (root first) as ``ONODE_DTYPE``."""
        if self._nodes is None:
            ipos = np.concatenate(self._ipos) if self._ipos else np.zeros((0, 3), np.int32)
            lvl = np.concatenate(self._lvl) if self._lvl else np.zeros(0, np.int32)
            key = np.concatenate(self._key) if self._key else np.zeros(0, np.int32)
            if not (ipos.shape[0] == lvl.size == key.size):
                raise ValueError("ipos, lvl and key must describe the same cells")
            L = _lib.lib()
            h = L.ytgb_octree_build(self.depth, self.LE.ctypes.data, self.RE.ctypes.data, ipos.ctypes.data,
                                    lvl.ctypes.data, key.ctypes.data, lvl.size)
            if not h:
                _lib.check(_lib.ERR_INVALID, "ytgb_octree_build")
            try:
                out = np.zeros(L.ytgb_octree_num_nodes(h), dtype=ONODE_DTYPE)
                _lib.check(L.ytgb_octree_nodes(h, out.ctypes.data), "ytgb_octree_nodes")
            finally:
                L.ytgb_octree_destroy(h)
            self._nodes = out
        return self._nodes


class OctreeVolume:
    """An octree and its cells resident on the device.  ``cells`` is yt's
    (n, 14) float64 layout: 8 vertex values ((i,j,k) C order), left edge,
    right edge; here split into float32 vertex values and float64 edges with
    ``1/(right - left)`` precomputed as cast_through_octree computes it, and a
    float32 copy (left edge as high and low parts, 1/(right - left)) from
    which the samplers form each cell's entry point."""

    def __init__(self, octree: Octree, cells, device="cuda"):
        self.device = torch.device(device)
        self.octree = octree
        cells = np.ascontiguousarray(cells, dtype=np.float64).reshape(-1, 14)
        nodes = octree.nodes()
        keys = nodes["key"][(nodes["flags"] & 1) != 0]
        if keys.size and (keys.min() < 0 or keys.max() >= cells.shape[0]):
            raise ValueError("an octree key is not a row of the cell array")
        le, re = cells[:, 8:11], cells[:, 11:14]
        idds = 1 / (re - le)
        edges = np.concatenate([le, re, idds], axis=1)
        # per cell: the left edge as float32 high and low parts, (float)idds
        leh = le.astype(np.float32)
        edges_f = np.zeros((cells.shape[0], 12), dtype=np.float32)
        edges_f[:, 0:3] = leh
        edges_f[:, 3:6] = (le - leh.astype(np.float64)).astype(np.float32)
        edges_f[:, 6:9] = idds.astype(np.float32)
        self.n_cells = cells.shape[0]
        self.n_nodes = nodes.size
        self.nodes = torch.from_numpy(nodes.view(np.uint8).copy()).to(self.device)
        self.verts = torch.from_numpy(cells[:, :8].astype(np.float32)).to(self.device).reshape(-1)
        self.edges = torch.from_numpy(np.ascontiguousarray(edges)).to(self.device).reshape(-1)
        self.edges_f = torch.from_numpy(edges_f).to(self.device).reshape(-1)
        self.upload_bytes = int(self.nodes.numel() + self.verts.numel() * 4 + self.edges.numel() * 8 +
                                self.edges_f.numel() * 4)

    def args(self) -> _lib.OctreeArgs:
        o = _lib.OctreeArgs()
        o.nodes = self.nodes.data_ptr()
        o.verts = self.verts.data_ptr()
        o.edges = self.edges.data_ptr()
        o.edges_f = self.edges_f.data_ptr()
        o.n_nodes = self.n_nodes
        o.n_cells = self.n_cells
        o.depth = self.octree.depth
        for i in range(3):
            o.dle[i] = float(self.octree.LE[i])
            o.dre[i] = float(self.octree.RE[i])
        return o


def render_octree(vol: OctreeVolume, view: _lib.View, kind: int, image: torch.Tensor, tf=None, n_samples=1,
                  flags=0, counters=None, error=None, light=None, stream=None):
    """One ``ytgb_render_octree`` launch into ``image`` ((nx, ny, 4) float64
    device tensor, updated in place -- or a host array, on a device that
    reads and writes pageable host memory)."""
    from .volume import _f64_contiguous, _ptr, device_reads_host, normalised_light

    if isinstance(image, np.ndarray) and not device_reads_host(vol.device):
        raise ValueError("a host image needs a device that reads pageable host memory")
    if tuple(image.shape) != (view.nx, view.ny, 4) or not _f64_contiguous(image, True):
        raise ValueError(f"image must be a contiguous float64 ({view.nx}, {view.ny}, 4) tensor or array")
    a = _lib.RenderArgs()
    a.kind = int(kind)
    a.n_samples = int(n_samples)
    a.flags = int(flags)
    a.view = view
    a.data = vol.verts.data_ptr()
    if tf is not None:
        a.tf = tf.header
        a.tf_tables = tf.device_tables(vol.device).data_ptr()
    a.image = _ptr(image)
    a.counters = _ptr(counters)
    a.error = _ptr(error)
    if kind == _lib.LIGHT_SOURCE:
        ld, rgba = light if light is not None else ((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0))
        ld = normalised_light(ld)
        for i in range(3):
            a.light_dir[i] = float(ld[i])
        for i in range(4):
            a.light_rgba[i] = float(rgba[i])
    o = vol.args()
    s = stream or torch.cuda.current_stream(vol.device)
    _lib.check(_lib.lib().ytgb_render_octree(C.byref(a), C.byref(o), C.c_void_p(s.cuda_stream)),
               "ytgb_render_octree")
    return a, o


def trace_octree(vol: OctreeVolume, view: _lib.View):
    """Per-pixel traversal hash and count (ytgb_trace_octree)."""
    a = _lib.RenderArgs()
    a.view = view
    a.data = vol.verts.data_ptr()
    a.n_samples = 1
    o = vol.args()
    n = view.nx * view.ny
    h = torch.full((n,), _lib.FNV_OFFSET, dtype=torch.int64, device=vol.device) if _lib.FNV_OFFSET < 2 ** 63 else \
        torch.from_numpy(np.full(n, _lib.FNV_OFFSET, dtype=np.uint64).view(np.int64)).to(vol.device)
    c = torch.zeros(n, dtype=torch.int64, device=vol.device)
    s = torch.cuda.current_stream(vol.device)
    _lib.check(_lib.lib().ytgb_trace_octree(C.byref(a), C.byref(o), h.data_ptr(), c.data_ptr(),
                                            C.c_void_p(s.cuda_stream)), "ytgb_trace_octree")
    torch.cuda.synchronize(vol.device)
    return h.cpu().numpy().view(np.uint64).reshape(view.nx, view.ny), c.cpu().numpy().reshape(view.nx, view.ny)
