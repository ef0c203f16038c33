"""AMR kd-tree bricks (the producer side of the sampler path).

``AMRKDTree`` mirrors yt's (``yt/utilities/amr_kdtree/amr_kdtree.py``): the
tree is built level by level over the grids (``Tree.build`` :109-118) with
yt's split rules, here in native C++ (``ytgb_kdtree_build``); each leaf
becomes a brick of the finest grid covering it, with vertex-centred data
(``get_vertex_centered_data(no_ghost=True)``, ``grid_patch.py:270-296``),
``log10`` where requested (values <= 0 become NaN, :346-352) and the slice
``[li:ri+1]`` (:325-374).  ``viewpoint_order`` gives the brick order of
``traverse(viewpoint)`` (``amr_kdtools.pyx:612-755``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .partitioned_grid import PartitionedGrid


def vertex_centred(cell: np.ndarray) -> np.ndarray:
    """ghost_zone_interpolate(1, cell, [0.5]*3, vertex, [0]*3)
    (interpolators.pyx:177-226) for the no-ghost-zone case.  With rf = 1 the
    weights are exactly {-0.5, 0.5, 1.5} per axis; the eight products are
    summed in the reference's order, so the result is bit-identical."""
    cell = np.ascontiguousarray(cell, dtype=np.float64)
    w = []
    for n in cell.shape:
        o = np.arange(n + 1, dtype=np.float64)
        ropos = o - 0.5
        ii = np.clip(ropos.astype(np.int64), 0, n - 2)
        xp = ropos - ii
        w.append((ii, xp, 1.0 - xp))
    (ii, xp, xm), (ij, yp, ym), (ik, zp, zm) = w
    I0, I1 = ii[:, None, None], ii[:, None, None] + 1
    J0, J1 = ij[None, :, None], ij[None, :, None] + 1
    K0, K1 = ik[None, None, :], ik[None, None, :] + 1
    XP, XM = xp[:, None, None], xm[:, None, None]
    YP, YM = yp[None, :, None], ym[None, :, None]
    ZP, ZM = zp[None, None, :], zm[None, None, :]
    c = cell
    out = c[I0, J0, K0] * (XM * YM * ZM)
    out = out + c[I1, J0, K0] * (XP * YM * ZM)
    out = out + c[I0, J1, K0] * (XM * YP * ZM)
    out = out + c[I0, J0, K1] * (XM * YM * ZP)
    out = out + c[I1, J0, K1] * (XP * YM * ZP)
    out = out + c[I0, J1, K1] * (XM * YP * ZP)
    out = out + c[I1, J1, K0] * (XP * YP * ZM)
    out = out + c[I1, J1, K1] * (XP * YP * ZP)
    return out


class AMRKDTree:
    """kd bricks over a list of grids (objects with ``id``, ``level``,
    ``left_edge``, ``right_edge``, ``dims``, ``data``)."""

    def __init__(self, grids, log_field=True):
        self.grids = list(grids)
        self.by_id = {g.id: g for g in self.grids}
        self.log_field = log_field
        n = len(self.grids)
        self._gles = np.ascontiguousarray([g.left_edge for g in self.grids], dtype=np.float64).reshape(n, 3)
        self._gres = np.ascontiguousarray([g.right_edge for g in self.grids], dtype=np.float64).reshape(n, 3)
        self._gids = np.ascontiguousarray([g.id for g in self.grids], dtype=np.int64)
        self._lvls = np.ascontiguousarray([g.level for g in self.grids], dtype=np.int32)
        L = _lib.lib()
        self._tree = L.ytgb_kdtree_build(n, self._gles.ctypes.data, self._gres.ctypes.data,
                                         self._gids.ctypes.data, self._lvls.ctypes.data)
        if not self._tree:
            _lib.check(_lib.ERR_INVALID, "ytgb_kdtree_build")
        nl = L.ytgb_kdtree_num_leaves(self._tree)
        self.leaf_le = np.zeros((nl, 3), dtype=np.float64)
        self.leaf_re = np.zeros((nl, 3), dtype=np.float64)
        self.leaf_grid = np.zeros(nl, dtype=np.int64)
        _lib.check(L.ytgb_kdtree_leaves(self._tree, self.leaf_le.ctypes.data, self.leaf_re.ctypes.data,
                                        self.leaf_grid.ctypes.data), "ytgb_kdtree_leaves")
        self._vcd = {}
        self._bricks = None

    def __del__(self):
        t = getattr(self, "_tree", None)
        if t:
            _lib.lib().ytgb_kdtree_destroy(t)
            self._tree = None

    @property
    def num_bricks(self) -> int:
        return int(self.leaf_grid.size)

    def viewpoint_order(self, viewpoint) -> np.ndarray:
        vp = np.ascontiguousarray(viewpoint, dtype=np.float64)
        out = np.empty(self.num_bricks, dtype=np.int32)
        _lib.check(_lib.lib().ytgb_kdtree_viewpoint_order(self._tree, vp.ctypes.data, out.ctypes.data),
                   "ytgb_kdtree_viewpoint_order")
        return out

    def viewpoint_orders(self, viewpoints) -> np.ndarray:
        vps = np.ascontiguousarray(viewpoints, dtype=np.float64).reshape(-1, 3)
        out = np.empty((vps.shape[0], self.num_bricks), dtype=np.int32)
        _lib.check(_lib.lib().ytgb_kdtree_viewpoint_orders(self._tree, vps.shape[0], vps.ctypes.data,
                                                           out.ctypes.data), "ytgb_kdtree_viewpoint_orders")
        return out

    def _vertex(self, g):
        v = self._vcd.get(g.id)
        if v is None:
            v = vertex_centred(g.data)
            if self.log_field:
                v = v.astype("float64")
                v[v <= 0] = np.nan
                v = np.log10(v)
            self._vcd[g.id] = v
        return v

    def brick(self, k: int):
        """(data, mask, left_edge, right_edge, dims) of leaf k
        (get_brick_data, amr_kdtree.py:325-374)."""
        g = self.by_id[int(self.leaf_grid[k])]
        dds = g.dds
        gle = g.left_edge
        nle, nre = self.leaf_le[k], self.leaf_re[k]
        li = np.rint((nle - gle) / dds).astype("int32")
        ri = np.rint((nre - gle) / dds).astype("int32")
        dims = ri - li
        v = self._vertex(g)
        data = [v[li[0]: ri[0] + 1, li[1]: ri[1] + 1, li[2]: ri[2] + 1].copy()]
        mask = np.ones(dims, dtype="uint8")
        return data, mask, nle.copy(), nre.copy(), dims.astype("int64")

    def bricks(self):
        if self._bricks is None:
            self._bricks = [self.brick(k) for k in range(self.num_bricks)]
        return self._bricks

    def leaf_slices(self):
        """(grid index, li, dims) of every leaf: the slice get_brick_data
        takes from its grid (amr_kdtree.py:329-335)."""
        gidx = {g.id: i for i, g in enumerate(self.grids)}
        lg = np.array([gidx[int(i)] for i in self.leaf_grid], dtype=np.int32)
        dds = np.array([np.asarray(g.dds, dtype=np.float64) for g in self.grids]).reshape(-1, 3)[lg]
        gle = self._gles[lg]
        li = np.rint((self.leaf_le - gle) / dds).astype("int32")
        ri = np.rint((self.leaf_re - gle) / dds).astype("int32")
        return lg, li, (ri - li).astype(np.int64)

    def device_brickset(self, device="cuda", stream=None, with_lo=False):
        """The bricks as a :class:`~yt_gb300.volume.BrickSet` prepared on the
        device: the grids' cell data is uploaded once and every leaf's
        vertex-centred (and log10'd) slice is computed there
        (``ytgb_vertex_bricks``) instead of on the host (:meth:`brick`).
        The vertex values are bit-identical to the host path's; with
        ``log_field`` the device log10 may differ from numpy's in the last
        float64 bit, which reaches the float32 brick value only when it sits
        on a float32 rounding boundary.  ``with_lo`` also fills the values'
        float32 rounding errors (the light-source sampler's gradient)."""
        import torch

        from .volume import BrickSet, _pinned

        dev = torch.device(device)
        lg, li, dims = self.leaf_slices()
        gshape = np.array([np.shape(g.data) for g in self.grids], dtype=np.int64).reshape(-1, 3)
        if (gshape < 2).any():
            raise ValueError("device brick preparation needs grids of at least 2 cells per axis")
        if (li < 0).any() or (li + dims > gshape[lg]).any():
            raise ValueError("a kd leaf does not lie inside its grid")
        bs = BrickSet.on_device(dims, self.leaf_le, self.leaf_re, dev, with_lo=with_lo)
        gsize = gshape.prod(axis=1)
        goff = np.concatenate([[0], np.cumsum(gsize)]).astype(np.int64)
        host = _pinned((max(int(goff[-1]), 1),), torch.float64, dev)
        hnp = host.numpy()
        for k, g in enumerate(self.grids):
            hnp[goff[k]: goff[k + 1]] = np.asarray(g.data, dtype=np.float64).ravel()
        s = stream or torch.cuda.current_stream(dev)
        with torch.cuda.stream(s):
            cells = host.to(dev, non_blocking=True)
            meta_i64 = torch.from_numpy(goff[:-1].copy()).to(dev, non_blocking=False)
            meta_i32 = torch.from_numpy(np.concatenate([gshape.ravel(), lg, li.ravel()]).astype(np.int32)).to(dev)
        error = torch.zeros(1, dtype=torch.int32, device=dev)
        ng, nb = len(self.grids), int(lg.size)
        base = meta_i32.data_ptr()
        L = _lib.lib()
        _lib.check(L.ytgb_vertex_bricks(cells.data_ptr(), int(goff[-1]), meta_i64.data_ptr(), base, ng,
                                        base + 4 * 3 * ng, base + 4 * (3 * ng + nb), bs.desc.data_ptr(), nb, 0,
                                        int(bool(self.log_field)), bs.data.data_ptr(), bs.data.numel(),
                                        error.data_ptr(), C.c_void_p(s.cuda_stream),
                                        bs.data_lo.data_ptr() if bs.data_lo is not None else None),
                   "ytgb_vertex_bricks")
        _lib.check(L.ytgb_check_error(error.data_ptr(), s.cuda_stream), "ytgb_vertex_bricks")
        bs.data_changed()
        self.device_upload_bytes = int(cells.numel() * 8 + meta_i64.numel() * 8 + meta_i32.numel() * 4 +
                                       bs.upload_bytes)
        return bs

    def traverse(self, viewpoint=None):
        """PartitionedGrid bricks in kd order (AMRKDTree.traverse, :248-250)."""
        order = range(self.num_bricks) if viewpoint is None else self.viewpoint_order(viewpoint)
        bs = self.bricks()
        for k in order:
            data, mask, le, re, dims = bs[k]
            yield PartitionedGrid(int(self.leaf_grid[k]), data, mask, le, re, dims)
