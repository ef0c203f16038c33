"""Transfer functions with yt's table semantics, and their device packing.

The classes reproduce the tables yt's transfer functions hand to the sampler
(``yt/visualization/volume_rendering/transfer_functions.py``):

* ``TransferFunction``            :8-79  (x = linspace(bounds, nbins), Gaussians)
* ``MultiVariateTransferFunction`` :249-360 (field tables, channel links)
* ``ColorTransferFunction``       :365-408, add_layers :822-894
* ``ProjectionTransferFunction``  :921-961

Any object with yt's attributes (``n_field_tables``, ``tables[i].y``,
``tables[i].x_bounds``, ``field_ids``, ``weight_field_ids``,
``weight_table_ids``, ``field_table_ids``, ``grey_opacity``) -- including
yt's own transfer functions -- can be packed by :func:`pack`.

``ColorTransferFunction.add_layers`` samples colours from a built-in
analytic colour map (matplotlib colour maps are not a dependency); the
layer positions, widths and alphas follow yt exactly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class TransferFunction:
    def __init__(self, x_bounds, nbins=256):
        self.pass_through = 0
        self.nbins = nbins
        self.x_bounds = [np.float64(xb) for xb in x_bounds]
        self.x = np.linspace(self.x_bounds[0], self.x_bounds[1], nbins, dtype="float64")
        self.y = np.zeros(nbins, dtype="float64")
        self.features = []

    def add_gaussian(self, location, width, height):
        """y = max(y, h exp(-(x-x0)^2 / w)), clipped at 0 (transfer_functions.py:46-79)."""
        vals = height * np.exp(-((self.x - location) ** 2.0) / width)
        self.y = np.clip(np.maximum(vals, self.y), 0.0, np.inf)
        self.features.append(("gaussian", location, width, height))

    def add_step(self, start, stop, value):
        """y = max(y, value) for start <= x <= stop (transfer_functions.py:121-152)."""
        vals = np.zeros(self.x.shape, "float64")
        vals[(self.x >= start) & (self.x <= stop)] = value
        self.y = np.clip(np.maximum(vals, self.y), 0.0, np.inf)
        self.features.append(("step", start, stop, value))

    def clear(self):
        self.y[:] = 0.0
        self.features = []


class MultiVariateTransferFunction:
    def __init__(self, grey_opacity=False):
        self.n_field_tables = 0
        self.tables = []
        self.field_ids = [0] * 6
        self.weight_field_ids = [-1] * 6
        self.field_table_ids = [0] * 6
        self.weight_table_ids = [-1] * 6
        self.grad_field = -1
        self.light_source_v = self.light_source_c = np.zeros(3, "float64")
        self.grey_opacity = grey_opacity

    def add_field_table(self, table, field_id, weight_field_id=-1, weight_table_id=-1):
        self.tables.append(table)
        self.field_ids[self.n_field_tables] = field_id
        self.weight_field_ids[self.n_field_tables] = weight_field_id
        self.weight_table_ids[self.n_field_tables] = weight_table_id
        self.n_field_tables += 1

    def link_channels(self, table_id, channels=0):
        for c in np.atleast_1d(channels):
            self.field_table_ids[int(c)] = table_id


def builtin_colormap(rel: float):
    """A smooth analytic RGB colour ramp on [0, 1] (stand-in for a matplotlib
    colour map; colours do not change the sampler's cost)."""
    rel = float(np.clip(rel, 0.0, 1.0))
    r = np.clip(1.5 * rel - 0.25, 0.0, 1.0)
    g = np.clip(1.0 - 2.0 * abs(rel - 0.5), 0.0, 1.0)
    b = np.clip(1.25 - 1.5 * rel, 0.0, 1.0)
    return float(r), float(g), float(b), 1.0


class ColorTransferFunction(MultiVariateTransferFunction):
    def __init__(self, x_bounds, nbins=256, grey_opacity=False):
        MultiVariateTransferFunction.__init__(self)
        self.x_bounds = [np.float64(xb) for xb in x_bounds]
        self.nbins = nbins
        self.red = TransferFunction(self.x_bounds, nbins)
        self.green = TransferFunction(self.x_bounds, nbins)
        self.blue = TransferFunction(self.x_bounds, nbins)
        self.alpha = TransferFunction(self.x_bounds, nbins)
        self.funcs = (self.red, self.green, self.blue, self.alpha)
        self.grey_opacity = grey_opacity
        self.features = []
        for i, tf in enumerate(self.funcs[:3]):
            self.add_field_table(tf, 0, weight_table_id=3)
            self.link_channels(i, i)
        self.add_field_table(self.funcs[3], 0)
        self.link_channels(3, 3)

    def add_gaussian(self, location, width, height):
        for tf, v in zip(self.funcs, height, strict=True):
            tf.add_gaussian(location, width, v)
        self.features.append(("gaussian", location, width, tuple(height)))

    def add_step(self, start, stop, value):
        for tf, v in zip(self.funcs, value, strict=True):
            tf.add_step(start, stop, v)

    def sample_colormap(self, v, w, alpha=None, colormap=None, col_bounds=None):
        v = np.float64(v)
        if col_bounds is None:
            rel = (v - self.x_bounds[0]) / (self.x_bounds[1] - self.x_bounds[0])
        else:
            rel = (v - col_bounds[0]) / (col_bounds[1] - col_bounds[0])
        cmap = colormap if callable(colormap) else builtin_colormap
        r, g, b, a = cmap(rel)
        if alpha is None:
            alpha = a
        self.add_gaussian(v, w, [r, g, b, alpha])

    def add_layers(self, N, w=None, mi=None, ma=None, alpha=None, colormap=None, col_bounds=None):
        """Evenly spaced Gaussian layers (transfer_functions.py:822-894)."""
        if col_bounds is None:
            dist = self.x_bounds[1] - self.x_bounds[0]
            if mi is None:
                mi = self.x_bounds[0] + dist / (10.0 * N)
            if ma is None:
                ma = self.x_bounds[1] - dist / (10.0 * N)
        else:
            dist = col_bounds[1] - col_bounds[0]
            if mi is None:
                mi = col_bounds[0] + dist / (10.0 * N)
            if ma is None:
                ma = col_bounds[1] - dist / (10.0 * N)
        if w is None:
            w = 0.001 * (ma - mi) / N
            w = max(w, 1.0 / self.nbins)
        if alpha is None and self.grey_opacity:
            alpha = np.ones(N, dtype="float64")
        elif alpha is None and not self.grey_opacity:
            alpha = np.logspace(-3, 0, N)
        for v, a in zip(np.mgrid[mi: ma: N * 1j], alpha, strict=True):
            self.sample_colormap(v, w, a, colormap=colormap, col_bounds=col_bounds)


class ProjectionTransferFunction(MultiVariateTransferFunction):
    def __init__(self, x_bounds=(-1e60, 1e60), n_fields=1):
        if n_fields > 3:
            raise NotImplementedError(f"supplied ${n_fields} but n_fields > 3 not implemented.")
        MultiVariateTransferFunction.__init__(self)
        self.x_bounds = [np.float64(xb) for xb in x_bounds]
        self.nbins = 2
        self.linear_mapping = TransferFunction(self.x_bounds, 2)
        self.linear_mapping.pass_through = 1
        self.link_channels(0, [0, 1, 2])
        for i in range(n_fields):
            self.add_field_table(self.linear_mapping, i)
            self.link_channels(i, i)
        self.link_channels(n_fields, [3, 4, 5])


class PackedTF:
    """A transfer function packed for the device: the ``ytgb_tf`` header (by
    value in every render) and the float32 table buffer."""

    def __init__(self, header: _lib.TF, tables: np.ndarray):
        self.header = header
        self.tables = tables
        self._dev = {}

    def device_tables(self, device):
        import torch

        key = str(device)
        t = self._dev.get(key)
        if t is None:
            t = torch.from_numpy(self.tables).to(device)
            self._dev[key] = t
        return t


def pack(tf_obj) -> PackedTF:
    """ytgb_tf_pack over yt's FieldInterpolationTable set
    (VolumeRenderSampler.__cinit__, image_samplers.pyx:425-447)."""
    n_fits = int(tf_obj.n_field_tables)
    assert n_fits <= 6
    ys = [np.ascontiguousarray(tf_obj.tables[i].y, dtype=np.float64) for i in range(n_fits)]
    nb = (C.c_int32 * 6)(*([y.shape[0] for y in ys] + [0] * (6 - n_fits)))
    vals = (C.POINTER(C.c_double) * 6)(*[y.ctypes.data_as(C.POINTER(C.c_double)) for y in ys])
    bounds = np.zeros(12, dtype=np.float64)
    for i in range(n_fits):
        bounds[2 * i] = float(tf_obj.tables[i].x_bounds[0])
        bounds[2 * i + 1] = float(tf_obj.tables[i].x_bounds[1])
    ids6 = lambda xs: (C.c_int32 * 6)(*[int(x) for x in list(xs)[:6]] + [0] * (6 - len(list(xs)[:6])))  # noqa: E731
    nbmax = max([y.shape[0] for y in ys] + [2])
    tables = np.zeros(max(n_fits, 1) * nbmax * 4, dtype=np.float32)
    hdr = _lib.TF()
    st = _lib.lib().ytgb_tf_pack(
        n_fits, vals, nb, bounds.ctypes.data_as(C.POINTER(C.c_double)), ids6(tf_obj.field_ids),
        ids6(tf_obj.weight_field_ids), ids6(tf_obj.weight_table_ids), ids6(tf_obj.field_table_ids),
        int(getattr(tf_obj, "grey_opacity", 0)), C.byref(hdr), tables.ctypes.data)
    _lib.check(st, "ytgb_tf_pack")
    return PackedTF(hdr, tables)
