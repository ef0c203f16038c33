"""Rendering views of a resident volume (the product-side driver).

``Renderer`` keeps a :class:`~yt_gb300.volume.BrickSet` and packed transfer
function resident on the device and renders ``Camera`` views with one launch
each -- what ``KDTreeVolumeSource.render`` (render_source.py:563-606) does
with a Python loop over bricks.  The returned image is the sampler's raw
``aimage`` (before ``finalize_image``), a (nx, ny, 4) float64 device tensor.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .autotune import tile_shape_for
from .image_samplers import make_view
from .transfer_functions import pack
from .volume import BrickSet, render as _render, trace as _trace


class Renderer:
    def __init__(self, bricks, tf=None, device="cuda", kdtree=None):
        self.device = torch.device(device)
        self.bricks = bricks if isinstance(bricks, BrickSet) else BrickSet(bricks, device=self.device)
        self.tf = tf
        self.packed = pack(tf) if tf is not None else None
        self.kdtree = kdtree
        self.counters = torch.zeros(4, dtype=torch.int64, device=self.device)
        self.error = torch.zeros(1, dtype=torch.int32, device=self.device)

    def view_args(self, camera, device_rays=True):
        """(view, per-pixel positions, per-pixel directions); with
        ``device_rays`` perspective rays are generated in the kernel and the
        arrays are None."""
        if device_rays:
            return camera.device_view(), None, None
        p = camera.sampler_params()
        nx, ny = camera.resolution
        view, ppos, pdir = make_view(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], nx, ny, p["x_vec"],
                                     p["y_vec"], p["width"], p["lens_type"], p["camera_data"])
        return view, ppos, pdir

    def order(self, camera):
        if self.kdtree is None:
            return np.arange(self.bricks.n, dtype=np.int32)
        return self.kdtree.viewpoint_order(camera.viewpoint)

    def render(self, camera, kind=_lib.VOLUME_RENDER, n_samples=1, order=None, image=None, zbuffer=None,
               flags=0, stream=None, keep=None, device_rays=True, tile_shape=None, light=None):
        """Render one view.  ``tile_shape`` None takes the tuned shape of the
        view's workload class (``yt_gb300/tuning.json``) unless ``flags``
        already carries one."""
        view, ppos, pdir = self.view_args(camera, device_rays)
        if tile_shape is None and not (flags >> _lib.FLAG_TILE_SHIFT) & 0xF:
            ctf = bool(kind == _lib.VOLUME_RENDER and self.packed is not None and self.packed.header.ctf_fast)
            tile_shape = tile_shape_for(kind, ctf, view.lens)
        if tile_shape is not None:
            flags = (flags & ~(0xF << _lib.FLAG_TILE_SHIFT)) | (int(tile_shape) << _lib.FLAG_TILE_SHIFT)
        nx, ny = camera.resolution
        if order is None:
            order = self.order(camera)
        if image is None:
            image = torch.zeros((nx, ny, 4), dtype=torch.float64, device=self.device)
        px_pos = px_dir = None
        if ppos is not None:
            px_pos = torch.from_numpy(ppos).to(self.device, non_blocking=False)
            px_dir = torch.from_numpy(pdir).to(self.device, non_blocking=False)
            if keep is not None:
                keep += [px_pos, px_dir]
        uses_tf = kind in (_lib.VOLUME_RENDER, _lib.LIGHT_SOURCE)
        tf = self.packed if uses_tf else None
        if uses_tf and tf is None:
            raise ValueError("volume rendering needs a transfer function")
        _render(self.bricks, view, order, kind, image, tf=tf, zbuffer=zbuffer, n_samples=n_samples, flags=flags,
                counters=self.counters, error=self.error, px_pos=px_pos, px_dir=px_dir, stream=stream, keep=keep,
                light=light)
        return image

    def check(self):
        s = torch.cuda.current_stream(self.device)
        _lib.check(_lib.lib().ytgb_check_error(self.error.data_ptr(), s.cuda_stream), "render")

    def trace(self, camera, order=None, device_rays=True):
        view, ppos, pdir = self.view_args(camera, device_rays)
        if order is None:
            order = self.order(camera)
        px_pos = px_dir = None
        if ppos is not None:
            px_pos = torch.from_numpy(ppos).to(self.device)
            px_dir = torch.from_numpy(pdir).to(self.device)
        return _trace(self.bricks, view, order, px_pos=px_pos, px_dir=px_dir)


def relative_error(gpu: np.ndarray, ref: np.ndarray, tau: float = 1e-6, channels=(0, 1, 2, 3)):
    """Per-pixel relative error max|g-o| / max(|o|, tau*max|o|) and its RMS over
    pixels with o != 0, per channel; returns (max over channels, rms over
    channels).  NaN pixels must coincide (a NaN against a number is an
    infinite error) and are otherwise left out."""
    mx, rms = 0.0, 0.0
    for c in channels:
        o = ref[..., c]
        g = gpu[..., c]
        on, gn = np.isnan(o), np.isnan(g)
        if not np.array_equal(on, gn):
            return float("inf"), float("inf")
        keep = ~on
        o, g = o[keep], g[keep]
        if o.size == 0:
            continue
        m = np.abs(o).max()
        if m == 0:
            e = np.abs(g).max()
            mx = max(mx, float(e))
            continue
        den = np.maximum(np.abs(o), tau * m)
        r = np.abs(g - o) / den
        mx = max(mx, float(r.max()))
        nz = o != 0
        if nz.any():
            rms = max(rms, float(np.sqrt(np.mean(r[nz] ** 2))))
    return mx, rms
