"""Drop-in replacements for yt's image samplers (yt/utilities/lib/image_samplers.pyx).

``VolumeRenderSampler``, ``ProjectionSampler``,
``InterpolatedProjectionSampler`` and the new ``MIPSampler`` take the same
constructor arguments as yt's classes (``ImageSampler.__init__``
:59-131, ``VolumeRenderSampler.__cinit__`` :406-446,
``InterpolatedProjectionSampler.__cinit__`` :347-366) and the same call,
``sampler(pg, num_threads=0)`` (:132-141), so yt's ``Scene`` /
``KDTreeVolumeSource.render`` / ``off_axis_projection`` drive them unchanged.

The difference is when the work happens.  yt casts every ray through each
brick as the brick is passed in.  Here ``__call__`` only records the brick;
the first read of ``aimage`` uploads all recorded bricks and renders them in
ONE CUDA launch, in the order they were passed (yt passes them in kd
viewpoint order), then writes the result into the caller's image array in
place -- the same array yt's sampler would have mutated.  Reading ``aimage``
is therefore the synchronisation point; ``flush()`` does the same
explicitly.
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np
import torch

from . import _lib
from . import transfer_functions as _tfm
from .volume import BrickSet, brick_parts, device_reads_host, render as _render


def _device():
    if not torch.cuda.is_available():
        raise _lib.YtgbError("yt_gb300 samplers need a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


_stage = {"buf": None, "lock": threading.Lock()}


def _staging(nbytes: int) -> torch.Tensor:
    """A page-locked float64 host buffer of at least ``nbytes``, kept for
    reuse (grown as needed).  flush() holds ``_stage["lock"]`` while it uses
    it."""
    b = _stage["buf"]
    if b is None or b.numel() * 8 < nbytes:
        b = torch.empty((nbytes + 7) // 8, dtype=torch.float64, pin_memory=True)
        _stage["buf"] = b
    return b


def make_view(vp_pos, vp_dir, center, bounds, nx, ny, x_vec, y_vec, width, lens_type, camera_data):
    """Build a ``ytgb_view`` from ImageSampler arguments.  Returns (view,
    per-pixel positions or None, per-pixel directions or None)."""
    v = _lib.View()
    v.nx, v.ny = int(nx), int(ny)
    vp_pos = np.asarray(vp_pos, dtype=np.float64)
    vp_dir = np.asarray(vp_dir, dtype=np.float64)
    px_pos = px_dir = None
    if lens_type == "plane-parallel":
        v.lens = _lib.LENS_PLANE_PARALLEL
        v.extent = _lib.EXTENT_PLANE_PARALLEL
        flat_p = vp_pos.ravel()
        flat_d = vp_dir.ravel()
        if flat_p.size != 12 or flat_d.size != 3:
            raise RuntimeError("plane-parallel lens needs 12 position and 3 direction parameters")
        for i in range(12):
            v.vp_pos[i] = float(flat_p[i])
        for i in range(3):
            v.vp_dir[i] = float(flat_d[i])
    else:
        # image_samplers.pyx:90-96
        if not (vp_pos.shape[0] == vp_dir.shape[0] == nx) or not (vp_pos.shape[1] == vp_dir.shape[1] == ny):
            msg = f"Bad lens shape / direction for {lens_type}\n"
            msg += "Shapes: ({} - {} - {}) and ({} - {} - {})".format(
                vp_pos.shape[0], vp_dir.shape[0], nx, vp_pos.shape[1], vp_dir.shape[1], ny)
            raise RuntimeError(msg)
        v.lens = _lib.LENS_PER_PIXEL
        if camera_data is not None and lens_type == "perspective":
            v.extent = _lib.EXTENT_PERSPECTIVE
        else:
            v.extent = _lib.EXTENT_NULL
        px_pos = np.ascontiguousarray(np.asarray(vp_pos).reshape(nx, ny, 3), dtype=np.float64)
        px_dir = np.ascontiguousarray(np.asarray(vp_dir).reshape(nx, ny, 3), dtype=np.float64)
    for i in range(3):
        v.center[i] = float(center[i])
        v.x_vec[i] = float(x_vec[i])
        v.y_vec[i] = float(y_vec[i])
        v.width[i] = float(width[i])
    for i in range(4):
        v.bounds[i] = float(bounds[i])
    v.pdx = (v.bounds[1] - v.bounds[0]) / v.nx
    v.pdy = (v.bounds[3] - v.bounds[2]) / v.ny
    if camera_data is not None:
        cd = np.asarray(camera_data, dtype=np.float64).ravel()
        for i in range(15):
            v.camera_data[i] = float(cd[i])
    return v, px_pos, px_dir


def brick_tuple(pg):
    """(data, mask, left_edge, right_edge, dims) of a PartitionedGrid (yt's
    own or :class:`yt_gb300.partitioned_grid.PartitionedGrid`)."""
    return brick_parts(pg)


class ImageSampler:
    kind = None
    _with_lo = False

    def __init__(self, vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width, volume_method, *args,
                 **kwargs):
        self.volume_method = volume_method
        camera_data = kwargs.pop("camera_data", None)
        if camera_data is not None:
            self.camera_data = camera_data
        zbuffer = kwargs.pop("zbuffer", None)
        if zbuffer is None:
            zbuffer = np.ones((image.shape[0], image.shape[1]), "float64")
        self.lens_type = kwargs.pop("lens_type", None)
        self.flags = int(kwargs.pop("flags", 0))
        self._image = image
        nx, ny = image.shape[0], image.shape[1]
        self._view, self._px_pos, self._px_dir = make_view(
            vp_pos, vp_dir, center, bounds, nx, ny, x_vec, y_vec, width, self.lens_type, camera_data)
        self.acenter = center
        self.ax_vec = x_vec
        self.ay_vec = y_vec
        self.azbuffer = np.asarray(zbuffer)
        self.nv = (nx, ny)
        self.bounds = tuple(float(b) for b in bounds)
        self.pdx = (self.bounds[1] - self.bounds[0]) / nx
        self.pdy = (self.bounds[3] - self.bounds[2]) / ny
        self.width = np.array(width, dtype=np.float64)
        self._pending = []
        self._prefault = None
        self.n_samples = 1
        self.last_counters = None
        self.last_h2d_bytes = 0
        self.last_d2h_bytes = 0
        self.last_timings = {}
        self._start_prefault()

    # ---- the call surface ---------------------------------------------------
    def __call__(self, pg, num_threads=0, **kwa):
        if self.volume_method == "KDTree":
            # cast_through_kdtree, inlined: yt makes one call per brick
            if len(pg.my_data) > 6:
                raise ValueError("at most 6 fields per brick are supported")
            self._pending.append(pg)
            return 0
        elif self.volume_method == "Octree":
            return self.cast_through_octree(pg, num_threads=num_threads, **kwa)
        else:
            raise NotImplementedError(
                f'Volume rendering has not been implemented for method: "{self.volume_method}"')

    def cast_through_kdtree(self, pg, num_threads=0):
        """Record the brick; it is rendered at the next ``aimage`` read."""
        if len(pg.my_data) > 6:
            raise ValueError("at most 6 fields per brick are supported")
        self._pending.append(pg)
        return 0

    def _await_prefault(self, img, L):
        """Wait for the prefault _start_prefault began, or fault ``img``'s
        pages in now if it was not that array or did not succeed.  Returns
        the prefault's record (or None)."""
        pre, self._prefault = self._prefault, None
        if pre is not None:
            pre["thread"].join()
        if pre is None or pre["array"] is not img or not pre["ok"]:
            _lib.check(L.ytgb_host_prefault(img.ctypes.data, img.nbytes), "image prefault")
        return pre

    def _start_prefault(self):
        """Fault the image's pages in for writing on a host thread while the
        caller passes its bricks in, where the render will write the image in
        place (the first flush() waits for it and faults in any image it was
        not given; a failure is left for flush() to meet and report)."""
        img = self._image
        if not (isinstance(img, np.ndarray) and img.dtype == np.float64 and img.flags.c_contiguous
                and img.flags.writeable and torch.cuda.is_available() and device_reads_host(_device())):
            return
        box = {"array": img, "ok": False}

        def run():
            box["start"] = time.perf_counter()
            try:
                _lib.check(_lib.lib().ytgb_host_prefault(img.ctypes.data, img.nbytes), "image prefault")
                box["ok"] = True
            except BaseException:
                pass
            box["end"] = time.perf_counter()

        box["thread"] = threading.Thread(target=run, daemon=True)
        box["thread"].start()
        self._prefault = box

    def cast_through_octree(self, pg, oct=None, num_threads=0):
        """ImageSampler.cast_through_octree (image_samplers.pyx:202-288): the
        octree volume source's one PartitionedGrid (14 values per cell, as
        render_source.py:667-680 packs them) rendered at once through
        ``oct``, a :class:`yt_gb300.octree.Octree` (the drop-in for yt's
        ``_OctreeRayTracing``)."""
        from .octree import Octree, OctreeVolume, render_octree

        if not isinstance(oct, Octree):
            raise TypeError("cast_through_octree needs a yt_gb300.octree.Octree (in place of _OctreeRayTracing)")
        if self._px_pos is None:
            raise ValueError("the octree path casts per-pixel rays: use a perspective (per-pixel) lens")
        self.flush()
        dev = _device()
        cells = np.asarray(pg.my_data[0], dtype=np.float64).reshape(-1, 14)
        vol = OctreeVolume(oct, cells, dev)
        img = self._image
        if not (isinstance(img, np.ndarray) and img.dtype == np.float64 and img.flags.c_contiguous):
            img = np.ascontiguousarray(img, dtype=np.float64)
        view = self._view
        in_place = device_reads_host(dev)
        if in_place:
            # the kernel reads the rays and accumulates into the image where
            # they lie (as flush() does)
            self._await_prefault(img, _lib.lib())
            image_d = img
            view.px_pos, view.px_dir = self._px_pos.ctypes.data, self._px_dir.ctypes.data
        else:
            image_d = torch.from_numpy(img).to(dev)
            px_pos = torch.from_numpy(self._px_pos).to(dev)
            px_dir = torch.from_numpy(self._px_dir).to(dev)
            view.px_pos, view.px_dir = px_pos.data_ptr(), px_dir.data_ptr()
        counters = torch.zeros(4, dtype=torch.int64, device=dev)
        error = torch.zeros(1, dtype=torch.int32, device=dev)
        try:
            render_octree(vol, view, self.kind, image_d, tf=self._tf(), n_samples=self.n_samples, flags=self.flags,
                          counters=counters, error=error, light=self._light())
            stream = torch.cuda.current_stream(dev)
            _lib.check(_lib.lib().ytgb_check_error(error.data_ptr(), stream.cuda_stream), "octree render")
        finally:
            view.px_pos = view.px_dir = None
        if not in_place:
            self._image[...] = image_d.cpu().numpy()
        elif img is not self._image:
            self._image[...] = img
        self.last_counters = counters.cpu().numpy()
        return 0

    @property
    def aimage(self):
        self.flush()
        return self._image

    @aimage.setter
    def aimage(self, value):
        self.flush()
        self._image = value

    @property
    def image(self):
        return self.aimage

    # ---- execution ------------------------------------------------------------
    def _tf(self):
        return None

    def _light(self):
        return None

    def flush(self):
        if not self._pending:
            return
        pending, self._pending = self._pending, []
        dev = _device()
        L = _lib.lib()
        t0 = time.perf_counter()
        img = self._image
        if not (isinstance(img, np.ndarray) and img.dtype == np.float64 and img.flags.c_contiguous):
            img = np.ascontiguousarray(img, dtype=np.float64)
        zb = np.ascontiguousarray(self.azbuffer, dtype=np.float64)
        if device_reads_host(dev):
            self._flush_in_place(pending, dev, L, img, zb, t0)
            return
        # Otherwise (a device that reaches host memory only through copies)
        # the render is launched on the usual inputs -- a new image (all zero
        # bits) and a zbuffer of ones, which clips nothing
        # (image_samplers.pyx:185, max_t = 1) -- while a host thread checks
        # that they are: it faults the image's pages in for writing (so that
        # its read does not map the shared zero page and make every page a
        # copy-on-write fault later) and reads both arrays on all cores.
        # Other inputs are uploaded and the view rendered again.
        checks = {}

        def host_checks():
            try:
                flag = C.c_int32()
                _lib.check(L.ytgb_host_prefault(img.ctypes.data, img.nbytes), "image prefault")
                _lib.check(L.ytgb_host_is_uniform(img.ctypes.data, img.size, 0.0, 0, C.byref(flag)), "image check")
                checks["img_zero"] = bool(flag.value)
                _lib.check(L.ytgb_host_is_uniform(zb.ctypes.data, zb.size, 1.0, 0, C.byref(flag)),
                           "zbuffer check")
                checks["zb_ones"] = bool(flag.value)
            except BaseException as e:  # re-raised on the calling thread
                checks["error"] = e

        bricks = BrickSet(pending, device=dev, with_lo=self._with_lo, direct=False)
        t1 = time.perf_counter()
        order = np.arange(len(pending), dtype=np.int32)
        # the pixel rectangles on all cores before the checks take them
        rects = bricks.rects(self._view, order)
        checker = threading.Thread(target=host_checks, daemon=True)
        checker.start()
        nx, ny = self.nv
        px_pos = px_dir = None
        h2d = 0
        if self._px_pos is not None:
            px_pos = torch.from_numpy(self._px_pos).to(dev)
            px_dir = torch.from_numpy(self._px_dir).to(dev)
            h2d += self._px_pos.nbytes + self._px_dir.nbytes
        counters = torch.zeros(4, dtype=torch.int64, device=dev)
        error = torch.zeros(1, dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev)
        keep = []

        def launch(image_d, zb_d):
            _render(bricks, self._view, order, self.kind, image_d, tf=self._tf(), zbuffer=zb_d,
                    n_samples=self.n_samples, flags=self.flags, counters=counters, error=error,
                    px_pos=px_pos, px_dir=px_dir, light=self._light(), keep=keep, rects=rects)

        image_d = torch.zeros((nx, ny, 4), dtype=torch.float64, device=dev)
        try:
            launch(image_d, None)
        finally:
            checker.join()
        if "error" in checks:
            raise checks["error"]
        img_zero, zb_ones = checks["img_zero"], checks["zb_ones"]
        if not (img_zero and zb_ones):
            image_d = torch.zeros((nx, ny, 4), dtype=torch.float64, device=dev) if img_zero else \
                torch.from_numpy(img).to(dev)
            zb_d = None if zb_ones else torch.from_numpy(zb).to(dev)
            h2d += (0 if img_zero else img.nbytes) + (0 if zb_ones else zb.nbytes)
            counters.zero_()
            error.zero_()
            launch(image_d, zb_d)
        t2 = time.perf_counter()
        _lib.check(L.ytgb_check_error(error.data_ptr(), stream.cuda_stream), "render")
        keep.clear()
        t3 = time.perf_counter()
        # device -> pinned staging (full link speed), then into the caller's
        # array on all host cores
        with _stage["lock"]:
            stage = _staging(img.nbytes)[: img.size].view(image_d.shape)
            stage.copy_(image_d)
            _lib.check(L.ytgb_host_copy(img.ctypes.data, stage.data_ptr(), img.nbytes, 0), "image copy")
        if img is not self._image:
            self._image[...] = img
        self.last_counters = counters.cpu().numpy()
        t4 = time.perf_counter()
        # bytes copied host -> device (bricks, boundary tables, descriptors,
        # masks, order and rectangles, and whichever of image, zbuffer and
        # per-pixel rays were needed) and device -> host (image, counters)
        self.last_h2d_bytes = int(bricks.upload_bytes + h2d + 20 * len(pending))
        self.last_d2h_bytes = int(img.nbytes + 4 * 8)
        # pack: bricks into the arena; launch: launch, host checks (the
        # device renders meanwhile); render: the rest of the render;
        # download: the image into the caller's array
        self.last_timings = {"pack_ms": 1e3 * (t1 - t0), "launch_ms": 1e3 * (t2 - t1), "render_ms": 1e3 * (t3 - t2),
                             "download_ms": 1e3 * (t4 - t3)}

    def _flush_in_place(self, pending, dev, L, img, zb, t0):
        """flush() on a device that reads and writes pageable host memory:
        the kernel accumulates straight into the caller's image and reads
        the zbuffer where they lie, so nothing is copied back.  The image's
        pages are faulted in for writing from the first brick on, on a host
        thread (the device would otherwise fault on each page); flush()
        waits for that once the bricks are gathered.  As with yt's sampler,
        a render that fails (an error word raised below) may have written
        part of the image."""
        # (the device gather runs while the rectangles are computed: pending
        # keeps the bricks alive and the stream is synchronised below before
        # they may change)
        bricks = BrickSet(pending, device=dev, with_lo=self._with_lo, direct=True, sync=False)
        order = np.arange(len(pending), dtype=np.int32)
        rects = bricks.rects(self._view, order)
        t_bricks = time.perf_counter()
        pre = self._await_prefault(img, L)
        t1 = time.perf_counter()
        counters = torch.zeros(4, dtype=torch.int64, device=dev)
        error = torch.zeros(1, dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev)
        keep = []
        _render(bricks, self._view, order, self.kind, img, tf=self._tf(), zbuffer=zb, n_samples=self.n_samples,
                flags=self.flags, counters=counters, error=error, px_pos=self._px_pos, px_dir=self._px_dir,
                light=self._light(), keep=keep, rects=rects)
        t2 = time.perf_counter()
        _lib.check(L.ytgb_check_error(error.data_ptr(), stream.cuda_stream), "render")
        keep.clear()
        t3 = time.perf_counter()
        if img is not self._image:
            self._image[...] = img
        self.last_counters = counters.cpu().numpy()
        t4 = time.perf_counter()
        # bytes the device read from host memory (bricks, boundary tables,
        # descriptors, masks, order and rectangles, per-pixel rays, image
        # and zbuffer) and wrote to it (image, counters)
        h2d = img.nbytes + zb.nbytes
        if self._px_pos is not None:
            h2d += self._px_pos.nbytes + self._px_dir.nbytes
        self.last_h2d_bytes = int(bricks.upload_bytes + h2d + 20 * len(pending))
        self.last_d2h_bytes = int(img.nbytes + 4 * 8)
        # pack: bricks gathered and rectangles computed (bricks_at), image
        # pages faulted in; launch; render: until the image is written;
        # download: the counters
        self.last_timings = {"pack_ms": 1e3 * (t1 - t0), "launch_ms": 1e3 * (t2 - t1), "render_ms": 1e3 * (t3 - t2),
                             "download_ms": 1e3 * (t4 - t3), "bricks_at_ms": 1e3 * (t_bricks - t0)}
        if pre is not None and "end" in pre:
            self.last_timings.update(prefault_from_ms=1e3 * (pre["start"] - t0), prefault_ms=1e3 * (pre["end"] - pre["start"]))

    def ensure_code_unit_params(self, params):
        for name in ["center", "vp_pos", "vp_dir", "width"]:
            p = params[name]
            if hasattr(p, "in_units"):
                params[name] = p.in_units("code_length")
        b = params["bounds"]
        if hasattr(b[0], "units"):
            params["bounds"] = tuple(x.in_units("code_length").d for x in b)
        return params


class ProjectionSampler(ImageSampler):
    """Line integral of cell-centred data (image_samplers.pyx:327-343):
    rgba[i] += data[i][cell] * (exit_t - enter_t), i < min(4, n_fields)."""
    kind = _lib.PROJECTION


class MIPSampler(ImageSampler):
    """Maximum-intensity projection: ProjectionSampler with max in place of +=
    (no counterpart in yt's ray caster)."""
    kind = _lib.MIP


class InterpolatedProjectionSampler(ImageSampler):
    """Trilinear samples of vertex-centred data summed along the ray
    (image_samplers.pyx:346-403)."""
    kind = _lib.INTERPOLATED_PROJECTION

    def __init__(self, vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width, volume_method,
                 n_samples=10, **kwargs):
        super().__init__(vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width, volume_method, **kwargs)
        self.n_samples = int(n_samples)


class VolumeRenderSampler(ImageSampler):
    """Emission-absorption volume rendering through yt's transfer-function
    tables (image_samplers.pyx:405-487)."""
    kind = _lib.VOLUME_RENDER

    def __init__(self, vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width, volume_method, tf_obj,
                 n_samples=10, **kwargs):
        super().__init__(vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width, volume_method, **kwargs)
        assert tf_obj.n_field_tables <= 6
        self.tf_obj = tf_obj
        self.n_samples = int(n_samples)
        self._packed = _tfm.pack(tf_obj)

    def _tf(self):
        return self._packed


class LightSourceRenderSampler(ImageSampler):
    """Volume rendering with a directional light on the gradient of field 0
    (image_samplers.pyx:496-590; eval_gradient, fixed_interpolator.cpp:
    116-148; FIT_eval_transfer_with_light, field_interpolation_tables.pxd:
    115-143).  ``light_dir`` is normalised as yt does.  ``gradient_lo``
    also uploads each value's float32 rounding error so the gradient's
    differences carry float64 accuracy (for fields whose cell-to-cell
    variation is near float32's resolution)."""
    kind = _lib.LIGHT_SOURCE

    def __init__(self, vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width, volume_method, tf_obj,
                 n_samples=10, light_dir=(1.0, 1.0, 1.0), light_rgba=(1.0, 1.0, 1.0, 1.0), gradient_lo=False,
                 **kwargs):
        super().__init__(vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width, volume_method, **kwargs)
        assert tf_obj.n_field_tables <= 6
        self.tf_obj = tf_obj
        self.n_samples = int(n_samples)
        self._packed = _tfm.pack(tf_obj)
        self.light_dir = np.asarray(light_dir, dtype=np.float64)
        self.light_rgba = np.asarray(light_rgba, dtype=np.float64)
        self._with_lo = bool(gradient_lo)

    def _tf(self):
        return self._packed

    def _light(self):
        return (self.light_dir, self.light_rgba)
