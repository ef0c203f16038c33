"""Many views in one persistent launch per sampler class (multi-view batching).

yt renders one camera at a time, each as a Python loop over bricks.  A
:class:`Batch` takes many views -- each a camera, a sampler kind, a resident
volume (``Renderer``) and an output image -- and renders them with one
``ytgb_batch_render`` launch per sampler class (volume rendering with a
ColorTransferFunction, general volume rendering, projection, interpolated
projection, MIP).  Blocks pull (view, tile) work items from a device counter,
so small and large images share the GPU without a launch or a tail per view.
The per-view inputs (kd order, pixel rectangles, launch arguments) are
prepared once on the host and kept in device memory; :meth:`Batch.launch`
only resets the work counters and launches, so a batch can be replayed and
captured in a CUDA graph (:meth:`Batch.capture`).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .autotune import tile_shape_for
from .render import Renderer
from .volume import check_inputs, set_light, set_range


@dataclass
class Job:
    renderer: Renderer
    camera: object
    kind: int = _lib.VOLUME_RENDER
    n_samples: int = 1
    image: torch.Tensor | None = None
    order: np.ndarray | None = None
    flags: int = 0
    light: tuple | None = None   # (light_dir, light_rgba) for the light-source sampler


@dataclass
class _Group:
    kind: int
    variant: int                    # YTGB_VARIANT_* bits
    entries: object = None          # ctypes array of BatchEntry
    dev: torch.Tensor | None = None  # the entries in device memory
    n: int = 0
    total_tiles: int = 0
    smem: int = 0
    jobs: list = field(default_factory=list)


class Batch:
    def __init__(self, jobs, device="cuda", tile_shape=None, blocks=0):
        """``tile_shape`` None: the tuned shape (``yt_gb300/tuning.json``) of
        the class most of the jobs belong to."""
        self.device = torch.device(device)
        if tile_shape is None:
            votes = {}
            for j in jobs:
                tf = j.renderer.packed if j.kind == _lib.VOLUME_RENDER else None
                lens = _lib.LENS_PLANE_PARALLEL if j.camera.lens_type == "plane-parallel" else _lib.LENS_PERSPECTIVE
                ts = tile_shape_for(j.kind, bool(tf is not None and tf.header.ctf_fast), lens)
                votes[ts] = votes.get(ts, 0) + 1
            tile_shape = max(votes, key=votes.get) if votes else 0
        self.tile_shape = int(tile_shape)
        self.blocks = int(blocks)
        self.jobs = list(jobs)
        self.queue = torch.zeros(8, dtype=torch.int32, device=self.device)
        self.error = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.counters = torch.zeros(4, dtype=torch.int64, device=self.device)
        self._keep = []
        groups = {}
        tables = []
        views = []
        for j in self.jobs:
            view = j.camera.device_view()
            nx, ny = j.camera.resolution
            if j.image is None:
                j.image = torch.zeros((nx, ny, 4), dtype=torch.float64, device=self.device)
            order = j.order if j.order is not None else j.renderer.order(j.camera)
            order = np.ascontiguousarray(order, dtype=np.int32)
            rects = j.renderer.bricks.rects(view, order)

            check_inputs(j.renderer.bricks, view, order, j.kind, j.image)
            # rects are read as 16-byte int4: every view's table starts on a
            # 16-byte boundary of the shared buffer
            t = np.concatenate([rects.ravel(), order]).astype(np.int32)
            pad = (-t.size) % 4
            tables.append(np.concatenate([t, np.zeros(pad, dtype=np.int32)]) if pad else t)
            views.append((view, order.size))
        offs = np.cumsum([0] + [t.size for t in tables])
        self.tables = torch.from_numpy(np.concatenate(tables)).to(self.device)
        base = self.tables.data_ptr()
        for j, (view, n_order), off in zip(self.jobs, views, offs[:-1]):
            uses_tf = j.kind in (_lib.VOLUME_RENDER, _lib.LIGHT_SOURCE)
            tf = j.renderer.packed if uses_tf else None
            if uses_tf and tf is None:
                raise ValueError("volume rendering needs a transfer function")
            a = _lib.RenderArgs()
            a.kind = j.kind
            a.n_samples = j.n_samples
            a.n_order = n_order
            a.flags = j.flags
            a.view = view
            a.bricks = j.renderer.bricks.desc.data_ptr()
            a.rects = base + 4 * int(off)
            a.order = base + 4 * (int(off) + 4 * n_order)
            a.data = j.renderer.bricks.data.data_ptr()
            a.bounds = j.renderer.bricks.bounds.data_ptr()
            a.masks = j.renderer.bricks.masks.data_ptr() if j.renderer.bricks.masks is not None else None
            if tf is not None:
                a.tf = tf.header
                a.tf_tables = tf.device_tables(self.device).data_ptr()
            a.image = j.image.data_ptr()
            if j.kind == _lib.LIGHT_SOURCE:
                set_light(a, j.renderer.bricks, j.light)
            elif j.kind == _lib.VOLUME_RENDER:
                set_range(a, j.renderer.bricks)
            a.counters = self.counters.data_ptr()
            a.error = self.error.data_ptr()
            var = _lib.render_variant(a)
            groups.setdefault((j.kind, var), _Group(j.kind, var)).jobs.append(a)
        self.groups = list(groups.values())
        L = _lib.lib()
        for g in self.groups:
            g.n = len(g.jobs)
            g.entries = (_lib.BatchEntry * g.n)()
            for k, a in enumerate(g.jobs):
                g.entries[k].args = a
            total = C.c_int32()
            smem = C.c_int32()
            _lib.check(L.ytgb_batch_plan(g.entries, g.n, self.tile_shape, C.byref(total), C.byref(smem)),
                       "ytgb_batch_plan")
            g.total_tiles, g.smem = total.value, smem.value
            raw = np.frombuffer(g.entries, dtype=np.uint8, count=C.sizeof(_lib.BatchEntry) * g.n).copy()
            g.dev = torch.from_numpy(raw).to(self.device)
            g.jobs = []
        self.images = [j.image for j in self.jobs]

    @property
    def total_tiles(self):
        return sum(g.total_tiles for g in self.groups)

    def launch(self, stream=None):
        """Zero the images and render every view (one launch per group)."""
        stream = stream or torch.cuda.current_stream(self.device)
        L = _lib.lib()
        with torch.cuda.stream(stream):
            for im in self.images:
                im.zero_()
        for q, g in enumerate(self.groups):
            _lib.check(L.ytgb_batch_render(g.dev.data_ptr(), g.n, g.kind, g.variant, self.tile_shape, g.total_tiles,
                                           g.smem, self.queue.data_ptr() + 4 * q, self.blocks,
                                           C.c_void_p(stream.cuda_stream)), "ytgb_batch_render")

    def capture(self):
        """A CUDA graph of :meth:`launch`; replay with ``graph.replay()``."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.launch(s)  # warm-up outside capture (sets kernel attributes)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(torch.cuda.current_stream(self.device))
        return g

    def check(self):
        s = torch.cuda.current_stream(self.device)
        _lib.check(_lib.lib().ytgb_check_error(self.error.data_ptr(), s.cuda_stream), "batch render")
