"""A render server: resident volumes, continuous batching, latency accounting.

Volumes (``BrickSet``) and transfer functions (packed tables) stay resident
in HBM.  Requests -- (volume, transfer function, camera, sampler) -- arrive
over time.  The loop:

* **admits** arrived requests while their output images fit the HBM budget
  (a request waits in the arrival queue otherwise);
* **batches** every admitted, not yet launched request into one group as
  soon as one of ``slots`` CUDA streams is free: the small requests of the
  group go into one :class:`~yt_gb300.batch.Batch` (one persistent launch
  per sampler class), the large ones -- which fill the GPU by themselves --
  and a lone small one take the single-view kernel one after another on
  the same stream, each request finishing with its own launch -- so requests that arrive while earlier batches are
  on the GPU start on another stream at once and their work overlaps on the
  device (continuous batching, not a queue in front of one stream).  Each
  launch takes a stream one priority level below every batch still in
  flight: the block scheduler gives SMs to the earliest batch's blocks
  first and lets later batches fill what it leaves, so a request is not
  slowed by requests that arrived after it (first come, first served, with
  backfill) -- the plain loop's order without its idle SMs;
* **retires** a batch when its completion event fires, frees its images'
  budget and records each request's latency (completion - arrival);
* **drops** requests cancelled before their launch (``Request.cancelled``),
  releasing their budget; they are listed in ``server.cancelled``.

With ``plain=True`` the same loop renders each request alone with the
single-view kernel (``ytgb_render``), one launch per request on one stream,
as yt renders one camera per ``Scene.render``: the comparator of the
served form.

Each request's image is exactly what rendering it alone gives (the same
per-ray code, independent of the batch it lands in).
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .autotune import tile_shape_for
from .batch import Batch, Job
from .render import Renderer


@dataclass
class Request:
    rid: int
    volume: str
    tf: str
    camera: object
    kind: int = _lib.VOLUME_RENDER
    arrival: float = 0.0          # seconds after the server's start
    n_samples: int = 1
    admitted: float = -1.0
    launched: float = -1.0
    done: float = -1.0
    image: torch.Tensor | None = None
    samples: int = 0
    cancelled: bool = False       # set before launch: the request is dropped, never rendered
    batch_size: int = 0           # requests in the launch that rendered it

    @property
    def pixels(self) -> int:
        nx, ny = self.camera.resolution
        return nx * ny

    @property
    def image_bytes(self) -> int:
        return self.pixels * 4 * 8

    @property
    def latency(self) -> float:
        return self.done - self.arrival


PRIORITY_LEVELS = 4  # stream priorities the served launches use (0 .. -3)


def split_group(reqs, batch_pixels: int):
    """A launch group's requests as (batched, alone): the small ones (under
    ``batch_pixels`` pixels) share one persistent batch launch; the large
    ones -- and a lone small one -- take the single-view kernel each."""
    small = [q for q in reqs if q.pixels < batch_pixels]
    large = [q for q in reqs if q.pixels >= batch_pixels]
    if len(small) == 1:
        return [], small + large
    return small, large


def launch_level(levels_in_flight) -> int:
    """The priority level of a new launch (0 the highest): one below every
    batch still in flight, the lowest level once that is reached."""
    return min(PRIORITY_LEVELS - 1, max((k + 1 for k in levels_in_flight), default=0))


@dataclass
class _InFlight:
    parts: list                                # [(requests, completion event)] in stream order
    stream: torch.cuda.Stream
    bytes: int
    counters: list                             # counter tensors of its launches
    errors: list                               # error words of its launches
    keep: list = field(default_factory=list)   # device inputs the launches read
    level: int = 0                             # its stream's priority level (0 the highest)


class _Plain:
    """The counters and error word of one plain launch."""

    def __init__(self, device):
        self.counters = torch.zeros(4, dtype=torch.int64, device=device)
        self.error = torch.zeros(1, dtype=torch.int32, device=device)


class RenderServer:
    def __init__(self, volumes: dict, tfs: dict, device="cuda", hbm_budget=8 << 30, slots=4, max_batch=64,
                 tile_shape=None, keep_images=False, plain=False, range64=True, batch_pixels=512 * 512):
        """``volumes``: name -> (bricks, kdtree or None); ``tfs``: name ->
        transfer function.  ``plain``: one single-view launch per request
        on one stream (``slots`` and ``max_batch`` are then 1).
        ``keep_images``: keep every finished request's image (True), none
        (False), or those a predicate of the request selects.
        ``range64``: resident volumes also keep their values' float32
        rounding errors (twice the device memory), so that a sample near a
        transfer-function bound is kept or dropped as yt's float64 test
        decides (field_interpolation_tables.pxd:72-73) -- a transfer
        function whose bounds lie inside the data's range otherwise drops or
        keeps a few such samples differently.
        ``batch_pixels``: requests with fewer pixels go into the persistent
        batch kernel together; larger ones, which fill the GPU on their own
        (512^2 pixels are 2048 tiles, several waves), take the single-view
        kernel one after another on the launch's stream."""
        self.device = torch.device(device)
        self.plain = bool(plain)
        if self.plain:
            slots, max_batch = 1, 1
        self.renderers = {}
        self.volumes = {}
        from .transfer_functions import pack
        from .volume import BrickSet

        for name, (bricks, kd) in volumes.items():
            bs = BrickSet(bricks, device=self.device, with_lo=range64)
            bs.range_eps  # its one synchronising reduction, here rather than in the request loop
            self.volumes[name] = (bs, kd)
        self.tfs = {name: (tf, pack(tf)) for name, tf in tfs.items()}
        self.budget = int(hbm_budget)
        self.in_use = 0
        self.n_slots = slots
        # slots streams per priority level, level 0 the highest (CUDA: lower
        # numbers are higher priorities; torch keeps PRIORITY_LEVELS pools)
        self.levels = [[torch.cuda.Stream(self.device, priority=-(PRIORITY_LEVELS - 1 - k)) for _ in range(slots)]
                       for k in range(PRIORITY_LEVELS)]
        self.slots = self.levels[0]
        self.max_batch = max_batch
        self.tile_shape = tile_shape
        self.keep_images = keep_images
        self.batch_pixels = int(batch_pixels)
        self.samples = 0
        self.cancelled = []
        self.on_tick = None   # test hook: called with (server, now) once per loop turn

    def renderer(self, volume: str, tf: str | None) -> Renderer:
        key = (volume, tf)
        r = self.renderers.get(key)
        if r is None:
            bricks, kd = self.volumes[volume]
            r = Renderer(bricks, None, device=self.device, kdtree=kd)
            if tf is not None:
                r.tf, r.packed = self.tfs[tf]
            self.renderers[key] = r
        return r

    def _launch(self, reqs, stream, now):
        """Launch a group of requests on one stream: the small ones (under
        batch_pixels) in one persistent batch launch first, then the large
        ones -- and a lone small one -- each through the single-view kernel
        (which stages its table in shared memory and needs no work queue),
        with a completion event after each launch so that every request
        finishes when its own launch does."""
        for q in reqs:
            q.batch_size = len(reqs)
        f = _InFlight([], stream, sum(q.image_bytes for q in reqs), [], [])
        if self.plain:
            self._launch_plain(reqs, stream, now, f)
            return f
        small, large = split_group(reqs, self.batch_pixels)
        if small:
            jobs = []
            for q in small:
                q.image = torch.empty((*q.camera.resolution, 4), dtype=torch.float64, device=self.device)
                r = self.renderer(q.volume, q.tf if q.kind == _lib.VOLUME_RENDER else None)
                jobs.append(Job(r, q.camera, q.kind, q.n_samples, q.image))
            b = Batch(jobs, device=self.device, tile_shape=self.tile_shape)
            # the batch's tables, counters and error word were written on
            # the current stream
            stream.wait_stream(torch.cuda.current_stream(self.device))
            b.launch(stream)
            ev = torch.cuda.Event()
            ev.record(stream)
            for q in small:
                q.launched = now
            f.parts.append((small, ev))
            f.counters.append(b.counters)
            f.errors.append(b.error)
            f.keep.append(b)
        if large:
            self._launch_plain(large, stream, now, f)
        return f

    def _launch_plain(self, reqs, stream, now, f):
        """Each request through the single-view kernel on ``stream``, one
        completion event per request, into the in-flight record ``f``."""
        from .volume import render as vrender

        pl = _Plain(self.device)
        f.counters.append(pl.counters)
        f.errors.append(pl.error)
        # the counters and error word were zeroed on the current stream
        stream.wait_stream(torch.cuda.current_stream(self.device))
        keep = f.keep
        for q in reqs:
            r = self.renderer(q.volume, q.tf if q.kind == _lib.VOLUME_RENDER else None)
            with torch.cuda.stream(stream):
                q.image = torch.zeros((*q.camera.resolution, 4), dtype=torch.float64, device=self.device)
            view = q.camera.device_view()
            ctf = bool(q.kind == _lib.VOLUME_RENDER and r.packed is not None and r.packed.header.ctf_fast)
            ts = self.tile_shape if self.tile_shape is not None else tile_shape_for(q.kind, ctf, view.lens)
            vrender(r.bricks, view, r.order(q.camera), q.kind, q.image,
                    tf=r.packed if q.kind in (_lib.VOLUME_RENDER, _lib.LIGHT_SOURCE) else None,
                    n_samples=q.n_samples, flags=int(ts) << _lib.FLAG_TILE_SHIFT, counters=pl.counters,
                    error=pl.error, stream=stream, keep=keep)
            q.launched = now
            ev = torch.cuda.Event()
            ev.record(stream)
            f.parts.append(([q], ev))

    def run(self, requests, realtime=True, timeout=600.0):
        """Serve ``requests`` (sorted by arrival).  With ``realtime`` the
        arrival times are honoured against the wall clock; otherwise every
        request is available at once.  Returns the requests with their
        timings filled in."""
        pending = deque(sorted(requests, key=lambda q: q.arrival))
        admitted = deque()
        inflight: list[_InFlight] = []
        t0 = time.perf_counter()
        done = []
        while pending or admitted or inflight:
            now = time.perf_counter() - t0
            if now > timeout:
                raise TimeoutError("render server: requests not finished in time")
            # requests cancelled before their launch leave without rendering
            for q in [q for q in pending if q.cancelled]:
                pending.remove(q)
                q.done = now
                self.cancelled.append(q)
            for q in [q for q in admitted if q.cancelled]:
                admitted.remove(q)
                self.in_use -= q.image_bytes
                q.done = now
                self.cancelled.append(q)
            # retire finished launches (a group's launches end in stream order);
            # a group frees its slot and budget when its last launch ends
            for f in list(inflight):
                while f.parts and f.parts[0][1].query():
                    part, _ = f.parts.pop(0)
                    t = time.perf_counter() - t0
                    for q in part:
                        q.done = t
                        keep = self.keep_images(q) if callable(self.keep_images) else self.keep_images
                        if not keep:
                            q.image = None
                    done += part
                if not f.parts:
                    self.in_use -= f.bytes
                    for c, e in zip(f.counters, f.errors):
                        self.samples += int(c[0].item())
                        _lib.check(_lib.lib().ytgb_check_error(e.data_ptr(), f.stream.cuda_stream), "serve")
                    inflight.remove(f)
            if self.on_tick is not None:
                self.on_tick(self, now)
            # admit arrivals within the HBM budget
            while pending and (not realtime or pending[0].arrival <= now):
                q = pending[0]
                if q.image_bytes > self.budget:
                    raise ValueError(f"request {q.rid} needs more than the whole HBM budget")
                if self.in_use + q.image_bytes > self.budget:
                    break
                pending.popleft()
                q.admitted = now
                self.in_use += q.image_bytes
                admitted.append(q)
            # launch everything admitted on a free slot, one priority level
            # below the batches in flight
            free = len(inflight) < self.n_slots
            if admitted and free:
                reqs = [admitted.popleft() for _ in range(min(self.max_batch, len(admitted)))]
                level = launch_level(f.level for f in inflight)
                busy = {f.stream for f in inflight}
                stream = next(st for st in self.levels[level] if st not in busy)
                f = self._launch(reqs, stream, now)
                f.level = level
                inflight.append(f)
                continue
            if not admitted and (not pending or pending[0].arrival > now):
                # nothing to launch: wait briefly for arrivals or completions
                nxt = pending[0].arrival - now if pending else 1e-3
                time.sleep(max(0.0, min(nxt, 2e-4)))
            elif admitted and not free:
                time.sleep(5e-5)
        torch.cuda.synchronize(self.device)
        return done


def latency_summary(reqs, seed=0, resamples=1000):
    """Latency percentiles (ms) of finished requests, with a bootstrap 95 %
    interval of the p99 (``resamples`` resamplings of the requests): with a
    few hundred requests the p99 is one of the largest few latencies, and two
    forms whose intervals overlap are not told apart by the run."""
    lat = np.array([q.latency for q in reqs]) * 1e3
    if lat.size == 0:
        nan = float("nan")
        return {"p50_ms": nan, "p99_ms": nan, "p99_ci95_ms": [nan, nan], "mean_ms": nan, "max_ms": nan, "n": 0}
    rng = np.random.default_rng(seed)
    boot = np.percentile(lat[rng.integers(0, lat.size, (resamples, lat.size))], 99, axis=1)
    lo, hi = np.percentile(boot, [2.5, 97.5])
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "p99_ci95_ms": [float(lo), float(hi)],
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "n": int(lat.size)}
