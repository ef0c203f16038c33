"""Tile-shape autotuning for the render and batch kernels.

A block renders a tile of 128 pixel rays: 8x16 (shape 0), 16x8 (shape 1) or
4x32 (shape 2) pixels.  Which shape is fastest depends on how coherent the
rays of a tile are (lens, image size relative to the bricks' footprints) and
on the sampler.  Every shape produces the same image bit for bit, so the
choice is purely a speed decision.

``tuning.json`` (next to this file) holds the shape measured fastest on
GB300 for each workload class -- ``"<sampler>/<lens>"`` with sampler one of
``vr-ctf``, ``vr``, ``projection``, ``interpolated_projection``, ``mip`` and
lens ``plane-parallel`` / ``perspective`` / ``per-pixel``.
:func:`tile_shape_for` looks a class up (shape 0 when absent);
:func:`autotune` times the shapes for one view; ``python -m
yt_gb300.autotune --out FILE`` re-measures the table on the current GPU over
the standard workloads.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from . import _lib

TABLE = Path(__file__).resolve().parent / "tuning.json"
SHAPES = (0, 1, 2)
_SAMPLER = {_lib.VOLUME_RENDER: "vr", _lib.PROJECTION: "projection",
            _lib.INTERPOLATED_PROJECTION: "interpolated_projection", _lib.MIP: "mip",
            _lib.LIGHT_SOURCE: "light_source"}
_LENS = {_lib.LENS_PLANE_PARALLEL: "plane-parallel", _lib.LENS_PERSPECTIVE: "perspective",
         _lib.LENS_PER_PIXEL: "per-pixel"}
_cache = None


def workload_class(kind: int, ctf_fast: bool, lens: int) -> str:
    s = _SAMPLER[int(kind)]
    if s == "vr" and ctf_fast:
        s = "vr-ctf"
    return f"{s}/{_LENS.get(int(lens), 'per-pixel')}"


def table() -> dict:
    global _cache
    if _cache is None:
        _cache = json.loads(TABLE.read_text())["shapes"] if TABLE.exists() else {}
    return _cache


def tile_shape_for(kind: int, ctf_fast: bool, lens: int) -> int:
    return int(table().get(workload_class(kind, ctf_fast, lens), 0))


def autotune(renderer, camera, kind=_lib.VOLUME_RENDER, n_samples=1, reps=5, warmup=2, shapes=SHAPES):
    """Median CUDA-event time (ms) of each tile shape for one view, and the
    fastest shape.  Every shape's image is checked to be identical."""
    import torch

    dev = renderer.device
    times, ref = {}, None
    for ts in shapes:
        ms = []
        for i in range(warmup + reps):
            img = torch.zeros((*camera.resolution, 4), dtype=torch.float64, device=dev)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            renderer.render(camera, kind=kind, n_samples=n_samples, image=img, tile_shape=ts)
            b.record()
            torch.cuda.synchronize(dev)
            if i >= warmup:
                ms.append(a.elapsed_time(b))
        renderer.check()
        if ref is None:
            ref = img
        elif not torch.equal(ref.view(torch.int64), img.view(torch.int64)):
            raise RuntimeError(f"tile shape {ts} changed the image")
        times[ts] = float(np.median(ms))
    best = min(times, key=times.get)
    return best, times


def _suite():
    """(renderer factory, camera, kind, n_samples) for the standard
    workloads at their benchmark sizes."""
    from . import testing, workloads
    from .amr_kdtree import AMRKDTree
    from .camera import Camera
    from .render import Renderer

    out = []
    w = workloads.amr_vr()
    out.append((lambda w=w: Renderer(w.bricks, w.tf, kdtree=w.kdtree), w.views[0].camera, _lib.VOLUME_RENDER, 1))
    pp = Camera((1.3, 0.2, -0.7), (0.5, 0.5, 0.5), 1.0, 1024, lens_type="plane-parallel")
    out.append((lambda w=w: Renderer(w.bricks, w.tf, kdtree=w.kdtree), pp, _lib.VOLUME_RENDER, 1))
    p = workloads.projection_study(n=256, res=1024, angles=(30.0,))
    for v in p.views:
        out.append((lambda p=p: Renderer(p.bricks, None), v.camera, v.kind, 1))
    kd = AMRKDTree(testing.amr_blob_grids(root=64, levels=2, patch=16, seed=0), log_field=False)
    out.append((lambda kd=kd: Renderer(kd.bricks(), None, kdtree=kd), w.views[0].camera,
                _lib.INTERPOLATED_PROJECTION, 2))
    out.append((lambda kd=kd: Renderer(kd.bricks(), None, kdtree=kd), pp, _lib.INTERPOLATED_PROJECTION, 2))
    return out


def main(argv=None):
    import argparse

    import torch

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=str(TABLE))
    args = ap.parse_args(argv)
    shapes, detail = {}, {}
    for make, cam, kind, ns in _suite():
        r = make()
        view = cam.device_view()
        ctf = bool(r.packed is not None and r.packed.header.ctf_fast)
        cls = workload_class(kind, ctf, view.lens)
        best, times = autotune(r, cam, kind, ns)
        shapes[cls] = best
        detail[cls] = {str(k): round(v, 4) for k, v in times.items()}
        print(cls, best, detail[cls], flush=True)
    meta = {"device": torch.cuda.get_device_name(), "method": "median of 5 CUDA-event timings after 2 warm-ups"}
    Path(args.out).write_text(json.dumps({"shapes": shapes, "ms": detail, "meta": meta}, indent=1) + "\n")


if __name__ == "__main__":
    main()
