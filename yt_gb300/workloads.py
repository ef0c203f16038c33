"""The sampler workloads: datasets, bricks, cameras and transfer functions.

* :func:`uniform_vr`   -- one 64^3 blob brick, plane-parallel view down +z,
  256^2, 4-layer ColorTransferFunction, 1 sample per cell.
* :func:`amr_vr`       -- 128^3 root + 3 levels of factor-2 refinement in 16^3
  patches (~1100 kd bricks), perspective view, 1024^2, 8 layers.
* :func:`projection_study` -- a 512^3 float32 lognormal random field,
  ProjectionSampler / MIP at 2048^2 and three orientations.
* :func:`multiview`    -- a 64^3-root 4-level AMR dataset (~4000 bricks of
  8^3..32^3 cells), 64 cameras on a Fibonacci sphere, mixed image sizes and
  samplers.

Every size is a parameter, so tests build the same workloads small.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib, testing
from .amr_kdtree import AMRKDTree
from .camera import Camera
from .transfer_functions import ColorTransferFunction


@dataclass
class View:
    camera: Camera
    kind: int = _lib.VOLUME_RENDER
    n_samples: int = 1


@dataclass
class Workload:
    name: str
    bricks: list               # (data, mask, le, re, dims) tuples, float64 data
    views: list                # View
    tf: object = None          # ColorTransferFunction for volume rendering
    kdtree: AMRKDTree | None = None
    info: dict = field(default_factory=dict)

    def order(self, camera: Camera) -> np.ndarray:
        if self.kdtree is None:
            return np.arange(len(self.bricks), dtype=np.int32)
        return self.kdtree.viewpoint_order(camera.viewpoint)


def color_tf(bounds, n_layers, nbins=256, width=0.01):
    tf = ColorTransferFunction(bounds, nbins=nbins)
    for loc, w, rgba in testing.ctf_layers(bounds, n_layers, width=width):
        tf.add_gaussian(loc, w, list(rgba))
    return tf


def uniform_vr(n=64, res=256, seed=0, n_layers=4) -> Workload:
    g = testing.blob_grid(n, seed=seed)
    kd = AMRKDTree([g], log_field=True)
    lg = np.log10(g.data)
    tf = color_tf((lg.min(), lg.max()), n_layers)
    cam = Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), res, lens_type="plane-parallel")
    return Workload("uniform_vr", kd.bricks(), [View(cam)], tf, kd,
                    {"cells": n ** 3, "resolution": res, "grid": n})


def amr_vr(root=128, levels=3, res=1024, seed=0, n_layers=8, patch=16, lens_type="perspective") -> Workload:
    grids = testing.amr_blob_grids(root=root, levels=levels, patch=patch, seed=seed)
    kd = AMRKDTree(grids, log_field=True)
    lg = np.log10(grids[0].data)
    tf = color_tf((lg.min(), lg.max()), n_layers)
    cam = Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), res, lens_type=lens_type)
    return Workload("amr_vr", kd.bricks(), [View(cam)], tf, kd,
                    {"grids": len(grids), "bricks": kd.num_bricks, "resolution": res, "root": root,
                     "levels": levels})


def grf_brick(field: np.ndarray):
    """One cell-centred brick over [0,1]^3 (off_axis_projection.py:506-524)."""
    n = field.shape
    return ([field], np.ones(n, dtype=np.uint8), np.zeros(3), np.ones(3), np.array(n, dtype=np.int64))


def projection_study(n=512, res=2048, angles=(0.0, 30.0, 57.0), seed=1, kinds=(_lib.PROJECTION, _lib.MIP),
                     field=None) -> Workload:
    if field is None:
        field = testing.lognormal_grf(n, seed=seed)
    views = []
    for kind in kinds:
        for a in angles:
            t = np.deg2rad(a)
            normal = np.array([0.0, np.sin(t), np.cos(t)])
            pos = np.array([0.5, 0.5, 0.5]) - 1.5 * normal
            views.append(View(Camera(pos, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), res, lens_type="plane-parallel"),
                              kind=kind))
    return Workload("projection_study", [grf_brick(field)], views, None, None,
                    {"cells": int(np.prod(field.shape)), "resolution": res, "angles": list(angles)})


def multiview(root=64, levels=4, n_cams=64, sizes=(128, 256, 512, 1024), seed=0, percentile=77.0,
              n_layers=8) -> Workload:
    grids = testing.amr_blob_grids(root=root, levels=levels, block_choices=(4, 8, 16), seed=seed,
                                   percentile=percentile)
    kd = AMRKDTree(grids, log_field=True)
    lg = np.log10(grids[0].data)
    tf = color_tf((lg.min(), lg.max()), n_layers)
    rng = np.random.default_rng(seed + 100)
    views = []
    for p in testing.fibonacci_sphere(n_cams, radius=1.5):
        res = int(rng.choice(sizes))
        kind = _lib.VOLUME_RENDER if rng.random() < 0.5 else _lib.INTERPOLATED_PROJECTION
        views.append(View(Camera(p, (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), res, lens_type="perspective"), kind=kind))
    return Workload("multiview", kd.bricks(), views, tf, kd,
                    {"grids": len(grids), "bricks": kd.num_bricks, "cameras": n_cams})
