"""Benchmark frames built and rendered by the reference alone -- TEST INFRASTRUCTURE.

``bench.py``'s CPU baseline and its accuracy check use these: the same seeded
grids the product renders (``yt_gb300.testing``, plain numpy), but every step
between the grids and the image is the reference's own compiled code, built
by ``oracle/build_ref.py``:

* the kd-tree: ``amr_kdtools.Node.add_grids`` level by level, as
  ``Tree.build`` drives it (``yt/utilities/amr_kdtree/amr_kdtree.py:109-118``,
  ``yt/utilities/lib/amr_kdtools.pyx:201-532``), and the brick order
  ``Node.kd_traverse(viewpoint)`` (``amr_kdtools.pyx:102-111,612-755``);
* the brick data: ``interpolators.ghost_zone_interpolate`` vertex centring
  (``interpolators.pyx:177-226``, as ``grid_patch.py:270-296`` calls it
  without ghost zones), ``log10`` with values <= 0 as NaN and the per-leaf
  slice (``amr_kdtree.py:325-374``);
* the render: ``image_samplers.VolumeRenderSampler`` called once per brick in
  kd order (``render_source.py:594-596`` over ``image_samplers.pyx:146-197``).

The camera and transfer function are the numpy restatements of
``oracle/glue.py``.  Nothing here loads ``libytgb``: a reference timing that
went through the product's kd-tree or brick preparation would not be the
reference.  ``loaded_native_libraries()`` lists what the process has mapped,
so a caller can show it.
"""
from __future__ import annotations

import sys
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import glue

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent


def ref_pkg(timed: bool) -> Path | None:
    """The compiled reference: ``pkg_timed`` (yt's own compiler flags) for
    timing, ``pkg`` (``-ffp-contract=off``, bit-exact float64) for checking.
    None when it was not built."""
    p = HERE / "_ref" / ("pkg_timed" if timed else "pkg")
    if any((p / "yt" / "utilities" / "lib").glob("image_samplers*.so")):
        return p
    return None


_MODULES = {}


def reference_modules(timed: bool):
    """Import the reference's compiled modules from one build.  Both builds
    define the same package name, so a process uses one of them; asking for
    the other afterwards raises."""
    key = "timed" if timed else "exact"
    if _MODULES:
        if key not in _MODULES:
            raise RuntimeError("a process can load only one build of the reference (both are package 'yt')")
        return _MODULES[key]
    pkg = ref_pkg(timed)
    if pkg is None:
        raise ImportError(f"the reference sampler is not built ({'pkg_timed' if timed else 'pkg'})")
    sys.path.insert(0, str(pkg))
    from yt.utilities.lib import image_samplers  # noqa: PLC0415
    from yt.utilities.lib.amr_kdtools import Node  # noqa: PLC0415
    from yt.utilities.lib.interpolators import ghost_zone_interpolate  # noqa: PLC0415
    from yt.utilities.lib.partitioned_grid import PartitionedGrid  # noqa: PLC0415

    _MODULES[key] = {"image_samplers": image_samplers, "Node": Node, "ghost_zone_interpolate": ghost_zone_interpolate,
                     "PartitionedGrid": PartitionedGrid, "pkg": str(pkg)}
    return _MODULES[key]


@dataclass
class Frame:
    """One view of a kd-decomposed volume, ready for the reference sampler.
    ``kind`` is "reference" when the reference's compiled kd-tree, vertex
    centring and sampler built and render it, "port" when the reference is
    not built and the restatements (``glue.KDTree``, the C oracle) stand in."""

    bricks: list          # (data list, mask, le, re, dims) in kd viewpoint order
    camera: glue.Camera
    tf: object            # glue.ColorTransferFunction
    n_grids: int
    build_seconds: float
    mods: dict | None
    kind: str = "reference"

    def partitioned_grids(self):
        if self.mods is None:
            return None
        PG = self.mods["PartitionedGrid"]
        return [PG(0, d, m, le, re, np.asarray(dims, dtype=np.int64)) for d, m, le, re, dims in self.bricks]

    def with_resolution(self, res) -> "Frame":
        cam = glue.Camera(self.camera.position, self.camera.focus, self.camera.width, res,
                          lens_type=self.camera.lens_type)
        return Frame(self.bricks, cam, self.tf, self.n_grids, 0.0, self.mods, self.kind)


def _vertex_log10(gzi, cell):
    out = np.zeros(tuple(s + 1 for s in cell.shape))
    gzi(1, np.ascontiguousarray(cell, dtype=np.float64), np.array([0.5] * 3), out, np.zeros(3))
    out[out <= 0] = np.nan
    return np.log10(out)


def _port_frame(grids, camera: glue.Camera, tf) -> Frame:
    """The same bricks from the restatements, where the reference is not built."""
    t0 = time.perf_counter()
    tree = glue.KDTree(grids)
    byid = {g.id: g for g in grids}
    vcd = {}
    bricks = []
    for node in tree.leaves(camera.viewpoint):
        g = byid[node.grid]
        if g.id not in vcd:
            vcd[g.id] = [glue.vertex_centred(g.data, log=True)]
        bricks.append(glue.brick_data(node, g, vcd[g.id]))
    return Frame(bricks, camera, tf, len(grids), time.perf_counter() - t0, None, "port")


def kd_frame(grids, camera: glue.Camera, tf, timed=True, allow_port=False) -> Frame:
    """Bricks of ``grids`` (objects with id, level, left_edge, right_edge,
    dims, data) in the reference's kd viewpoint order for ``camera``.  With
    ``allow_port`` a missing reference build falls back to the restatements."""
    try:
        mods = reference_modules(timed)
    except ImportError:
        if not allow_port:
            raise
        return _port_frame(grids, camera, tf)
    t0 = time.perf_counter()
    gles = np.array([g.left_edge for g in grids], dtype=np.float64)
    gres = np.array([g.right_edge for g in grids], dtype=np.float64)
    gids = np.array([g.id for g in grids], dtype=np.int64)
    levels = np.array([g.level for g in grids], dtype=np.int32)
    trunk = mods["Node"](None, None, None, np.array([-np.inf] * 3), np.array([np.inf] * 3), -1, 1)
    for lvl in range(int(levels.max()) + 1):
        sel = levels == lvl
        if sel.any():
            trunk.add_grids(int(sel.sum()), np.ascontiguousarray(gles[sel]), np.ascontiguousarray(gres[sel]),
                            np.ascontiguousarray(gids[sel]), 0, 1)
    byid = {g.id: g for g in grids}
    vcd = {}
    bricks = []
    for node in trunk.kd_traverse(viewpoint=camera.viewpoint):
        g = byid[node.grid]
        if g.id not in vcd:
            vcd[g.id] = _vertex_log10(mods["ghost_zone_interpolate"], g.data)
        nle, nre = np.array(node.get_left_edge()), np.array(node.get_right_edge())
        dds = (g.right_edge - g.left_edge) / g.dims
        li = np.rint((nle - g.left_edge) / dds).astype("int32")
        ri = np.rint((nre - g.left_edge) / dds).astype("int32")
        dims = (ri - li).astype("int64")
        d = vcd[g.id][li[0]: ri[0] + 1, li[1]: ri[1] + 1, li[2]: ri[2] + 1].copy()
        bricks.append(([d], np.ones(dims, "uint8"), nle, nre, dims))
    return Frame(bricks, camera, tf, len(grids), time.perf_counter() - t0, mods)


def amr_frame(root=128, levels=3, res=1024, seed=0, n_layers=8, patch=16, timed=True, allow_port=False) -> Frame:
    """The AMR volume-render benchmark frame: a ``root``^3 blob grid refined
    by factor 2 ``levels`` times in ``patch``^3 patches, an ``n_layers``
    ColorTransferFunction over the root grid's log10 range (256 bins, width
    0.01), a perspective camera at (0.5, 0.5, -1) looking at the centre with
    width 1.5, ``res``^2 pixels."""
    from yt_gb300 import testing  # noqa: PLC0415  (numpy-only dataset generator)

    grids = testing.amr_blob_grids(root=root, levels=levels, patch=patch, seed=seed)
    lg = np.log10(grids[0].data)
    bounds = (float(lg.min()), float(lg.max()))
    tf = glue.color_tf_from_layers(bounds, 256, testing.ctf_layers(bounds, n_layers, width=0.01))
    cam = glue.Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), res, lens_type="perspective")
    return kd_frame(grids, cam, tf, timed=timed, allow_port=allow_port)


def uniform_frame(n=64, res=256, seed=0, n_layers=4, timed=True, allow_port=False) -> Frame:
    """The small uniform case: one ``n``^3 blob grid as one brick, a
    plane-parallel view down +z (width 1), ``n_layers`` ColorTransferFunction."""
    from yt_gb300 import testing  # noqa: PLC0415

    g = testing.blob_grid(n, seed=seed)
    lg = np.log10(g.data)
    bounds = (float(lg.min()), float(lg.max()))
    tf = glue.color_tf_from_layers(bounds, 256, testing.ctf_layers(bounds, n_layers, width=0.01))
    cam = glue.Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), res, lens_type="plane-parallel")
    return kd_frame([g], cam, tf, timed=timed, allow_port=allow_port)


def render(frame: Frame, threads: int, pgs=None):
    """yt's brick loop over the reference's compiled VolumeRenderSampler:
    returns (seconds spent in the sampler calls, float64 image).  A "port"
    frame is rendered by the C oracle instead."""
    if frame.mods is None:
        t0 = time.perf_counter()
        img, _ = oracle_render(frame, threads)
        return time.perf_counter() - t0, img
    p = frame.camera.sampler_params()
    RIS = frame.mods["image_samplers"]
    pgs = pgs if pgs is not None else frame.partitioned_grids()
    s = RIS.VolumeRenderSampler(np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"], p["bounds"],
                                p["image"], p["x_vec"], p["y_vec"], p["width"], "KDTree", frame.tf, 1,
                                lens_type=p["lens_type"], camera_data=p["camera_data"],
                                zbuffer=np.ones(p["image"].shape[:2]))
    t0 = time.perf_counter()
    for pg in pgs:
        s(pg, num_threads=threads)
    dt = time.perf_counter() - t0
    return dt, np.array(s.aimage)


def oracle_render(frame: Frame, threads: int):
    """The C oracle (``ytoracle.c``, pinned bit for bit to the reference) on
    the same frame: (float64 image, samples).  The sample count is the
    number of cells the walk visits, which the reference sampler does not
    report."""
    from . import cpu  # noqa: PLC0415

    p = frame.camera.sampler_params()
    s = cpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                          p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                          camera_data=p["camera_data"], tf=frame.tf, n_samples=1)
    samples = s.render(cpu.OracleBricks(frame.bricks), None, num_threads=threads)
    return p["image"], int(samples)


def loaded_native_libraries():
    """Shared objects mapped into this process that belong to this checkout."""
    out = set()
    try:
        for line in Path("/proc/self/maps").read_text().splitlines():
            parts = line.split()
            if len(parts) < 6:
                continue
            path = parts[-1]
            if (path.endswith(".so") or ".so." in path) and path.startswith(str(ROOT)):
                out.add(str(Path(path).relative_to(ROOT)))
    except OSError:
        pass
    return sorted(out)
