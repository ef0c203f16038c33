"""Generate the golden fixtures of tests/golden/ from yt's own compiled sampler.

Run in a checkout where the reference's sources are available (the build
recipe oracle/build_ref.py compiles them into oracle/_ref/pkg):

    python oracle/build_ref.py && python tests/golden/make_golden.py

Every fixture stores its inputs as well as the reference's outputs, so the
tests do not depend on the synthetic generators staying bit-stable.

* gz.npz        ghost_zone_interpolate (interpolators.pyx:177-226) on a 6x7x5
                random array and on a linear field (exactly reproduced, as in
                yt's own test_interpolators.py:107-150)
* trace.npz     walk_volume (grid_traversal.pyx:26-140) cell sequences and
                enter/exit t for 400 rays through an 8x6x7 brick, through
                yt's compiled walk_volume via oracle/ref_trace.pyx
* vr.npz        VolumeRenderSampler images: a 16^3 blob brick, 4-layer CTF,
                three cameras (axis-aligned and oblique plane-parallel,
                perspective), n_samples 1 and 3
* light.npz     LightSourceRenderSampler images on the vr.npz brick: three
                cameras x two lights (n_samples 1 and 3) x grey opacity {0,1}
* octree.npz    cast_through_octree with the reference's _OctreeRayTracing on a
                ~1500-cell octree: VolumeRenderSampler (1 and 2 samples),
                ProjectionSampler, InterpolatedProjectionSampler
* proj.npz      ProjectionSampler (cell-centred) and
                InterpolatedProjectionSampler (vertex-centred) images
* kd.npz        AMRKDTree leaves and viewpoint orders (amr_kdtools.pyx
                Node.add_grids / kd_traverse) for a small AMR hierarchy
* amr_vr.npz    a full AMR render: bricks from the reference's kd tree and
                vertex centring, rendered by the reference sampler in
                viewpoint order through a perspective camera
* offaxis.npz   add_cells_to_image_offaxis (image_utilities.pyx:167-289):
                octree cells splatted along oblique normals (offaxis_cases)
* near_bound.npz VolumeRenderSampler on a field within 1e-9 of a
                transfer-function bound float32 cannot represent (the
                float64 range decisions), two cameras, 1 and 3 samples
* amr_cut.npz   the amr_vr.npz render under three ColorTransferFunctions
                whose bounds cut through the data

Pass fixture names (gz trace vr light octree proj kd offaxis near_bound
amr_cut) to make only those.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle" / "_ref" / "pkg"))

from yt.utilities.lib import image_samplers as RIS  # noqa: E402
from yt.utilities.lib.amr_kdtools import Node  # noqa: E402
from yt.utilities.lib.interpolators import ghost_zone_interpolate  # noqa: E402
from yt.utilities.lib.partitioned_grid import PartitionedGrid  # noqa: E402

import ytref_trace  # noqa: E402
from oracle import glue  # noqa: E402
from yt_gb300 import testing  # noqa: E402


def ref_vertex(cell):
    out = np.zeros(tuple(s + 1 for s in cell.shape))
    ghost_zone_interpolate(1, np.ascontiguousarray(cell, dtype=np.float64), np.array([0.5] * 3), out, np.zeros(3))
    return out


def gz():
    rng = np.random.default_rng(11)
    a = rng.random((6, 7, 5))
    x, y, z = np.meshgrid(np.arange(6) + 0.5, np.arange(7) + 0.5, np.arange(5) + 0.5, indexing="ij")
    lin = 2.0 * x - 3.0 * y + 0.5 * z + 1.0
    np.savez_compressed(HERE / "gz.npz", a=a, a_out=ref_vertex(a), lin=lin, lin_out=ref_vertex(lin))


def trace():
    rng = np.random.default_rng(12)
    le, re = np.array([0.1, 0.2, 0.15]), np.array([0.9, 0.8, 0.85])
    dims = np.array([8, 6, 7], dtype=np.int64)
    n = 400
    pos = rng.uniform(-0.5, 1.5, (n, 3))
    target = rng.uniform(0.1, 0.9, (n, 3))
    dirs = (target - pos) * rng.uniform(1.0, 2.5, (n, 1))
    # axis-parallel rays, rays on cell faces and through brick corners
    for k in range(0, 60):
        ax = k % 3
        d = np.zeros(3)
        d[ax] = (1.0 if k % 2 else -1.0) * 2.0
        p = rng.uniform(0.1, 0.9, 3)
        if k % 4 == 0:
            o = (ax + 1) % 3
            p[o] = le[o] + (re[o] - le[o]) * rng.integers(0, int(dims[o]) + 1) / dims[o]
        p[ax] = -0.5 if d[ax] > 0 else 1.5
        pos[k], dirs[k] = p, d
    for k in range(60, 90):
        c = np.array([le[0], re[1], le[2]]) if k % 2 else re.copy()
        pos[k] = c - dirs[k]
    max_t = np.where(rng.random(n) < 0.2, rng.uniform(0.2, 0.9, n), 1.0)
    pg = PartitionedGrid(0, [np.zeros(tuple(dims + 1))], np.ones(tuple(dims), "uint8"), le, re, dims)
    cap = 64
    count, cells, ts = ytref_trace.trace_rays(pg, np.ascontiguousarray(pos), np.ascontiguousarray(dirs),
                                              np.ascontiguousarray(max_t), cap)
    np.savez_compressed(HERE / "trace.npz", le=le, re=re, dims=dims, pos=pos, dirs=dirs, max_t=max_t,
                        count=count, cells=cells, ts=ts)


def sampler_args(p):
    return (np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"], p["bounds"], p["image"],
            p["x_vec"], p["y_vec"], p["width"], "KDTree")


CAMS = [((0.5, 0.5, -1.0), (1.0, 1.0, 1.0), (24, 20), "plane-parallel"),
        ((1.3, 0.2, -0.7), (1.0, 1.0, 1.0), (24, 24), "plane-parallel"),
        ((0.4, 0.6, -1.2), (1.5, 1.5, 1.5), (20, 24), "perspective")]


def vr():
    g = testing.blob_grid(16, seed=0)
    v = np.log10(ref_vertex(g.data))
    lg = np.log10(g.data)
    bounds = (float(lg.min()), float(lg.max()))
    layers = testing.ctf_layers(bounds, 4)
    tf = glue.color_tf_from_layers(bounds, 64, layers)
    out = {"vertex": v, "tf_y": np.array([t.y for t in tf.tables]), "tf_bounds": np.array(bounds)}
    dims = np.array([16, 16, 16], dtype=np.int64)
    for ci, (pos, width, res, lens) in enumerate(CAMS):
        for ns in (1, 3):
            cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
            p = cam.sampler_params()
            s = RIS.VolumeRenderSampler(*sampler_args(p), tf, ns, lens_type=p["lens_type"],
                                        camera_data=p["camera_data"], zbuffer=np.ones(res))
            s(PartitionedGrid(0, [v], np.ones((16, 16, 16), "uint8"), np.zeros(3), np.ones(3), dims), num_threads=1)
            out[f"img_{ci}_{ns}"] = np.array(s.aimage)
    np.savez_compressed(HERE / "vr.npz", **out)


NB_CAMS = [((0.3, 0.6, -1.0), (1.5, 1.5, 1.5), (24, 24), "perspective"),
           ((1.2, 0.3, -0.8), (1.0, 1.0, 1.0), (20, 24), "plane-parallel")]


def near_bound():
    """VolumeRenderSampler on a field whose every vertex value lies within
    1e-9 of the upper bound b = 1 + 2^-30 of its ColorTransferFunction, a
    value float32 cannot represent: yt's float64 test keeps the samples
    below b and drops the others (field_interpolation_tables.pxd:72-73)."""
    rng = np.random.default_rng(3)
    n = 8
    b = 1.0 + 2.0 ** -30
    v = b + rng.uniform(-1e-9, 1e-9, (n + 1,) * 3)
    bounds = (b - 1.0, b)
    tf = glue.color_tf_from_layers(bounds, 256, testing.ctf_layers(bounds, 4))
    out = {"vertex": v, "tf_y": np.array([t.y for t in tf.tables]), "tf_bounds": np.array(bounds)}
    dims = np.array([n, n, n], dtype=np.int64)
    for ci, (pos, width, res, lens) in enumerate(NB_CAMS):
        for ns in (1, 3):
            cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
            p = cam.sampler_params()
            s = RIS.VolumeRenderSampler(*sampler_args(p), tf, ns, lens_type=p["lens_type"],
                                        camera_data=p["camera_data"], zbuffer=np.ones(res))
            s(PartitionedGrid(0, [v], np.ones((n, n, n), "uint8"), np.zeros(3), np.ones(3), dims), num_threads=1)
            out[f"img_{ci}_{ns}"] = np.array(s.aimage)
    np.savez_compressed(HERE / "near_bound.npz", **out)


LIGHTS = [((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0)), ((-0.3, 0.8, 0.2), (0.9, 0.5, 0.2, 1.0))]


def light():
    """LightSourceRenderSampler (image_samplers.pyx:496-590): the vr.npz brick
    and three cameras, two lights (the first at n_samples 1, the second at
    3), each with and without grey opacity."""
    g = testing.blob_grid(16, seed=0)
    v = np.log10(ref_vertex(g.data))
    lg = np.log10(g.data)
    bounds = (float(lg.min()), float(lg.max()))
    layers = testing.ctf_layers(bounds, 4)
    tf = glue.color_tf_from_layers(bounds, 64, layers)
    tfg = glue.color_tf_from_layers(bounds, 64, layers)
    tfg.grey_opacity = 1
    out = {"vertex": v, "tf_y": np.array([t.y for t in tf.tables]), "tf_bounds": np.array(bounds)}
    dims = np.array([16, 16, 16], dtype=np.int64)
    for ci, (pos, width, res, lens) in enumerate(CAMS):
        for li, (ldir, lrgba) in enumerate(LIGHTS):
            for ns in ((1,) if li == 0 else (3,)):
                for grey, t in ((0, tf), (1, tfg)):
                    cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
                    p = cam.sampler_params()
                    s = RIS.LightSourceRenderSampler(*sampler_args(p), t, ns, light_dir=np.array(ldir),
                                                     light_rgba=np.array(lrgba), lens_type=p["lens_type"],
                                                     camera_data=p["camera_data"], zbuffer=np.ones(res))
                    s(PartitionedGrid(0, [v], np.ones((16, 16, 16), "uint8"), np.zeros(3), np.ones(3), dims),
                      num_threads=1)
                    out[f"img_{ci}_{li}_{ns}_{grey}"] = np.array(s.aimage)
    np.savez_compressed(HERE / "light.npz", **out)


def octree():
    """cast_through_octree (image_samplers.pyx:202-288) with the reference's
    _OctreeRayTracing (_octree_raytracing.hpp): a ~1500-cell octree (levels
    2-5) through a perspective camera (the octree path reads per-pixel ray
    arrays), VolumeRenderSampler with 1 and 2 samples, ProjectionSampler and
    InterpolatedProjectionSampler."""
    from yt.utilities.lib._octree_raytracing import _OctreeRayTracing

    depth, ipos, lvl, cells = testing.octree_cells(base_level=2, max_level=5, seed=2)
    key = np.arange(ipos.shape[0], dtype=np.int32)
    le, re = np.zeros(3), np.ones(3)
    oc = _OctreeRayTracing(le, re, depth)
    oc.add_nodes(ipos, lvl, key)
    vmin, vmax = float(cells[:, :8].min()), float(cells[:, :8].max())
    layers = testing.ctf_layers((vmin, vmax), 4)
    tf = glue.color_tf_from_layers((vmin, vmax), 64, layers)
    out = {"depth": depth, "ipos": ipos, "lvl": lvl, "cells": cells, "tf_y": np.array([t.y for t in tf.tables]),
           "tf_bounds": np.array((vmin, vmax))}
    dt = cells.reshape(1, -1, 14, 1)
    pg = PartitionedGrid(0, dt, np.ones(dt.shape[1:], dtype=np.uint8), le, re, np.array([1, 1, 1], dtype="int64"),
                         n_fields=1)
    cam = glue.Camera((0.3, 1.45, -0.9), (0.5, 0.5, 0.5), (1.3, 1.3, 1.3), (26, 22), lens_type="perspective")
    for name, make in (("vr1", lambda p: RIS.VolumeRenderSampler(*sampler_args_oct(p), tf, 1, **lens_kw(p))),
                       ("vr2", lambda p: RIS.VolumeRenderSampler(*sampler_args_oct(p), tf, 2, **lens_kw(p))),
                       ("proj", lambda p: RIS.ProjectionSampler(*sampler_args_oct(p), **lens_kw(p))),
                       ("iproj", lambda p: RIS.InterpolatedProjectionSampler(*sampler_args_oct(p), 2,
                                                                             **lens_kw(p)))):
        p = cam.sampler_params()
        s = make(p)
        s(pg, oct=oc)
        out[f"img_{name}"] = np.array(s.aimage)
    np.savez_compressed(HERE / "octree.npz", **out)


def sampler_args_oct(p):
    return (p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"], p["x_vec"], p["y_vec"], p["width"],
            "Octree")


def lens_kw(p):
    return {"lens_type": p["lens_type"], "camera_data": p["camera_data"], "zbuffer": np.ones(p["image"].shape[:2])}


def proj():
    rng = np.random.default_rng(13)
    cell = np.exp(rng.standard_normal((12, 12, 12)))
    v = ref_vertex(cell)
    dims = np.array([12, 12, 12], dtype=np.int64)
    out = {"cell": cell}
    for ci, (pos, width, res, lens) in enumerate(CAMS):
        cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
        p = cam.sampler_params()
        s = RIS.ProjectionSampler(*sampler_args(p), 1, lens_type=p["lens_type"], camera_data=p["camera_data"],
                                  zbuffer=np.ones(res))
        s(PartitionedGrid(0, [cell], np.ones((12, 12, 12), "uint8"), np.zeros(3), np.ones(3), dims), num_threads=1)
        out[f"proj_{ci}"] = np.array(s.aimage)
        cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
        p = cam.sampler_params()
        s = RIS.InterpolatedProjectionSampler(*sampler_args(p), 2, lens_type=p["lens_type"],
                                              camera_data=p["camera_data"], zbuffer=np.ones(res))
        s(PartitionedGrid(0, [v], np.ones((12, 12, 12), "uint8"), np.zeros(3), np.ones(3), dims), num_threads=1)
        out[f"iproj_{ci}"] = np.array(s.aimage)
    np.savez_compressed(HERE / "proj.npz", **out)


def ref_tree(gles, gres, gids, levels):
    trunk = Node(None, None, None, np.array([-np.inf] * 3), np.array([np.inf] * 3), -1, 1)
    for lvl in range(int(levels.max()) + 1):
        sel = levels == lvl
        if sel.any():
            trunk.add_grids(int(sel.sum()), np.ascontiguousarray(gles[sel]), np.ascontiguousarray(gres[sel]),
                            np.ascontiguousarray(gids[sel]), 0, 1)
    return trunk


def kd_and_amr():
    grids = testing.amr_blob_grids(root=16, levels=2, patch=8, seed=3)
    gles = np.array([g.left_edge for g in grids])
    gres = np.array([g.right_edge for g in grids])
    gids = np.array([g.id for g in grids], dtype=np.int64)
    levels = np.array([g.level for g in grids], dtype=np.int32)
    trunk = ref_tree(gles, gres, gids, levels)
    leaves = list(trunk.kd_traverse())
    le = np.array([n.get_left_edge() for n in leaves])
    re = np.array([n.get_right_edge() for n in leaves])
    lg = np.array([n.grid for n in leaves], dtype=np.int64)
    vps = np.array([[0.5, 0.5, -5.0], [2.0, 0.3, 0.6], [0.2, 1.7, 1.9], [0.55, 0.45, 0.5]])
    keyidx = {(tuple(a), tuple(b)): k for k, (a, b) in enumerate(zip(le, re))}
    orders = []
    for vp in vps:
        orders.append([keyidx[(tuple(n.get_left_edge()), tuple(n.get_right_edge()))]
                       for n in trunk.kd_traverse(viewpoint=vp)])
    cells = [g.data for g in grids]
    np.savez_compressed(HERE / "kd.npz", gles=gles, gres=gres, gids=gids, levels=levels, leaf_le=le, leaf_re=re,
                        leaf_grid=lg, viewpoints=vps, orders=np.array(orders, dtype=np.int32),
                        **{f"cell_{g.id}": g.data for g in grids})
    # a full AMR render through the reference
    vcd = {g.id: np.log10(ref_vertex(g.data)) for g in grids}
    byid = {g.id: g for g in grids}
    lg0 = np.log10(cells[0])
    bounds = (float(lg0.min()), float(lg0.max()))
    tf = glue.color_tf_from_layers(bounds, 128, testing.ctf_layers(bounds, 6))
    cam = glue.Camera((0.3, 0.6, -1.1), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), (32, 28), lens_type="perspective")
    p = cam.sampler_params()
    s = RIS.VolumeRenderSampler(*sampler_args(p), tf, 1, lens_type=p["lens_type"], camera_data=p["camera_data"],
                                zbuffer=np.ones((32, 28)))
    for node in trunk.kd_traverse(viewpoint=cam.viewpoint):
        g = byid[node.grid]
        nle, nre = node.get_left_edge(), node.get_right_edge()
        li = np.rint((nle - g.left_edge) / g.dds).astype("int32")
        ri = np.rint((nre - g.left_edge) / g.dds).astype("int32")
        dims = (ri - li).astype("int64")
        d = vcd[g.id][li[0]: ri[0] + 1, li[1]: ri[1] + 1, li[2]: ri[2] + 1].copy()
        s(PartitionedGrid(g.id, [d], np.ones(dims, "uint8"), nle, nre, dims), num_threads=1)
    np.savez_compressed(HERE / "amr_vr.npz", image=np.array(s.aimage), tf_y=np.array([t.y for t in tf.tables]),
                        tf_bounds=np.array(bounds), viewpoint=cam.viewpoint)


AMR_CUT_BOUNDS = [(0.05, 0.55), (0.25, 0.95), (-0.1, 0.4)]


def amr_cut():
    """The amr_vr.npz render with ColorTransferFunctions whose bounds cut
    through the data (the served form's kind: samples at the bounds are
    common, the brightest layer 1/60 of the range from the upper bound)."""
    grids = testing.amr_blob_grids(root=16, levels=2, patch=8, seed=3)
    gles = np.array([g.left_edge for g in grids])
    gres = np.array([g.right_edge for g in grids])
    gids = np.array([g.id for g in grids], dtype=np.int64)
    levels = np.array([g.level for g in grids], dtype=np.int32)
    trunk = ref_tree(gles, gres, gids, levels)
    vcd = {g.id: np.log10(ref_vertex(g.data)) for g in grids}
    byid = {g.id: g for g in grids}
    cam = glue.Camera((0.3, 0.6, -1.1), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), (32, 28), lens_type="perspective")
    out = {"viewpoint": cam.viewpoint}
    for k, bounds in enumerate(AMR_CUT_BOUNDS):
        tf = glue.color_tf_from_layers(bounds, 128, testing.ctf_layers(bounds, 6))
        p = cam.sampler_params()  # (a new image for each render)
        s = RIS.VolumeRenderSampler(*sampler_args(p), tf, 1, lens_type=p["lens_type"], camera_data=p["camera_data"],
                                    zbuffer=np.ones((32, 28)))
        for node in trunk.kd_traverse(viewpoint=cam.viewpoint):
            g = byid[node.grid]
            nle, nre = node.get_left_edge(), node.get_right_edge()
            li = np.rint((nle - g.left_edge) / g.dds).astype("int32")
            ri = np.rint((nre - g.left_edge) / g.dds).astype("int32")
            dims = (ri - li).astype("int64")
            d = vcd[g.id][li[0]: ri[0] + 1, li[1]: ri[1] + 1, li[2]: ri[2] + 1].copy()
            s(PartitionedGrid(g.id, [d], np.ones(dims, "uint8"), nle, nre, dims), num_threads=1)
        out[f"image_{k}"] = np.array(s.aimage)
        out[f"tf_y_{k}"] = np.array([t.y for t in tf.tables])
        out[f"tf_bounds_{k}"] = np.array(bounds)
    np.savez_compressed(HERE / "amr_cut.npz", **out)


def offaxis_cases():
    """Inputs of offaxis.npz: the cells of a small octree (levels 2-5) seen
    along oblique normals on square, non-square (Nx < Ny), one- and
    two-pixel images; the last case adds cells wider than the image (more
    stamp subcells per row than the device table holds) and cells partly
    or wholly outside the image.  Returns (base cells, extra cells, views)."""
    from yt_gb300.camera import Camera

    _, _, _, cells = testing.octree_cells(base_level=2, max_level=5, seed=2)
    le, re = cells[:, 8:11], cells[:, 11:14]
    rng = np.random.default_rng(21)
    base = ((le + re) / 2 - 0.5, np.ascontiguousarray((re - le)[:, 0]), cells[:, :8].mean(axis=1),
            rng.uniform(0.5, 2.0, cells.shape[0]))
    bx = np.array([[0.1, -0.2, 0.05], [-0.3, 0.25, 0.0], [0.45, 0.45, -0.1]])
    extra = (np.concatenate([bx, rng.uniform(-0.8, 0.8, (40, 3))]),
             np.concatenate([[1.3, 0.6, 0.35], rng.choice([1 / 16, 1 / 32, 1 / 64], 40)]),
             rng.uniform(0.1, 3, 43), rng.uniform(0.5, 2, 43))
    views = []
    for pos, nx, ny, ext in [((0.1, 0.3, -1.2), 40, 40, False), ((1.3, 0.2, 0.4), 32, 56, False),
                             ((0.5, 0.5, -1.0), 1, 1, False), ((0.2, 0.9, -0.7), 2, 2, False),
                             ((-0.4, 1.1, 0.3), 120, 120, True)]:
        cam = Camera(pos, (0.5, 0.5, 0.5), (1, 1, 1), (nx, ny), lens_type="plane-parallel")
        views.append((np.ascontiguousarray(cam.inv_mat.T), nx, ny, ext))
    return base, extra, views


def offaxis_inputs(base, extra, ext):
    """The cell arrays of one offaxis.npz case (base cells, plus the extra
    ones when ext)."""
    if not ext:
        return tuple(np.ascontiguousarray(a) for a in base)
    return tuple(np.ascontiguousarray(np.concatenate([a, b])) for a, b in zip(base, extra))


def offaxis():
    from yt.utilities.lib import image_utilities as RIU

    base, extra, views = offaxis_cases()
    arrays = {"X": base[0], "D": base[1], "Q": base[2], "W": base[3], "eX": extra[0], "eD": extra[1],
              "eQ": extra[2], "eW": extra[3]}
    for i, (rot, nx, ny, ext) in enumerate(views):
        X, D, Q, W = offaxis_inputs(base, extra, ext)
        b, bw = np.zeros((nx, ny)), np.zeros((nx, ny))
        RIU.add_cells_to_image_offaxis(Xp=X, dXp=D, qty=Q, weight=W, rotation=rot, buffer=b, buffer_weight=bw,
                                       Nx=nx, Ny=ny)
        arrays.update({f"rot{i}": rot, f"view{i}": np.array([nx, ny, int(ext)]), f"b{i}": b, f"bw{i}": bw})
    np.savez_compressed(HERE / "offaxis.npz", n=len(views), **arrays)


ALL = {"gz": gz, "trace": trace, "vr": vr, "light": light, "octree": octree, "proj": proj, "kd": kd_and_amr,
       "offaxis": offaxis, "near_bound": near_bound, "amr_cut": amr_cut}

if __name__ == "__main__":
    for name in sys.argv[1:] or list(ALL):
        ALL[name]()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)
