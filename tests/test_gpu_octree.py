"""The octree path (ytgb_render_octree) against the oracle's
cast_through_octree (pinned to the compiled reference by
tests/golden/octree.npz): traversal bit for bit, images within 1e-5, for
every sampler; and the drop-in sampler with yt's call."""
import numpy as np
import pytest
import torch

from oracle import cpu as ocpu
from yt_gb300 import _lib, testing
from yt_gb300.camera import Camera
from yt_gb300.octree import Octree, OctreeVolume, render_octree, trace_octree
from yt_gb300.render import relative_error
from yt_gb300.transfer_functions import ColorTransferFunction, pack

pytestmark = pytest.mark.gpu

KN = {_lib.VOLUME_RENDER: "volume_render", _lib.PROJECTION: "projection",
      _lib.INTERPOLATED_PROJECTION: "interpolated_projection", _lib.MIP: "mip", _lib.LIGHT_SOURCE: "light_source"}
LIGHT = ((-0.3, 0.8, 0.2), (0.9, 0.5, 0.2, 1.0))


def dataset(seed=2, base=3, top=6):
    depth, ipos, lvl, cells = testing.octree_cells(base_level=base, max_level=top, seed=seed)
    oc = Octree(np.zeros(3), np.ones(3), depth)
    oc.add_nodes(ipos, lvl, np.arange(ipos.shape[0], dtype=np.int32))
    vmin, vmax = float(cells[:, :8].min()), float(cells[:, :8].max())
    tf = ColorTransferFunction((vmin, vmax), nbins=64)
    for loc, wd, rgba in testing.ctf_layers((vmin, vmax), 4):
        tf.add_gaussian(loc, wd, list(rgba))
    return depth, ipos, lvl, cells, oc, tf


@pytest.mark.parametrize("kind", list(KN))
def test_octree_matches_oracle(cuda, kind):
    depth, ipos, lvl, cells, oc, tf = dataset()
    vol = OctreeVolume(oc, cells, cuda)
    cam = Camera((0.3, 1.45, -0.9), (0.5, 0.5, 0.5), (1.3, 1.3, 1.3), (48, 40), lens_type="perspective")
    view = cam.device_view()
    uses_tf = kind in (_lib.VOLUME_RENDER, _lib.LIGHT_SOURCE)
    light = LIGHT if kind == _lib.LIGHT_SOURCE else None
    oo = ocpu.OracleOctree(depth, np.zeros(3), np.ones(3), ipos, lvl)
    for ns in ((1, 3) if kind in (_lib.VOLUME_RENDER, _lib.INTERPOLATED_PROJECTION) else (1,)):
        img = torch.zeros((48, 40, 4), dtype=torch.float64, device=cuda)
        counters = torch.zeros(4, dtype=torch.int64, device=cuda)
        error = torch.zeros(1, dtype=torch.int32, device=cuda)
        render_octree(vol, view, kind, img, tf=pack(tf) if uses_tf else None, n_samples=ns, counters=counters,
                      error=error, light=light)
        torch.cuda.synchronize()
        assert int(error.item()) == 0
        p = cam.sampler_params()
        ld, lrgba = light if light else ((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0))
        s = ocpu.OracleSampler(KN[kind], p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"], p["x_vec"],
                               p["y_vec"], p["width"], lens_type=p["lens_type"], camera_data=p["camera_data"],
                               n_samples=ns, tf=tf if uses_tf else None, light_dir=ld, light_rgba=lrgba)
        visits = ocpu.render_octree(s, cells, oo)
        assert int(counters[0].item()) == visits > 0
        mx, rms = relative_error(img.cpu().numpy(), p["image"], channels=(0, 1, 2) if uses_tf else (0,))
        assert mx <= 1e-5, f"max relative error {mx:.3e} (rms {rms:.3e})"
    h, c = trace_octree(vol, view)
    hr, cr = ocpu.trace_octree(s, cells, oo)
    assert np.array_equal(c, cr) and np.array_equal(h, hr)


@pytest.mark.parametrize("held", [False, True])
@pytest.mark.parametrize("host_pack", ["0", "1"])
def test_octree_drop_in(cuda, held, host_pack, monkeypatch):
    """VolumeRenderSampler(..., "Octree") called as OctreeVolumeSource.render
    calls it: sampler(pg, oct=octree) with the 14-values-per-cell grid,
    into a new image or one that holds values; rendered in the caller's host
    arrays where the device reads host memory, else through device copies
    (YTGB_HOST_PACK=1)."""
    from yt_gb300.image_samplers import VolumeRenderSampler
    from yt_gb300.partitioned_grid import PartitionedGrid

    depth, ipos, lvl, cells, oc, tf = dataset(seed=4)
    cam = Camera((1.4, 0.3, -0.6), (0.5, 0.5, 0.5), (1.2, 1.2, 1.2), (32, 32), lens_type="perspective")
    p = cam.sampler_params()
    le, re = np.zeros(3), np.ones(3)
    dt = cells.reshape(1, -1, 14, 1)
    pg = PartitionedGrid(0, dt, np.ones(dt.shape[1:], dtype=np.uint8), le, re, np.array([1, 1, 1]), n_fields=1)
    monkeypatch.setenv("YTGB_HOST_PACK", host_pack)
    init = np.random.default_rng(2).uniform(0.0, 0.3, p["image"].shape) if held else np.zeros(p["image"].shape)
    p["image"][...] = init
    s = VolumeRenderSampler(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"], p["x_vec"], p["y_vec"],
                            p["width"], "Octree", tf, 2, lens_type=p["lens_type"], camera_data=p["camera_data"])
    s(pg, oct=oc)
    img = s.aimage.copy()
    p2 = cam.sampler_params()
    p2["image"][...] = init
    so = ocpu.OracleSampler("volume_render", p2["vp_pos"], p2["vp_dir"], p2["center"], p2["bounds"], p2["image"],
                            p2["x_vec"], p2["y_vec"], p2["width"], lens_type=p2["lens_type"],
                            camera_data=p2["camera_data"], n_samples=2, tf=tf)
    ocpu.render_octree(so, cells, ocpu.OracleOctree(depth, le, re, ipos, lvl))
    assert relative_error(img, p2["image"], channels=(0, 1, 2))[0] <= 1e-5


@pytest.mark.parametrize("kind", [_lib.PROJECTION, _lib.MIP])
def test_octree_axis_rays(cuda, kind):
    """Per-pixel rays with zero direction components (infinite slab t, NaN
    midpoints: the traversal's float64-comparison branch) through the
    drop-in sampler, and their traversal bit for bit."""
    from yt_gb300.image_samplers import MIPSampler, ProjectionSampler, make_view
    from yt_gb300.partitioned_grid import PartitionedGrid

    depth, ipos, lvl, cells, oc, tf = dataset()
    nx, ny = 40, 36
    pos, d = testing.axis_rays(nx, ny)
    cam = Camera((0.3, 1.45, -0.9), (0.5, 0.5, 0.5), (1.3, 1.3, 1.3), (nx, ny), lens_type="perspective")
    p = cam.sampler_params()
    le, re = np.zeros(3), np.ones(3)
    dt = cells.reshape(1, -1, 14, 1)
    pg = PartitionedGrid(0, dt, np.ones(dt.shape[1:], dtype=np.uint8), le, re, np.array([1, 1, 1]), n_fields=1)
    cls = ProjectionSampler if kind == _lib.PROJECTION else MIPSampler
    s = cls(pos, d, p["center"], p["bounds"], np.zeros((nx, ny, 4)), p["x_vec"], p["y_vec"], p["width"], "Octree",
            lens_type="perspective", camera_data=p["camera_data"])
    s(pg, oct=oc)
    img = s.aimage.copy()
    ref = np.zeros((nx, ny, 4))
    so = ocpu.OracleSampler(KN[kind], pos, d, p["center"], p["bounds"], ref, p["x_vec"], p["y_vec"], p["width"],
                            lens_type="perspective", camera_data=p["camera_data"])
    oo = ocpu.OracleOctree(depth, le, re, ipos, lvl)
    ocpu.render_octree(so, cells, oo)
    assert relative_error(img, ref, channels=(0,))[0] <= 1e-5
    vol = OctreeVolume(oc, cells, cuda)
    view, ppos, pdir = make_view(pos, d, p["center"], p["bounds"], nx, ny, p["x_vec"], p["y_vec"], p["width"],
                                 "perspective", p["camera_data"])
    tp, td = torch.from_numpy(ppos).to(cuda), torch.from_numpy(pdir).to(cuda)
    view.px_pos, view.px_dir = tp.data_ptr(), td.data_ptr()
    h, c = trace_octree(vol, view)
    hr, cr = ocpu.trace_octree(so, cells, oo)
    assert np.array_equal(c, cr) and np.array_equal(h, hr) and c.sum() > 0
