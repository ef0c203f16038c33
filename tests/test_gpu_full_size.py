"""The benchmark frame itself against the oracle: the default bench.py
workload (128^3 root + 3 levels, 1145 kd bricks, perspective 1024^2, 8-layer
ColorTransferFunction; 101 M samples).  Every ray's visited-cell trace is
bit-identical to the oracle's walk_volume, the sample counts are equal and
the image is within 1e-5 of the float64 render."""
import pytest

from test_gpu_parity import check_view
from yt_gb300 import _lib, workloads
from yt_gb300.render import Renderer

pytestmark = pytest.mark.gpu


def test_benchmark_frame_matches_oracle(cuda):
    w = workloads.amr_vr()
    assert w.kdtree.num_bricks == 1145
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    img, ref, mx = check_view(r, w.bricks, w.views[0].camera, _lib.VOLUME_RENDER, tf=w.tf)
    assert img.shape == (1024, 1024, 4) and ref.max() > 0


def test_octree_benchmark_frame_matches_oracle(cuda):
    """The octree benchmark frame (217,512 cells on levels 5-9, perspective
    1024^2, VolumeRenderSampler): traversal hash and counts per pixel equal
    the oracle's cast_through_octree, image within 1e-5."""
    import numpy as np
    import torch

    from oracle import cpu as ocpu
    from yt_gb300 import testing
    from yt_gb300.camera import Camera
    from yt_gb300.octree import Octree, OctreeVolume, render_octree, trace_octree
    from yt_gb300.render import relative_error
    from yt_gb300.transfer_functions import pack

    depth, ipos, lvl, cells = testing.octree_cells(base_level=5, max_level=9, seed=0, percentile=85.0)
    oc = Octree(np.zeros(3), np.ones(3), depth)
    oc.add_nodes(ipos, lvl, np.arange(ipos.shape[0], dtype=np.int32))
    vol = OctreeVolume(oc, cells, cuda)
    vmin, vmax = float(cells[:, :8].min()), float(cells[:, :8].max())
    tf = workloads.color_tf((vmin, vmax), 8)
    cam = Camera((0.52, 0.47, -1.0), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), 1024, lens_type="perspective")
    img = torch.zeros((1024, 1024, 4), dtype=torch.float64, device=cuda)
    counters = torch.zeros(4, dtype=torch.int64, device=cuda)
    render_octree(vol, cam.device_view(), _lib.VOLUME_RENDER, img, tf=pack(tf), counters=counters)
    h, c = trace_octree(vol, cam.device_view())
    p = cam.sampler_params()
    s = ocpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                           p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                           camera_data=p["camera_data"], tf=tf)
    oo = ocpu.OracleOctree(depth, np.zeros(3), np.ones(3), ipos, lvl)
    visits = ocpu.render_octree(s, cells, oo)
    hr, cr = ocpu.trace_octree(s, cells, oo)
    assert int(counters[0].item()) == visits and visits > 27_000_000
    assert np.array_equal(c, cr) and np.array_equal(h, hr)
    mx, rms = relative_error(img.cpu().numpy(), p["image"], channels=(0, 1, 2))
    assert mx <= 1e-5, f"max relative error {mx:.3e}"
