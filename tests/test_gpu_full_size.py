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
