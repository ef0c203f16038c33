"""GPU renders of the golden inputs against yt's own images (tests/golden/,
made by tests/golden/make_golden.py from the reference's compiled sampler).
Tolerance: 1e-5 per-pixel relative error (tau = 1e-6)."""
from pathlib import Path

import numpy as np
import pytest

from yt_gb300 import _lib
from yt_gb300.camera import Camera
from yt_gb300.render import Renderer, relative_error
from yt_gb300.transfer_functions import ColorTransferFunction

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
CAMS = [((0.5, 0.5, -1.0), (1.0, 1.0, 1.0), (24, 20), "plane-parallel"),
        ((1.3, 0.2, -0.7), (1.0, 1.0, 1.0), (24, 24), "plane-parallel"),
        ((0.4, 0.6, -1.2), (1.5, 1.5, 1.5), (20, 24), "perspective")]


def golden_tf(bounds, ys):
    tf = ColorTransferFunction(tuple(bounds), nbins=ys.shape[1])
    for t, y in zip(tf.funcs, ys):
        t.y = y.copy()
    return tf


@pytest.mark.parametrize("ci", range(3))
@pytest.mark.parametrize("ns", [1, 3])
def test_vr_against_reference_images(cuda, ci, ns):
    f = np.load(GOLD / "vr.npz")
    tf = golden_tf(f["tf_bounds"], f["tf_y"])
    pos, width, res, lens = CAMS[ci]
    r = Renderer([([f["vertex"]], None, np.zeros(3), np.ones(3), [16, 16, 16])], tf, device=cuda)
    img = r.render(Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens), kind=_lib.VOLUME_RENDER,
                   n_samples=ns).cpu().numpy()
    mx, _ = relative_error(img, f[f"img_{ci}_{ns}"], channels=(0, 1, 2))
    assert mx <= 1e-5


@pytest.mark.parametrize("ci", range(3))
def test_projections_against_reference_images(cuda, ci):
    from yt_gb300.amr_kdtree import vertex_centred

    f = np.load(GOLD / "proj.npz")
    pos, width, res, lens = CAMS[ci]
    cam = Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
    r = Renderer([([f["cell"]], None, np.zeros(3), np.ones(3), [12, 12, 12])], None, device=cuda)
    img = r.render(cam, kind=_lib.PROJECTION).cpu().numpy()
    assert relative_error(img, f[f"proj_{ci}"], channels=(0,))[0] <= 1e-5
    r = Renderer([([vertex_centred(f["cell"])], None, np.zeros(3), np.ones(3), [12, 12, 12])], None, device=cuda)
    img = r.render(cam, kind=_lib.INTERPOLATED_PROJECTION, n_samples=2).cpu().numpy()
    assert relative_error(img, f[f"iproj_{ci}"], channels=(0,))[0] <= 1e-5


def test_amr_against_reference_image(cuda):
    from yt_gb300.amr_kdtree import AMRKDTree

    f = np.load(GOLD / "kd.npz")
    g = np.load(GOLD / "amr_vr.npz")

    class G:
        def __init__(self, gid, level, le, re, data):
            self.id, self.level, self.left_edge, self.right_edge, self.data = gid, level, le, re, data
            self.dims = np.array(data.shape, dtype=np.int64)

        @property
        def dds(self):
            return (self.right_edge - self.left_edge) / self.dims

    grids = [G(int(i), int(lv), a, b, f[f"cell_{int(i)}"])
             for i, lv, a, b in zip(f["gids"], f["levels"], f["gles"], f["gres"])]
    kd = AMRKDTree(grids)
    tf = golden_tf(g["tf_bounds"], g["tf_y"])
    cam = Camera((0.3, 0.6, -1.1), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), (32, 28), lens_type="perspective")
    r = Renderer(kd.bricks(), tf, device=cuda, kdtree=kd)
    img = r.render(cam, kind=_lib.VOLUME_RENDER).cpu().numpy()
    assert relative_error(img, g["image"], channels=(0, 1, 2))[0] <= 1e-5
