"""The known answers of tests/test_known_answers.py on the GPU path:
axis-aligned projection (column sums) and MIP (column maxima, exact), a
constant field's projection (path lengths) and a uniform field's volume
rendering (the closed-form recurrence)."""
import numpy as np
import pytest
import torch

from yt_gb300 import _lib
from yt_gb300.camera import Camera
from yt_gb300.render import Renderer

from test_known_answers import N, axis_camera, expected_axis, field, ray_origins

pytestmark = pytest.mark.gpu


def gpu_render(cells_or_verts, kind, cam, tf=None, dims=N):
    r = Renderer([([cells_or_verts], None, np.zeros(3), np.ones(3), np.array([dims] * 3))], tf, device="cuda")
    img = r.render(cam, kind=kind)
    r.check()
    return img.cpu().numpy()


def test_axis_projection_and_mip(cuda):
    cells = field()
    cam = axis_camera()
    img = gpu_render(cells, _lib.PROJECTION, cam)
    want = expected_axis(cells.astype(np.float32).astype(np.float64), lambda col: col.sum() / N, cam)
    assert np.allclose(img[..., 0], want, rtol=1e-6, atol=0)
    img = gpu_render(cells, _lib.MIP, cam)
    want = expected_axis(cells.astype(np.float32).astype(np.float64), np.max, cam)
    assert np.array_equal(img[..., 0], want)


@pytest.mark.parametrize("pos", [(1.3, 0.2, -0.7), (-0.4, 1.1, 1.6)])
def test_constant_field_projection(cuda, pos):
    from test_known_answers import render

    cam = Camera(pos, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 20, lens_type="plane-parallel")
    cells = np.full((N, N, N), 2.5)
    img = gpu_render(cells, _lib.PROJECTION, cam)
    ref = render("projection", cells, cam)
    assert np.allclose(img[..., 0], ref[..., 0], rtol=1e-6, atol=1e-7)


def test_uniform_field_recurrence(cuda):
    from yt_gb300.transfer_functions import ColorTransferFunction

    v = 0.3
    tf = ColorTransferFunction((0.0, 1.0), nbins=64)
    tf.add_gaussian(v, 0.05, [0.9, 0.6, 0.3, 0.8])
    cam = axis_camera()
    img = gpu_render(np.full((N + 1,) * 3, v), _lib.VOLUME_RENDER, cam, tf=tf)
    ys = [np.interp(v, np.linspace(0, 1, 64), t.y) for t in tf.funcs]
    o = ray_origins(cam)
    hit = (o[..., 0] < 1) & (o[..., 1] < 1)
    for ch in range(3):
        want = 1 - (1 - ys[ch] * ys[3] / N) ** N
        assert np.allclose(img[hit, ch], want, rtol=1e-6), ch
        assert np.all(img[~hit, ch] == 0)
