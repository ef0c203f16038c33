"""The small plain configuration and the projection / MIP precision study at
their full sizes, against the oracle.

* One 64^3 blob grid as one brick, plane-parallel view down +z (width 1),
  256^2, 4-layer ColorTransferFunction, 1 sample per cell: every ray's
  visited-cell trace bit-identical to the oracle's walk_volume, equal sample
  counts, image within 1e-5 of the float64 render.
* A 512^3 float32 lognormal random field (P(k) ~ k^-3, seed 1), 2048^2
  plane-parallel: ProjectionSampler and the MIP sampler at 57 degrees (the
  orientation with the most cell visits per ray) traced bit for bit and
  compared with the float64 oracle; the 0 and 30 degree views compared
  image against image, with and without compensated accumulation.  The
  oracle reads the float32 field upcast to float64.
"""
import numpy as np
import pytest

from oracle import cpu as ocpu
from test_gpu_parity import TOL, check_view
from yt_gb300 import _lib, testing, workloads
from yt_gb300.render import Renderer, relative_error

pytestmark = pytest.mark.gpu


def test_uniform_64_full_size(cuda):
    w = workloads.uniform_vr()
    cam = w.views[0].camera
    assert cam.resolution == (256, 256) and tuple(w.bricks[0][4]) == (64, 64, 64)
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    img, ref, mx = check_view(r, w.bricks, cam, _lib.VOLUME_RENDER, tf=w.tf)
    assert ref.max() > 0 and int(r.counters[0].item()) > 4_000_000


@pytest.fixture(scope="module")
def grf():
    field = testing.lognormal_grf(512, seed=1)
    return workloads.projection_study(n=512, res=2048, field=field)


def _view(w, kind, angle):
    for v in w.views:
        a = float(np.rad2deg(np.arctan2(v.camera.unit_vectors[2][1], v.camera.unit_vectors[2][2])))
        if v.kind == kind and abs(a - angle) < 1e-6:
            return v
    raise KeyError((kind, angle))


@pytest.mark.parametrize("kind", [_lib.PROJECTION, _lib.MIP])
def test_grf_512_at_2048_oblique_traced(cuda, grf, kind):
    v = _view(grf, kind, 57.0)
    assert v.camera.resolution == (2048, 2048)
    r = Renderer(grf.bricks, None, device=cuda)
    img, ref, mx = check_view(r, grf.bricks, v.camera, kind, channels=(0,))
    assert int(r.counters[0].item()) > 2_000_000_000


@pytest.mark.parametrize("angle", [0.0, 30.0])
def test_grf_512_at_2048_other_angles(cuda, grf, angle):
    r = Renderer(grf.bricks, None, device=cuda)
    for kind in (_lib.PROJECTION, _lib.MIP):
        v = _view(grf, kind, angle)
        order = r.order(v.camera)
        p = v.camera.sampler_params()
        s = ocpu.OracleSampler("projection" if kind == _lib.PROJECTION else "mip", p["vp_pos"], p["vp_dir"],
                               p["center"], p["bounds"], p["image"], p["x_vec"], p["y_vec"], p["width"],
                               lens_type=p["lens_type"], camera_data=p["camera_data"])
        visits = s.render(ocpu.OracleBricks(grf.bricks), order)
        for flags in (0, _lib.FLAG_NO_COMPENSATION):
            r.counters.zero_()
            img = r.render(v.camera, kind=kind, order=order, flags=flags).cpu().numpy()
            r.check()
            assert int(r.counters[0].item()) == visits
            mx, _ = relative_error(img, p["image"], channels=(0,))
            assert mx <= TOL, (kind, angle, flags, mx)
