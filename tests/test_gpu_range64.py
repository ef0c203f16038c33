"""GPU: float64 range decisions near a transfer-function bound.

yt keeps or drops a sample by comparing its float64 value with the table's
bounds (FIT_get_value, field_interpolation_tables.pxd:72-73).  The kernels
sample in float32; where the bricks carry their values' float32 rounding
errors (``BrickSet(with_lo=True)``) they decide every sample whose float32
value lies within its error bound of a bound (or is 0) from yt's float64
value instead.  These tests check the single-view kernel, the persistent
batch kernel and the allocation-free batch entry point against the oracle
on a field built so that float32 decides every sample differently from
float64, and on AMR bricks cut by transfer-function bounds inside the
data's range -- the served form's transfer functions.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from test_gpu_parity import oracle_render
from test_kernel_host import near_bound_case
from yt_gb300 import _lib, workloads
from yt_gb300.batch import Batch, Job
from yt_gb300.camera import Camera
from yt_gb300.render import Renderer, relative_error
from yt_gb300.transfer_functions import pack
from yt_gb300.volume import BrickSet

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def cuda():
    return torch.device("cuda", 0)


@pytest.mark.parametrize("which,kind,ns", [("ctf", _lib.VOLUME_RENDER, 1), ("ctf", _lib.VOLUME_RENDER, 3),
                                           ("general", _lib.VOLUME_RENDER, 1),
                                           ("ctf", _lib.LIGHT_SOURCE, 2)])
def test_near_bound_single_view(cuda, which, kind, ns):
    bricks, tfs = near_bound_case()
    tf = tfs[which]
    cam = Camera((0.3, 0.6, -1.0), 0.5, 1.5, 48, lens_type="perspective")
    light = ((1.0, 1.0, 1.0), (0.0, 0.0, 0.0, 0.0)) if kind == _lib.LIGHT_SOURCE else None
    ref, visits, *_ = oracle_render(bricks, cam, np.array([0]), kind, tf=tf, n_samples=ns, light=light)
    r = Renderer(BrickSet(bricks, device=cuda, with_lo=True), tf, device=cuda)
    assert r.bricks.range_eps > 0
    img = r.render(cam, kind=kind, n_samples=ns, light=light).cpu().numpy()
    r.check()
    assert relative_error(img, ref, channels=(0, 1, 2))[0] <= TOL
    assert int(r.counters[0].item()) == visits
    if kind == _lib.VOLUME_RENDER:
        f32 = Renderer(BrickSet(bricks, device=cuda), tf, device=cuda).render(cam, n_samples=ns).cpu().numpy()
        assert relative_error(f32, ref, channels=(0, 1, 2))[0] > 1e-2


def test_near_bound_batch_and_noalloc(cuda):
    """The batch kernel's float64-decision variant gives the single-view
    kernel's images bit for bit, through ytgb_batch_render and through the
    allocation-free entry point."""
    bricks, tfs = near_bound_case()
    r = Renderer(BrickSet(bricks, device=cuda, with_lo=True), tfs["ctf"], device=cuda)
    cams = [Camera(p, 0.5, 1.5, res, lens_type="perspective")
            for p, res in (((0.3, 0.6, -1.0), 40), ((1.4, 0.2, 1.3), (24, 56)), ((-0.8, 1.2, 0.4), 32))]
    b = Batch([Job(r, c) for c in cams], device=cuda)
    assert [g.variant for g in b.groups] == [_lib.VARIANT_CTF | _lib.VARIANT_RANGE64]
    b.launch()
    torch.cuda.synchronize()
    singles = [r.render(c) for c in cams]
    for a, s in zip(b.images, singles):
        assert torch.equal(a.view(torch.int64), s.view(torch.int64))
    L = _lib.lib()
    g = b.groups[0]
    for im in b.images:
        im.zero_()
    _lib.check(L.ytgb_batch_render_noalloc(g.entries, g.n, g.kind, g.variant, b.tile_shape, g.total_tiles, g.smem,
                                           0, C.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "ytgb_batch_render_noalloc")
    torch.cuda.synchronize()
    for a, s in zip(b.images, singles):
        assert torch.equal(a.view(torch.int64), s.view(torch.int64))


def test_amr_bounds_inside_the_data(cuda):
    """The served form's kind of transfer function -- bounds inside the
    data's range, the brightest layer next to the upper bound -- on the
    AMR bricks: within 1e-5 of the oracle with the float64 decisions."""
    w = workloads.amr_vr(root=64, levels=2, patch=16, res=192)
    r = Renderer(BrickSet(w.bricks, device=cuda, with_lo=True), None, device=cuda, kdtree=w.kdtree)
    rng = np.random.default_rng(11)
    for k in range(4):
        lo, hi = sorted(rng.uniform(-0.3, 1.6, 2))
        tf = workloads.color_tf((lo - 0.2, hi + 0.2), int(rng.integers(3, 9)))
        r.tf, r.packed = tf, pack(tf)
        d = rng.normal(0.0, 1.0, 3)
        cam = Camera(0.5 + 1.3 * d / np.linalg.norm(d), (0.5, 0.5, 0.5), 1.5, 192, lens_type="perspective")
        order = r.order(cam)
        img = r.render(cam, order=order).cpu().numpy()
        r.check()
        ref, *_ = oracle_render(w.bricks, cam, order, _lib.VOLUME_RENDER, tf=tf)
        assert relative_error(img, ref, channels=(0, 1, 2))[0] <= TOL, (k, lo, hi)
