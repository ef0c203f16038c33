"""GPU parity: the CUDA samplers against the C oracle on the same inputs.

Bar: the visited-cell trace (brick, cell index, enter/exit t bits) is
bit-identical to the oracle's walk_volume; images are within 1e-5 relative
error per pixel (max|g-o| / max(|o|, 1e-6 max|o|)) of the oracle's float64
render; cell-visit counters equal the oracle's.
"""
import numpy as np
import pytest

from oracle import cpu as ocpu
from yt_gb300 import _lib, testing, workloads
from yt_gb300.camera import Camera
from yt_gb300.render import Renderer, relative_error
from yt_gb300.transfer_functions import pack

pytestmark = pytest.mark.gpu

TOL = 1e-5
KIND_NAME = {_lib.VOLUME_RENDER: "volume_render", _lib.PROJECTION: "projection",
             _lib.INTERPOLATED_PROJECTION: "interpolated_projection", _lib.MIP: "mip",
             _lib.LIGHT_SOURCE: "light_source"}


def oracle_render(bricks, cam, order, kind, tf=None, n_samples=1, zbuffer=None, image=None, light=None):
    p = cam.sampler_params()
    img = p["image"] if image is None else image.copy()
    ld, lrgba = light if light is not None else ((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0))
    s = ocpu.OracleSampler(KIND_NAME[kind], p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], img,
                           p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                           camera_data=p["camera_data"], zbuffer=zbuffer, n_samples=n_samples, tf=tf,
                           light_dir=ld, light_rgba=lrgba)
    ob = ocpu.OracleBricks(bricks)
    visits = s.render(ob, order)
    h, c = s.trace(ob, order)
    return img, visits, h, c


def check_view(r: Renderer, bricks, cam, kind, tf=None, n_samples=1, channels=(0, 1, 2), zbuffer=None,
               light=None):
    import torch

    order = r.order(cam)
    zb = None if zbuffer is None else torch.from_numpy(zbuffer).to(r.device)
    r.counters.zero_()
    img = r.render(cam, kind=kind, n_samples=n_samples, order=order, zbuffer=zb, light=light).cpu().numpy()
    r.check()
    ref, visits, h_ref, c_ref = oracle_render(bricks, cam, order, kind, tf=tf, n_samples=n_samples, zbuffer=zbuffer,
                                              light=light)
    mx, rms = relative_error(img, ref, channels=channels)
    assert mx <= TOL, f"max relative error {mx:.3e} (rms {rms:.3e})"
    assert int(r.counters[0].item()) == visits
    if zbuffer is None:
        h, c = r.trace(cam, order)
        assert np.array_equal(c, c_ref)
        assert np.array_equal(h, h_ref)
    return img, ref, mx


@pytest.mark.parametrize("pos", [(0.5, 0.5, -1.0), (1.3, 0.2, -0.7), (-0.4, 1.1, 1.6)])
def test_uniform_vr_plane_parallel(cuda, pos):
    w = workloads.uniform_vr(n=32, res=64)
    cam = Camera(pos, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), (64, 60), lens_type="plane-parallel")
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    check_view(r, w.bricks, cam, _lib.VOLUME_RENDER, tf=w.tf)


@pytest.mark.parametrize("pos", [(0.5, 0.5, -1.0), (1.6, 1.4, 1.9)])
def test_uniform_vr_perspective(cuda, pos):
    w = workloads.uniform_vr(n=32, res=64)
    cam = Camera(pos, (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), (56, 64), lens_type="perspective")
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    check_view(r, w.bricks, cam, _lib.VOLUME_RENDER, tf=w.tf)


def test_amr_vr_perspective(cuda):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=96)
    assert w.kdtree.num_bricks > 50
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    check_view(r, w.bricks, w.views[0].camera, _lib.VOLUME_RENDER, tf=w.tf)


def test_amr_vr_plane_parallel_oblique(cuda):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=96, lens_type="plane-parallel")
    cam = Camera((1.4, -0.3, 1.2), (0.5, 0.5, 0.5), (1.2, 1.2, 1.2), 80, lens_type="plane-parallel")
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    check_view(r, w.bricks, cam, _lib.VOLUME_RENDER, tf=w.tf)


@pytest.mark.parametrize("kind", [_lib.PROJECTION, _lib.MIP])
@pytest.mark.parametrize("angle", [0.0, 30.0, 57.0])
def test_projection_and_mip(cuda, kind, angle):
    w = workloads.projection_study(n=48, res=80, angles=(angle,), kinds=(kind,))
    r = Renderer(w.bricks, None, device=cuda)
    check_view(r, w.bricks, w.views[0].camera, kind, channels=(0,))


def test_interpolated_projection_multi_sample(cuda):
    """Projections integrate the linear (positive) field, as yt's projection
    transfer function expects (transfer_functions.py:921-961)."""
    from yt_gb300.amr_kdtree import AMRKDTree

    kd = AMRKDTree([testing.blob_grid(24, seed=0)], log_field=False)
    cam = Camera((1.2, 0.3, -0.8), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 40, lens_type="plane-parallel")
    r = Renderer(kd.bricks(), None, device=cuda, kdtree=kd)
    check_view(r, kd.bricks(), cam, _lib.INTERPOLATED_PROJECTION, n_samples=3, channels=(0,))
    grids = testing.amr_blob_grids(root=32, levels=2, patch=8, seed=2)
    kd = AMRKDTree(grids, log_field=False)
    cam = Camera((0.4, 0.5, -1.0), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), 48, lens_type="perspective")
    r = Renderer(kd.bricks(), None, device=cuda, kdtree=kd)
    check_view(r, kd.bricks(), cam, _lib.INTERPOLATED_PROJECTION, n_samples=2, channels=(0,))


def test_vr_multi_sample_and_zbuffer(cuda):
    w = workloads.uniform_vr(n=24, res=40)
    cam = Camera((0.2, 1.3, -0.8), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 40, lens_type="plane-parallel")
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    zb = np.random.default_rng(3).uniform(0.2, 1.5, (40, 40))
    check_view(r, w.bricks, cam, _lib.VOLUME_RENDER, tf=w.tf, n_samples=4, zbuffer=zb)


def test_grey_opacity_and_weighted_tables(cuda):
    from yt_gb300.transfer_functions import ColorTransferFunction, MultiVariateTransferFunction, TransferFunction

    g = testing.blob_grid(20, seed=5)
    from yt_gb300.amr_kdtree import vertex_centred

    v0 = np.log10(vertex_centred(g.data))
    v1 = vertex_centred(np.sqrt(g.data))
    bricks = [([v0, v1], None, np.zeros(3), np.ones(3), np.array([20, 20, 20]))]
    lo, hi = float(np.nanmin(v0)), float(np.nanmax(v0))
    # grey opacity colour TF
    ctf = ColorTransferFunction((lo, hi), nbins=128, grey_opacity=True)
    for loc, wdt, rgba in testing.ctf_layers((lo, hi), 3, width=0.02):
        ctf.add_gaussian(loc, wdt, list(rgba))
    cam = Camera((1.1, 0.4, -0.9), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 48, lens_type="plane-parallel")
    r = Renderer(bricks, ctf, device=cuda)
    check_view(r, bricks, cam, _lib.VOLUME_RENDER, tf=ctf, channels=(0, 1, 2, 3))
    # multivariate TF
    mv = MultiVariateTransferFunction()
    t0 = TransferFunction((lo, hi), 64)
    t0.add_gaussian(0.5 * (lo + hi), 0.05, 1.0)
    # a second table on field 0 weighted by the positive linear field 1 and
    # by table 0 (emission from one table, weighted by density and another
    # table).  Weighting by a signed field instead would amplify the float32
    # storage error of the data near its zero crossings.
    t1 = TransferFunction((lo, hi), 200)
    t1.add_gaussian(0.7 * lo + 0.3 * hi, 0.05, 0.8)
    mv.add_field_table(t0, 0)
    mv.add_field_table(t1, 0, weight_field_id=1, weight_table_id=0)
    mv.link_channels(1, [0, 1, 2])
    r2 = Renderer(bricks, mv, device=cuda)
    check_view(r2, bricks, cam, _lib.VOLUME_RENDER, tf=mv)


def test_drop_in_sampler_api(cuda):
    """VolumeRenderSampler driven exactly as KDTreeVolumeSource.render drives
    yt's: construct from the camera's sampler params, call per brick in kd
    order, read aimage."""
    from yt_gb300.image_samplers import VolumeRenderSampler

    w = workloads.amr_vr(root=32, levels=2, patch=8, res=64)
    cam = w.views[0].camera
    p = cam.sampler_params()
    s = VolumeRenderSampler(np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"], p["bounds"],
                            p["image"], p["x_vec"], p["y_vec"], p["width"], "KDTree", w.tf, 1,
                            lens_type=p["lens_type"], camera_data=p["camera_data"],
                            zbuffer=np.ones(p["image"].shape[:2]))
    for pg in w.kdtree.traverse(cam.viewpoint):
        s(pg, num_threads=0)
    img = s.aimage
    assert img is p["image"]
    ref, visits, _, _ = oracle_render(w.bricks, cam, w.order(cam), _lib.VOLUME_RENDER, tf=w.tf)
    mx, _ = relative_error(img, ref, channels=(0, 1, 2))
    assert mx <= TOL
    assert int(s.last_counters[0]) == visits


LIGHTS = [((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0)), ((-0.3, 0.8, 0.2), (0.9, 0.5, 0.2, 1.0))]


@pytest.mark.parametrize("lens", ["plane-parallel", "perspective"])
@pytest.mark.parametrize("with_lo", [False, True])
def test_light_source(cuda, lens, with_lo):
    """LightSourceRenderSampler: uniform brick (grey and colour opacity, two
    lights, 1 and 3 samples) and the AMR bricks (NaN vertices from log10 of
    extrapolated non-positive values included: NaN pixels coincide)."""
    from yt_gb300.volume import BrickSet

    w = workloads.uniform_vr(n=24, res=40)
    cam = Camera((1.2, 0.35, -0.8), (0.5, 0.5, 0.5), 1.2 if lens == "perspective" else 1.0, 40, lens_type=lens)
    r = Renderer(BrickSet(w.bricks, device=cuda, with_lo=with_lo), w.tf, device=cuda, kdtree=w.kdtree)
    for grey in (False, True):
        w.tf.grey_opacity = grey
        r.packed = pack(w.tf)
        for light in LIGHTS:
            for ns in (1, 3):
                check_view(r, w.bricks, cam, _lib.LIGHT_SOURCE, tf=w.tf, n_samples=ns, light=light)
    w.tf.grey_opacity = False
    a = workloads.amr_vr(root=32, levels=2, patch=8, res=48)
    ra = Renderer(BrickSet(a.bricks, device=cuda, with_lo=with_lo), a.tf, device=cuda, kdtree=a.kdtree)
    check_view(ra, a.bricks, a.views[0].camera, _lib.LIGHT_SOURCE, tf=a.tf, light=LIGHTS[1])


def test_light_source_drop_in(cuda):
    """The LightSourceRenderSampler class driven like yt drives its sampler."""
    from yt_gb300.image_samplers import LightSourceRenderSampler
    from yt_gb300.partitioned_grid import PartitionedGrid

    w = workloads.amr_vr(root=32, levels=2, patch=8, res=32)
    cam = w.views[0].camera
    p = cam.sampler_params()
    order = w.order(cam)
    s = LightSourceRenderSampler(np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"], p["bounds"],
                                 p["image"], p["x_vec"], p["y_vec"], p["width"], "KDTree", w.tf, 2,
                                 light_dir=np.array([0.2, -1.0, 0.5]), light_rgba=np.array([1.0, 0.8, 0.6, 1.0]),
                                 lens_type=p["lens_type"], camera_data=p["camera_data"])
    for k in order:
        s(PartitionedGrid(0, *w.bricks[k]), num_threads=0)
    img = s.aimage
    ref, *_ = oracle_render(w.bricks, cam, order, _lib.LIGHT_SOURCE, tf=w.tf, n_samples=2,
                            light=((0.2, -1.0, 0.5), (1.0, 0.8, 0.6, 1.0)))
    assert relative_error(img, ref, channels=(0, 1, 2))[0] <= TOL


@pytest.mark.parametrize("res", [(1, 1), (1, 7), (9, 1)])
@pytest.mark.parametrize("lens", ["perspective", "plane-parallel"])
def test_degenerate_images(cuda, res, lens):
    """One-pixel rows and columns (the perspective lens's per-view linspace
    step is 0 there, the plane-parallel lens divides by zero as yt does):
    walk, visit count and image as the oracle's, NaN pixels included."""
    w = workloads.uniform_vr(n=12, res=8)
    cam = Camera((0.45, 0.55, -1.0), (0.5, 0.5, 0.5), 1.0, res, lens_type=lens)
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    order = r.order(cam)
    r.counters.zero_()
    img = r.render(cam, order=order).cpu().numpy()
    r.check()
    ref, visits, h_ref, c_ref = oracle_render(w.bricks, cam, order, _lib.VOLUME_RENDER, tf=w.tf)
    assert np.array_equal(np.isnan(img), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.allclose(img[ok], ref[ok], rtol=TOL, atol=1e-12)
    assert int(r.counters[0].item()) == visits
    h, c = r.trace(cam, order)
    assert np.array_equal(c, c_ref) and np.array_equal(h, h_ref)


def test_empty_brick_list(cuda):
    """An empty order renders nothing: the image is left as it was."""
    import torch

    w = workloads.uniform_vr(n=8, res=8)
    cam = Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), 1.0, 8)
    r = Renderer(w.bricks, w.tf, device=cuda)
    start = torch.full((8, 8, 4), 0.25, dtype=torch.float64, device=cuda)
    img = r.render(cam, order=np.zeros(0, dtype=np.int32), image=start.clone())
    r.check()
    assert torch.equal(img, start)
