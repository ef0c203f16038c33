"""The GPU kernels' per-ray walk, compiled for the CPU, against the oracle.

tests/kernel_host/harness.cpp builds yt_gb300/csrc/ytgb_ray.cuh -- the same
source render_kernel executes per ray -- with g++ (no floating-point
contraction), so these cases check the exact traversal (trace hashes), the
float32 sample geometry and the compensated compositing without a GPU.  The
bar is the GPU parity bar: bit-identical traces and visit counts, image
within 1e-5 per-pixel relative error.
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import cpu as ocpu
from yt_gb300 import _lib, testing, workloads
from yt_gb300.amr_kdtree import AMRKDTree, vertex_centred
from yt_gb300.camera import Camera
from yt_gb300.image_samplers import make_view
from yt_gb300.render import relative_error
from yt_gb300.transfer_functions import (ColorTransferFunction, MultiVariateTransferFunction, TransferFunction,
                                         pack)
from yt_gb300.volume import BrickSet, set_light, set_range

ROOT = Path(__file__).resolve().parent.parent
HERE = Path(__file__).resolve().parent / "kernel_host"
KN = {0: "volume_render", 1: "projection", 2: "interpolated_projection", 3: "mip", 4: "light_source"}
TOL = 1e-5


@pytest.fixture(scope="module")
def emu():
    src = HERE / "harness.cpp"
    out = HERE / "_build" / "libytgb_host_walk.so"
    deps = [src, ROOT / "yt_gb300" / "csrc" / "ytgb_ray.cuh", ROOT / "yt_gb300" / "csrc" / "ytgb_vertex.cuh",
            ROOT / "yt_gb300" / "csrc" / "ytgb_octree.cuh",
            ROOT / "include" / "ytgb.h",
            ROOT / "yt_gb300" / "csrc" / "ytgb_internal.h"]
    if not out.exists() or out.stat().st_mtime < max(d.stat().st_mtime for d in deps):
        out.parent.mkdir(exist_ok=True)
        tmp = out.with_suffix(f".{os.getpid()}.tmp")
        cuda_inc = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                        f"-I{ROOT / 'include'}", f"-I{ROOT / 'yt_gb300' / 'csrc'}", f"-I{cuda_inc}", str(src),
                        "-o", str(tmp)], check=True)
        os.replace(tmp, out)
    L = C.CDLL(str(out))
    L.emu_render.argtypes = [C.POINTER(_lib.RenderArgs), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.emu_rays.argtypes = [C.POINTER(_lib.View), C.c_void_p, C.c_void_p]
    return L


def run_emu(L, bricks, cam, order, kind, tf=None, ns=1, zbuffer=None, light=None, with_lo=None):
    """with_lo: the arena's float32 rounding errors (None: for the light
    source, whose gradient uses them; True also takes the float64 range
    decisions of volume rendering and the light source)."""
    lo = (kind == _lib.LIGHT_SOURCE) if with_lo is None else bool(with_lo)
    bs = BrickSet(bricks, device="cpu", with_lo=lo)
    p = cam.sampler_params()
    nx, ny = cam.resolution
    view, ppos, pdir = make_view(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], nx, ny, p["x_vec"],
                                 p["y_vec"], p["width"], p["lens_type"], p["camera_data"])
    order = np.ascontiguousarray(order, dtype=np.int32)
    rects = np.ascontiguousarray(bs.rects(view, order))
    a = _lib.RenderArgs()
    a.kind, a.n_samples, a.n_order, a.view = kind, ns, order.size, view
    if ppos is not None:
        a.view.px_pos, a.view.px_dir = ppos.ctypes.data, pdir.ctypes.data
    a.bricks, a.order, a.rects, a.data = bs.desc.data_ptr(), order.ctypes.data, rects.ctypes.data, bs.data.data_ptr()
    a.bounds = bs.bounds.data_ptr()
    keep = []
    if bs.masks is not None:
        a.masks = bs.masks.data_ptr()
    if tf is not None:
        pk = pack(tf)
        keep.append(pk)
        a.tf, a.tf_tables = pk.header, pk.tables.ctypes.data
    if zbuffer is not None:
        zbuffer = np.ascontiguousarray(zbuffer, dtype=np.float64)
        a.zbuffer = zbuffer.ctypes.data
    if kind == _lib.LIGHT_SOURCE:
        set_light(a, bs, light)
    elif kind == _lib.VOLUME_RENDER:
        set_range(a, bs)
    img = np.zeros((nx, ny, 4))
    a.image = img.ctypes.data
    cnt = np.zeros(4, dtype=np.uint64)
    L.emu_render(C.byref(a), 0, None, None, cnt.ctypes.data)
    h = np.full(nx * ny, _lib.FNV_OFFSET, dtype=np.uint64)
    c = np.zeros(nx * ny, dtype=np.int64)
    L.emu_render(C.byref(a), 1, h.ctypes.data, c.ctypes.data, np.zeros(4, dtype=np.uint64).ctypes.data)
    return img, cnt, h.reshape(nx, ny), c.reshape(nx, ny)


def run_oracle(bricks, cam, order, kind, tf=None, ns=1, zbuffer=None, light=None):
    p = cam.sampler_params()
    ld, lrgba = light if light is not None else ((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0))
    s = ocpu.OracleSampler(KN[kind], p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"], p["x_vec"],
                           p["y_vec"], p["width"], lens_type=p["lens_type"], camera_data=p["camera_data"],
                           zbuffer=zbuffer, n_samples=ns, tf=tf, light_dir=ld, light_rgba=lrgba)
    ob = ocpu.OracleBricks(bricks)
    visits = s.render(ob, order)
    h, c = s.trace(ob, order)
    return p["image"], visits, h, c


def check(L, bricks, cam, order, kind, tf=None, ns=1, channels=(0, 1, 2), zbuffer=None, light=None):
    img, cnt, h, c = run_emu(L, bricks, cam, order, kind, tf, ns, zbuffer, light)
    ref, visits, hr, cr = run_oracle(bricks, cam, order, kind, tf, ns, zbuffer, light)
    mx, rms = relative_error(img, ref, channels=channels)
    assert mx <= TOL, f"max relative error {mx:.3e} (rms {rms:.3e})"
    assert int(cnt[0]) == visits
    if zbuffer is None:
        assert np.array_equal(c, cr) and np.array_equal(h, hr)
    return mx


@pytest.mark.parametrize("pos,lens,width", [((0.5, 0.5, -1.0), "plane-parallel", 1.0),
                                            ((1.3, 0.2, -0.7), "plane-parallel", 1.0),
                                            ((-0.4, 1.1, 1.6), "plane-parallel", 0.8),
                                            ((1.6, 1.4, 1.9), "perspective", 1.5),
                                            ((0.45, 0.55, 0.5), "perspective", 1.5)])
def test_uniform_vr(emu, pos, lens, width):
    w = workloads.uniform_vr(n=24, res=40)
    cam = Camera(pos, (0.5, 0.5, 0.5), width, (40, 36), lens_type=lens)
    check(emu, w.bricks, cam, w.order(cam), _lib.VOLUME_RENDER, tf=w.tf)


@pytest.mark.parametrize("lens", ["perspective", "plane-parallel"])
def test_amr_vr(emu, lens):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=64, lens_type=lens)
    cam = w.views[0].camera if lens == "perspective" else Camera((1.4, -0.3, 1.2), (0.5, 0.5, 0.5), 1.2, 64)
    check(emu, w.bricks, cam, w.order(cam), _lib.VOLUME_RENDER, tf=w.tf)


@pytest.mark.parametrize("kind", [_lib.PROJECTION, _lib.MIP])
@pytest.mark.parametrize("angle", [0.0, 30.0, 57.0])
def test_projection_mip(emu, kind, angle):
    w = workloads.projection_study(n=24, res=40, angles=(angle,), kinds=(kind,))
    check(emu, w.bricks, w.views[0].camera, np.array([0]), kind, channels=(0,))


def test_interpolated_projection(emu):
    grids = testing.amr_blob_grids(root=32, levels=2, patch=8, seed=2)
    kd = AMRKDTree(grids, log_field=False)
    for cam, ns in ((Camera((0.4, 0.5, -1.0), 0.5, 1.5, 40, lens_type="perspective"), 2),
                    (Camera((1.2, 0.3, -0.8), 0.5, 1.0, 40), 3)):
        check(emu, kd.bricks(), cam, kd.viewpoint_order(cam.viewpoint), _lib.INTERPOLATED_PROJECTION, ns=ns,
              channels=(0,))


def test_zbuffer_and_samples(emu):
    w = workloads.uniform_vr(n=20, res=32)
    cam = Camera((0.2, 1.3, -0.8), 0.5, 1.0, 32)
    zb = np.random.default_rng(3).uniform(0.2, 1.5, (32, 32))
    check(emu, w.bricks, cam, w.order(cam), _lib.VOLUME_RENDER, tf=w.tf, ns=4, zbuffer=zb)


def test_grey_opacity_and_multivariate(emu):
    g = testing.blob_grid(20, seed=5)
    v0 = np.log10(vertex_centred(g.data))
    v1 = vertex_centred(np.sqrt(g.data))
    bricks = [([v0, v1], None, np.zeros(3), np.ones(3), np.array([20, 20, 20]))]
    lo, hi = float(np.nanmin(v0)), float(np.nanmax(v0))
    ctf = ColorTransferFunction((lo, hi), nbins=128, grey_opacity=True)
    for loc, wd, rgba in testing.ctf_layers((lo, hi), 3, width=0.02):
        ctf.add_gaussian(loc, wd, list(rgba))
    cam = Camera((1.1, 0.4, -0.9), 0.5, 1.0, 40)
    check(emu, bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf=ctf, channels=(0, 1, 2, 3))
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
    check(emu, bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf=mv)


@pytest.mark.parametrize("res", [(1, 1), (1, 7), (9, 1)])
@pytest.mark.parametrize("lens", ["perspective", "plane-parallel"])
def test_degenerate_images(emu, res, lens):
    """One-pixel rows and columns: the perspective lens's linspace of one
    point is its start (-0.5), the plane-parallel lens's pixel position
    divides by zero as yt's does; walk and image as the oracle's."""
    w = workloads.uniform_vr(n=12, res=8)
    cam = Camera((0.45, 0.55, -1.0), (0.5, 0.5, 0.5), 1.0, res, lens_type=lens)
    img, cnt, h, c = run_emu(emu, w.bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf=w.tf)
    ref, visits, hr, cr = run_oracle(w.bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf=w.tf)
    assert np.array_equal(np.isnan(img), np.isnan(ref))
    assert np.array_equal(c, cr) and np.array_equal(h, hr) and int(cnt[0]) == visits
    ok = ~np.isnan(ref)
    assert np.allclose(img[ok], ref[ok], rtol=1e-5, atol=1e-12)


@pytest.mark.parametrize("kind", [_lib.PROJECTION, _lib.MIP, _lib.INTERPOLATED_PROJECTION])
@pytest.mark.parametrize("nf", [2, 4, 5])
def test_multi_field_projections(emu, kind, nf):
    """Bricks of several fields: the projection samplers write min(nf, 4)
    channels (interpolated projection min(nf, 3)), through the cell loop
    that reads the channel count from the brick (one-field bricks take the
    loop compiled for one channel)."""
    grids = testing.amr_blob_grids(root=16, levels=2, patch=8, seed=4)
    kd = AMRKDTree(grids, log_field=False)
    vertex = kind == _lib.INTERPOLATED_PROJECTION
    bricks = []
    for d, m, le, re, dims in kd.bricks():
        base = d[0] if vertex else d[0][:-1, :-1, :-1].copy()
        bricks.append(([base * (1.0 + 0.25 * k) + k for k in range(nf)], m, le, re, dims))
    cam = Camera((1.2, 0.35, -0.8), 0.5, 1.2, 24, lens_type="perspective")
    order = kd.viewpoint_order(cam.viewpoint)
    chans = tuple(range(min(nf, 3 if vertex else 4)))
    check(emu, bricks, cam, order, kind, channels=chans)


def test_empty_brick_list(emu):
    """No bricks in the order: no walk, the image as it was."""
    w = workloads.uniform_vr(n=8, res=8)
    cam = Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), 1.0, 8)
    img, cnt, h, c = run_emu(emu, w.bricks, cam, np.zeros(0, dtype=np.int32), _lib.VOLUME_RENDER, tf=w.tf)
    assert not img.any() and int(cnt[0]) == 0 and int(cnt[1]) == 0 and not c.any()


def near_bound_case(n=8, seed=3):
    """One brick whose every vertex value lies within 1e-9 of b = 1 + 2^-30,
    the upper bound of the transfer functions below: float32 has no value
    between 1 and 1 + 2^-23, so every stored value is 1.0 and every float32
    sample falls inside the range, while yt's float64 test drops the samples
    at or above b -- about half (field_interpolation_tables.pxd:72-73)."""
    rng = np.random.default_rng(seed)
    b = 1.0 + 2.0 ** -30
    v = b + rng.uniform(-1e-9, 1e-9, (n + 1,) * 3)
    bricks = [([v], None, np.zeros(3), np.ones(3), np.array([n, n, n]))]
    ctf = workloads.color_tf((b - 1.0, b), 4)
    grey = workloads.color_tf((b - 1.0, b), 4)
    grey.grey_opacity = True
    tf = TransferFunction((b - 1.0, b), 64)
    tf.add_gaussian(b - 0.02, 0.01, 1.0)
    mv = MultiVariateTransferFunction()
    mv.add_field_table(tf, 0)
    mv.link_channels(0, [0, 1, 2, 3])
    return bricks, {"ctf": ctf, "grey": grey, "general": mv}


@pytest.mark.parametrize("which,kind,ns", [("ctf", _lib.VOLUME_RENDER, 1), ("ctf", _lib.VOLUME_RENDER, 3),
                                           ("grey", _lib.VOLUME_RENDER, 1), ("grey", _lib.VOLUME_RENDER, 2),
                                           ("general", _lib.VOLUME_RENDER, 1),
                                           ("ctf", _lib.LIGHT_SOURCE, 2)])
def test_range_decisions_near_a_bound(emu, which, kind, ns):
    """With the arena's rounding errors (data_lo) and their scale
    (range_eps) the kernel decides every sample within its float32 error of
    a bound from yt's float64 value, and matches the oracle; without them it
    keeps every sample of this field and misses by far."""
    bricks, tfs = near_bound_case()
    tf = tfs[which]
    cam = Camera((0.3, 0.6, -1.0), 0.5, 1.5, 24, lens_type="perspective")
    order = np.array([0])
    # (the light source with light_rgba 0: this field's gradient is rounding
    # noise, which yt normalises into an arbitrary direction)
    light = ((1.0, 1.0, 1.0), (0.0, 0.0, 0.0, 0.0)) if kind == _lib.LIGHT_SOURCE else None
    ref, visits, *_ = run_oracle(bricks, cam, order, kind, tf, ns, light=light)
    chans = (0, 1, 2)
    img, cnt, *_ = run_emu(emu, bricks, cam, order, kind, tf, ns, light=light, with_lo=True)
    assert relative_error(img, ref, channels=chans)[0] <= TOL and int(cnt[0]) == visits
    if kind == _lib.VOLUME_RENDER:
        f32, *_ = run_emu(emu, bricks, cam, order, kind, tf, ns, with_lo=False)
        assert relative_error(f32, ref, channels=chans)[0] > 1e-2


@pytest.mark.parametrize("ci", range(2))
@pytest.mark.parametrize("ns", [1, 3])
def test_range_decisions_match_yt(emu, ci, ns):
    """Against yt's own images of the near-bound field (near_bound.npz, from
    yt's compiled VolumeRenderSampler): the kernel's walk with the float64
    range decisions within 1e-5, without them far off."""
    from test_oracle_golden import NB_CAMS, GoldenTF

    f = np.load(ROOT / "tests" / "golden" / "near_bound.npz")
    tf = GoldenTF(f["tf_bounds"], f["tf_y"])
    pos, width, res, lens = NB_CAMS[ci]
    cam = Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
    n = f["vertex"].shape[0] - 1
    bricks = [([f["vertex"]], None, np.zeros(3), np.ones(3), np.array([n, n, n]))]
    ref = f[f"img_{ci}_{ns}"]
    img, *_ = run_emu(emu, bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf, ns, with_lo=True)
    assert relative_error(img, ref, channels=(0, 1, 2))[0] <= TOL
    f32, *_ = run_emu(emu, bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf, ns, with_lo=False)
    assert relative_error(f32, ref, channels=(0, 1, 2))[0] > 1e-2


@pytest.mark.parametrize("k", range(3))
def test_amr_cut_bounds_match_yt(emu, k):
    """yt's own AMR renders under transfer functions whose bounds cut through
    the data (amr_cut.npz): the kernel's walk with float64 range decisions
    within 1e-5."""
    from test_oracle_golden import GoldenTF, amr_cut_bricks

    g = np.load(ROOT / "tests" / "golden" / "amr_cut.npz")
    bricks, gcam = amr_cut_bricks()
    cam = Camera((0.3, 0.6, -1.1), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), (32, 28), lens_type="perspective")
    assert np.array_equal(cam.viewpoint, gcam.viewpoint)
    tf = GoldenTF(g[f"tf_bounds_{k}"], g[f"tf_y_{k}"])
    img, *_ = run_emu(emu, bricks, cam, np.arange(len(bricks)), _lib.VOLUME_RENDER, tf, with_lo=True)
    assert relative_error(img, g[f"image_{k}"], channels=(0, 1, 2))[0] <= TOL


def test_range_decision_tolerance_covers_float32_error(emu):
    """The tolerance (range_tol) bounds the float32 sample value's error:
    on AMR bricks with a transfer function whose bounds cut through the
    data, the float32 and the float64-decided renders differ only where a
    sample lies within the tolerance of a bound, and the float64-decided
    one matches the oracle."""
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=48)
    cam = Camera((1.3, -0.4, 1.1), (0.5, 0.5, 0.5), 1.4, 48, lens_type="perspective")
    order = w.order(cam)
    for lo, hi in ((0.1, 0.9), (0.35, 1.25)):
        tf = workloads.color_tf((lo, hi), 6)
        ref, *_ = run_oracle(w.bricks, cam, order, _lib.VOLUME_RENDER, tf)
        img, *_ = run_emu(emu, w.bricks, cam, order, _lib.VOLUME_RENDER, tf, with_lo=True)
        assert relative_error(img, ref, channels=(0, 1, 2))[0] <= TOL


def test_projection_transfer_function_bounds(emu):
    """ProjectionTransferFunction's +-1e60 bounds have no float32 form; yt's
    float64 lookup of its all-zero table gives 0 everywhere, and so must the
    packed table (not NaN)."""
    from yt_gb300.transfer_functions import ProjectionTransferFunction

    w = workloads.uniform_vr(n=16, res=24)
    cam = Camera((1.2, 0.3, -0.8), 0.5, 1.0, 24)
    img, *_ = run_emu(emu, w.bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf=ProjectionTransferFunction())
    assert not np.isnan(img).any()
    check(emu, w.bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf=ProjectionTransferFunction())


def test_masked_cells(emu):
    w = workloads.uniform_vr(n=16, res=32)
    data, _, le, re, dims = w.bricks[0]
    mask = (np.random.default_rng(7).random(tuple(dims)) < 0.7).astype(np.uint8)
    bricks = [(data, mask, le, re, dims)]
    cam = Camera((1.2, 0.3, -0.8), 0.5, 1.0, 32)
    check(emu, bricks, cam, np.array([0]), _lib.VOLUME_RENDER, tf=w.tf)


@pytest.mark.parametrize("pos,res", [((0.5, 0.5, -1.0), (64, 64)), ((1.6, 1.4, 1.9), (48, 40)),
                                     ((0.1, 0.9, 0.3), (1, 7)), ((-2.0, 0.3, 0.2), (33, 1))])
def test_device_perspective_rays_match_numpy(emu, pos, res):
    """YTGB_LENS_PERSPECTIVE regenerates PerspectiveLens's numpy rays
    (lens.py:186-225) bit for bit."""
    cam = Camera(pos, (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), res, lens_type="perspective")
    p = cam.sampler_params()
    v = Camera(pos, (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), res, lens_type="perspective").device_view()
    nx, ny = res
    got_p = np.zeros((nx, ny, 3))
    got_d = np.zeros((nx, ny, 3))
    emu.emu_rays(C.byref(v), got_p.ctypes.data, got_d.ctypes.data)
    assert np.array_equal(got_p, p["vp_pos"])
    assert np.array_equal(got_d, p["vp_dir"])
    # the view's culling parameters equal the per-pixel sampler's
    view, _, _ = make_view(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], nx, ny, p["x_vec"], p["y_vec"],
                           p["width"], p["lens_type"], p["camera_data"])
    assert list(view.camera_data) == list(v.camera_data) and view.extent == v.extent
    assert list(view.center) == list(v.center) and view.pdx == v.pdx and view.pdy == v.pdy


def test_device_perspective_render_matches_oracle(emu):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=48)
    cam = w.views[0].camera
    bs = BrickSet(w.bricks, device="cpu")
    order = np.ascontiguousarray(w.order(cam), dtype=np.int32)
    view = cam.device_view()
    rects = np.ascontiguousarray(bs.rects(view, order))
    a = _lib.RenderArgs()
    a.kind, a.n_samples, a.n_order, a.view = _lib.VOLUME_RENDER, 1, order.size, view
    a.bricks, a.order, a.rects, a.data = bs.desc.data_ptr(), order.ctypes.data, rects.ctypes.data, bs.data.data_ptr()
    a.bounds = bs.bounds.data_ptr()
    pk = pack(w.tf)
    a.tf, a.tf_tables = pk.header, pk.tables.ctypes.data
    img = np.zeros((48, 48, 4))
    a.image = img.ctypes.data
    emu.emu_render(C.byref(a), 0, None, None, np.zeros(4, dtype=np.uint64).ctypes.data)
    ref, *_ = run_oracle(w.bricks, cam, order, _lib.VOLUME_RENDER, w.tf)
    assert relative_error(img, ref)[0] <= TOL


def test_integer_float64_stepping_matches_dadd(emu):
    """step_advance (the walk's tmax += tdelta on bit patterns) equals float64
    addition over 200k random walks of 64 steps, including short mantissas
    that produce exact half-ulp ties."""
    emu.emu_check_step.restype = C.c_longlong
    emu.emu_check_step.argtypes = [C.c_longlong, C.c_int, C.c_ulonglong]
    assert emu.emu_check_step(200_000, 64, 1) == 0


def test_integer_conversions_match(emu):
    emu.emu_check_convert.restype = C.c_longlong
    emu.emu_check_convert.argtypes = [C.c_longlong, C.c_ulonglong]
    assert emu.emu_check_convert(1_000_000, 2) == 0


def test_device_vertex_centring_matches_host(emu):
    """The device brick preparation's vertex value (ytgb_vertex.cuh) equals
    vertex_centred (itself pinned to the reference's ghost_zone_interpolate)
    bit for bit, on grids from 2 cells per axis up, with negative, zero and
    non-finite cells."""
    emu.emu_vertex.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
    rng = np.random.default_rng(4)
    for shape in [(2, 2, 2), (2, 3, 5), (7, 4, 9), (16, 16, 16), (33, 9, 17)]:
        cells = rng.lognormal(0.0, 2.0, shape) * rng.choice([-1.0, 1.0], shape)
        cells.flat[rng.integers(0, cells.size, 3)] = [0.0, np.inf, np.nan]
        cells = np.ascontiguousarray(cells)
        out = np.empty(tuple(n + 1 for n in shape))
        emu.emu_vertex(cells.ctypes.data, *shape, out.ctypes.data)
        want = vertex_centred(cells)
        assert np.array_equal(out.view(np.int64), want.view(np.int64)), shape


LIGHT_CASES = [((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0)), ((-0.3, 0.8, 0.2), (0.9, 0.5, 0.2, 1.0))]


@pytest.mark.parametrize("lens", ["plane-parallel", "perspective"])
@pytest.mark.parametrize("grey", [False, True])
def test_light_source(emu, lens, grey):
    """LightSourceRenderSampler on a uniform blob brick and the AMR bricks:
    the float32 sampler with the analytic gradient (low parts included)
    within 1e-5 of the float64 oracle, the walk bit for bit."""
    w = workloads.uniform_vr(n=20, res=32)
    lo, hi = w.tf.x_bounds if hasattr(w.tf, "x_bounds") else (None, None)
    tf = w.tf
    tf.grey_opacity = grey
    cam = Camera((1.2, 0.35, -0.8), 0.5, 1.2 if lens == "perspective" else 1.0, 32, lens_type=lens)
    for light in LIGHT_CASES:
        for ns in (1, 3):
            check(emu, w.bricks, cam, np.array([0]), _lib.LIGHT_SOURCE, tf=tf, ns=ns, light=light)
    tf.grey_opacity = False


def test_light_source_amr(emu):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=40)
    cam = w.views[0].camera
    check(emu, w.bricks, cam, w.order(cam), _lib.LIGHT_SOURCE, tf=w.tf, light=LIGHT_CASES[1])


def run_octree_both(L, kind, cam, tf=None, ns=1, seed=2, light=None, rays=None, float_edges=True):
    """The octree path on the CPU harness and on the oracle, same inputs
    (``rays``: per-pixel (positions, directions) replacing the camera's)."""
    from yt_gb300.octree import ONODE_DTYPE, Octree

    depth, ipos, lvl, cells = testing.octree_cells(base_level=2, max_level=5, seed=seed)
    oc = Octree(np.zeros(3), np.ones(3), depth)
    oc.add_nodes(ipos, lvl, np.arange(ipos.shape[0], dtype=np.int32))
    nodes = oc.nodes()
    verts = np.ascontiguousarray(cells[:, :8].astype(np.float32))
    le, re = cells[:, 8:11], cells[:, 11:14]
    edges = np.ascontiguousarray(np.concatenate([le, re, 1 / (re - le)], axis=1))
    o = _lib.OctreeArgs()
    o.nodes, o.verts, o.edges = nodes.ctypes.data, verts.ctypes.data, edges.ctypes.data
    if float_edges:
        leh = le.astype(np.float32)
        edges_f = np.zeros((cells.shape[0], 12), dtype=np.float32)
        edges_f[:, 0:3] = leh
        edges_f[:, 3:6] = (le - leh.astype(np.float64)).astype(np.float32)
        edges_f[:, 6:9] = (1 / (re - le)).astype(np.float32)
        o.edges_f = edges_f.ctypes.data
    o.n_nodes, o.n_cells, o.depth = nodes.size, cells.shape[0], depth
    for i in range(3):
        o.dle[i], o.dre[i] = 0.0, 1.0
    p = cam.sampler_params()
    nx, ny = cam.resolution
    if rays is not None:
        p["vp_pos"], p["vp_dir"] = rays
    view, ppos, pdir = make_view(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], nx, ny, p["x_vec"],
                                 p["y_vec"], p["width"], p["lens_type"], p["camera_data"])
    a = _lib.RenderArgs()
    a.kind, a.n_samples, a.view = kind, ns, view
    a.view.px_pos, a.view.px_dir = ppos.ctypes.data, pdir.ctypes.data
    a.data = verts.ctypes.data
    keep = []
    if tf is not None:
        pk = pack(tf)
        keep.append(pk)
        a.tf, a.tf_tables = pk.header, pk.tables.ctypes.data
    if kind == _lib.LIGHT_SOURCE:
        from yt_gb300.volume import normalised_light

        ld, rgba = light
        ld = normalised_light(ld)
        for i in range(3):
            a.light_dir[i] = float(ld[i])
        for i in range(4):
            a.light_rgba[i] = float(rgba[i])
    img = np.zeros((nx, ny, 4))
    a.image = img.ctypes.data
    cnt = np.zeros(4, dtype=np.uint64)
    L.emu_octree.argtypes = [C.POINTER(_lib.RenderArgs), C.POINTER(_lib.OctreeArgs), C.c_int, C.c_void_p,
                             C.c_void_p, C.c_void_p]
    assert L.emu_octree(C.byref(a), C.byref(o), 0, None, None, cnt.ctypes.data) == 0
    h = np.full(nx * ny, _lib.FNV_OFFSET, dtype=np.uint64)
    c = np.zeros(nx * ny, dtype=np.int64)
    assert L.emu_octree(C.byref(a), C.byref(o), 1, h.ctypes.data, c.ctypes.data,
                        np.zeros(4, dtype=np.uint64).ctypes.data) == 0
    # oracle
    ld, lrgba = light if light is not None else ((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0))
    ref = np.zeros((nx, ny, 4))
    s = ocpu.OracleSampler(KN[kind], p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], ref, p["x_vec"],
                           p["y_vec"], p["width"], lens_type=p["lens_type"], camera_data=p["camera_data"],
                           n_samples=ns, tf=tf, light_dir=ld, light_rgba=lrgba)
    oo = ocpu.OracleOctree(depth, np.zeros(3), np.ones(3), ipos, lvl)
    visits = ocpu.render_octree(s, cells, oo)
    hr, cr = ocpu.trace_octree(s, cells, oo)
    return img, cnt, h.reshape(nx, ny), c.reshape(nx, ny), ref, visits, hr, cr, cells


@pytest.mark.parametrize("float_edges", [True, False])
@pytest.mark.parametrize("kind", [_lib.VOLUME_RENDER, _lib.PROJECTION, _lib.INTERPOLATED_PROJECTION, _lib.MIP,
                                  _lib.LIGHT_SOURCE])
def test_octree_path(emu, kind, float_edges):
    """cast_through_octree: traversal (cell keys, enter/exit t bits) bit for
    bit against the oracle (itself pinned to the compiled reference), images
    within 1e-5, for every sampler."""
    cam = Camera((0.3, 1.45, -0.9), (0.5, 0.5, 0.5), (1.3, 1.3, 1.3), (26, 22), lens_type="perspective")
    tf = None
    if kind in (_lib.VOLUME_RENDER, _lib.LIGHT_SOURCE):
        depth, ipos, lvl, cells = testing.octree_cells(base_level=2, max_level=5, seed=2)
        vmin, vmax = float(cells[:, :8].min()), float(cells[:, :8].max())
        tf = ColorTransferFunction((vmin, vmax), nbins=64)
        for loc, wd, rgba in testing.ctf_layers((vmin, vmax), 4):
            tf.add_gaussian(loc, wd, list(rgba))
    light = ((-0.3, 0.8, 0.2), (0.9, 0.5, 0.2, 1.0)) if kind == _lib.LIGHT_SOURCE else None
    for ns in ((1, 2) if kind in (_lib.VOLUME_RENDER, _lib.INTERPOLATED_PROJECTION) else (1,)):
        img, cnt, h, c, ref, visits, hr, cr, _ = run_octree_both(emu, kind, cam, tf, ns, light=light,
                                                                 float_edges=float_edges)
        assert np.array_equal(c, cr) and np.array_equal(h, hr)
        assert int(cnt[0]) == visits and visits > 0
        mx, rms = relative_error(img, ref, channels=(0, 1, 2) if tf is not None else (0,))
        assert mx <= TOL, f"max relative error {mx:.3e} (rms {rms:.3e})"


@pytest.mark.parametrize("kind", [_lib.PROJECTION, _lib.MIP])
def test_octree_axis_rays(emu, kind):
    """Rays with zero direction components (infinite slab t, NaN midpoints)
    traverse bit for bit as the reference's do."""
    cam = Camera((0.3, 1.45, -0.9), (0.5, 0.5, 0.5), (1.3, 1.3, 1.3), (24, 20), lens_type="perspective")
    img, cnt, h, c, ref, visits, hr, cr, _ = run_octree_both(emu, kind, cam, rays=testing.axis_rays(24, 20))
    assert np.array_equal(c, cr) and np.array_equal(h, hr)
    assert int(cnt[0]) == visits and visits > 0
    mx, rms = relative_error(img, ref, channels=(0,))
    assert mx <= TOL, f"max relative error {mx:.3e} (rms {rms:.3e})"
