"""Bricks gathered by the device from the caller's host arrays
(ytgb_gather_fields, on GPUs that read pageable host memory) against the
host pack into pinned memory: the same float32 arena and low parts bit for
bit, and the same drop-in sampler images."""
import os

import numpy as np
import pytest
import torch

from yt_gb300 import workloads
from yt_gb300.volume import BrickSet, device_reads_host

pytestmark = pytest.mark.gpu


def fields(bs, lo=False):
    """Each brick field's values in the arena (without the padding)."""
    arena = (bs.data_lo if lo else bs.data).cpu().numpy()
    d = bs.desc_host
    out = []
    for k in range(bs.n):
        for f in range(int(d["n_fields"][k])):
            o = int(d["data_offset"][k] + f * d["field_stride"][k])
            out.append(arena[o: o + int(bs.verts[k])])
    return np.concatenate(out)


def odd_bricks(seed=4):
    """Bricks with 1-3 fields of vertex data: views and transposes (not
    C-contiguous), float32 input, NaN, infinities and values beyond float32."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(40):
        dims = rng.integers(2, 9, 3)
        shape = tuple(int(v) + 1 for v in dims)
        data = []
        for f in range(int(rng.integers(1, 4))):
            a = rng.normal(0, 1, shape) * 10.0 ** rng.integers(-3, 4)
            if k % 5 == 1:
                a = np.ascontiguousarray(a.transpose(2, 1, 0)).transpose(2, 1, 0)  # F-order view
            if k % 7 == 2:
                a = a.astype(np.float32)
            if k % 6 == 3:
                flat = a.reshape(-1)
                flat[:4] = [np.nan, np.inf, -np.inf, 1e300]
            data.append(a)
        le = rng.uniform(0, 0.5, 3)
        out.append((data, np.ones(tuple(int(v) for v in dims), np.uint8), le, le + 0.5, dims))
    return out


@pytest.mark.parametrize("with_lo", [False, True])
def test_direct_gather_matches_host_pack(cuda, with_lo):
    if not device_reads_host(cuda):
        pytest.skip("the device does not read pageable host memory")
    bricks = odd_bricks()
    a = BrickSet(bricks, device=cuda, with_lo=with_lo, direct=False)
    b = BrickSet(bricks, device=cuda, with_lo=with_lo, direct=True)
    assert b.direct and not a.direct
    assert np.array_equal(a.desc.cpu().numpy(), b.desc.cpu().numpy())
    for lo in ((False, True) if with_lo else (False,)):
        x, y = fields(a, lo), fields(b, lo)
        # NaN payloads differ between host and device conversions
        nan = np.isnan(x)
        assert np.array_equal(nan, np.isnan(y)) and (lo or nan.any())
        assert np.array_equal(x[~nan].view(np.int32), y[~nan].view(np.int32))


def test_direct_sampler_matches_host_pack(cuda):
    """The drop-in VolumeRenderSampler with device gather and the render
    written straight into the caller's host image, against the host pack
    and staged download: identical images."""
    if not device_reads_host(cuda):
        pytest.skip("the device does not read pageable host memory")
    from yt_gb300.image_samplers import VolumeRenderSampler

    w = workloads.amr_vr(root=32, levels=2, patch=8, res=64)
    cam = w.views[0].camera
    imgs = []
    for host_pack in ("1", "0"):
        os.environ["YTGB_HOST_PACK"] = host_pack
        try:
            p = cam.sampler_params()
            s = VolumeRenderSampler(np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"],
                                    p["bounds"], p["image"], p["x_vec"], p["y_vec"], p["width"], "KDTree", w.tf, 1,
                                    lens_type=p["lens_type"], camera_data=p["camera_data"])
            for pg in w.kdtree.traverse(cam.viewpoint):
                s(pg, num_threads=0)
            imgs.append(s.aimage.copy())
        finally:
            os.environ.pop("YTGB_HOST_PACK", None)
    assert np.abs(imgs[0]).max() > 0
    assert np.array_equal(imgs[0].view(np.int64), imgs[1].view(np.int64))


@pytest.mark.parametrize("case", ["image", "zbuffer", "zbuffer-readonly", "both", "fortran", "fortran-zero"])
@pytest.mark.parametrize("host_pack", ["0", "1"])
def test_sampler_reads_inputs_that_are_not_default(cuda, case, host_pack):
    """An image that already holds values (accumulation) or a zbuffer below
    1 is read by the render: in place where the device reads host memory,
    else uploaded for a second launch (the first assumed a zero image and
    no zbuffer).  A Fortran-ordered image goes through a C-ordered copy.
    A read-only zbuffer is read where it lies.  Each matches the oracle's
    image and sample count."""
    from test_gpu_parity import oracle_render
    from yt_gb300 import _lib
    from yt_gb300.image_samplers import VolumeRenderSampler
    from yt_gb300.render import relative_error

    w = workloads.amr_vr(root=32, levels=2, patch=8, res=48)
    cam = w.views[0].camera
    p = cam.sampler_params()
    rng = np.random.default_rng(9)
    nx, ny = p["image"].shape[:2]
    init = np.zeros((nx, ny, 4))
    if case in ("image", "both", "fortran"):
        init = rng.uniform(0.0, 0.5, (nx, ny, 4))
    zb = np.ones((nx, ny))
    if case in ("zbuffer", "zbuffer-readonly", "both"):
        zb = rng.uniform(0.2, 1.0, (nx, ny))
    zb.flags.writeable = case != "zbuffer-readonly"
    img = np.asfortranarray(init) if case.startswith("fortran") else init.copy()
    os.environ["YTGB_HOST_PACK"] = host_pack
    s = VolumeRenderSampler(np.atleast_3d(p["vp_pos"]), np.atleast_3d(p["vp_dir"]), p["center"], p["bounds"], img,
                            p["x_vec"], p["y_vec"], p["width"], "KDTree", w.tf, 1, lens_type=p["lens_type"],
                            camera_data=p["camera_data"], zbuffer=zb)
    try:
        for pg in w.kdtree.traverse(cam.viewpoint):
            s(pg, num_threads=0)
        out = s.aimage
    finally:
        os.environ.pop("YTGB_HOST_PACK", None)
    assert out is img
    ref, visits, _, _ = oracle_render(w.bricks, cam, w.order(cam), _lib.VOLUME_RENDER, tf=w.tf,
                                      zbuffer=None if case in ("image", "fortran") else zb, image=init)
    assert relative_error(out, ref, channels=(0, 1, 2))[0] <= 1e-5
    assert int(s.last_counters[0]) == visits


def test_direct_masks_match_host_pack(cuda):
    """Masks with cells switched off: the device gather marks the same bricks
    (mask_offset) and copies the same bytes as the host check and pack, and
    both render the same image bit for bit."""
    if not device_reads_host(cuda):
        pytest.skip("the device does not read pageable host memory")
    from yt_gb300.render import Renderer

    w = workloads.amr_vr(root=32, levels=2, patch=8, res=48)
    rng = np.random.default_rng(2)
    bricks = []
    for k, (data, mask, le, re, dims) in enumerate(w.bricks):
        shape = tuple(int(d) for d in dims)
        m = np.ones(shape, np.uint8) if k % 3 else (rng.random(shape) < 0.8).astype(np.uint8)
        if k % 4 == 1:
            # a view starting off a 16-byte boundary
            raw = np.empty(m.size + 7, np.uint8)
            v = raw[k % 7 + 1: k % 7 + 1 + m.size].reshape(shape)
            v[...] = m
            m = v
        bricks.append((data, m, le, re, dims))
    a = BrickSet(bricks, device=cuda, direct=False)
    b = BrickSet(bricks, device=cuda, direct=True)
    da = a.desc.cpu().numpy().view(a.desc_host.dtype)
    db = b.desc.cpu().numpy().view(b.desc_host.dtype)
    # the host path keeps every mask once one is not all ones; the device
    # marks only the bricks whose mask is not: the same cells are sampled
    ma, mb = a.masks.cpu().numpy(), b.masks.cpu().numpy()
    assert (db["mask_offset"] >= 0).sum() > 0
    for oa, ob, c in zip(da["mask_offset"], db["mask_offset"], a.cells):
        if ob >= 0:
            assert oa == ob and np.array_equal(ma[oa: oa + c], mb[ob: ob + c]) and (mb[ob: ob + c] != 1).any()
        elif oa >= 0:
            assert (ma[oa: oa + c] == 1).all()
    cam = w.views[0].camera
    ia = Renderer(a, w.tf, device=cuda, kdtree=w.kdtree).render(cam).cpu().numpy()
    ib = Renderer(b, w.tf, device=cuda, kdtree=w.kdtree).render(cam).cpu().numpy()
    assert np.abs(ia).max() > 0 and np.array_equal(ia.view(np.int64), ib.view(np.int64))


def test_render_with_resident_tables(cuda):
    """render(..., tables=render_tables(...)) -- the rectangles and order kept
    on the device across launches -- gives the same image, bit for bit, as
    the per-launch upload, and a table made for another order is
    rejected."""
    from yt_gb300 import _lib
    from yt_gb300.render import Renderer
    from yt_gb300.volume import render, render_tables

    w = workloads.amr_vr(root=32, levels=2, patch=8, res=64)
    cam = w.views[0].camera
    r = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    order = r.order(cam)
    view, ppos, pdir = r.view_args(cam)
    px_pos = torch.from_numpy(ppos).to(cuda) if ppos is not None else None
    px_dir = torch.from_numpy(pdir).to(cuda) if pdir is not None else None
    nx, ny = cam.resolution
    tables = render_tables(r.bricks, view, order)
    imgs = []
    for tab in (None, tables, tables):
        img = torch.zeros((nx, ny, 4), dtype=torch.float64, device=cuda)
        render(r.bricks, view, order, _lib.VOLUME_RENDER, img, tf=r.packed, px_pos=px_pos, px_dir=px_dir,
               tables=tab)
        torch.cuda.synchronize()
        imgs.append(img.cpu().numpy())
    assert np.abs(imgs[0]).max() > 0
    for x in imgs[1:]:
        assert np.array_equal(imgs[0].view(np.int64), x.view(np.int64))
    with pytest.raises(ValueError):
        render(r.bricks, view, order, _lib.VOLUME_RENDER, torch.zeros((nx, ny, 4), dtype=torch.float64, device=cuda),
               tf=r.packed, px_pos=px_pos, px_dir=px_dir, tables=render_tables(r.bricks, view, order[::-1]))
    # a narrower field of view keeps the kd order (same viewpoint) but not
    # the rectangles: the table made for the first view is rejected
    from yt_gb300.camera import Camera

    moved = Camera(cam.position, cam.focus, (1.3, 1.3, 1.5), cam.resolution, lens_type=cam.lens_type)
    assert np.array_equal(r.order(moved), order)
    view2, _, _ = r.view_args(moved)
    with pytest.raises(ValueError, match="another view"):
        render(r.bricks, view2, order, _lib.VOLUME_RENDER,
               torch.zeros((nx, ny, 4), dtype=torch.float64, device=cuda), tf=r.packed, tables=tables)
