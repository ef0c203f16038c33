"""Multi-view batches: every view of a persistent batched launch (and of its
CUDA-graph replay) equals the same view rendered alone, bit for bit, and the
oracle within 1e-5."""
import numpy as np
import pytest
import torch

from oracle import cpu as ocpu
from yt_gb300 import _lib, testing, workloads
from yt_gb300.amr_kdtree import AMRKDTree
from yt_gb300.batch import Batch, Job
from yt_gb300.camera import Camera
from yt_gb300.render import Renderer, relative_error

pytestmark = pytest.mark.gpu


def cams(n, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for k, p in enumerate(testing.fibonacci_sphere(n, radius=1.4)):
        res = (int(rng.choice([24, 40, 64])), int(rng.choice([32, 48])))
        lens = "perspective" if k % 3 else "plane-parallel"
        out.append(Camera(p, (0.5, 0.5, 0.5), 1.5 if lens == "perspective" else 1.1, res, lens_type=lens))
    return out


def same_bits(a, b):
    """Bit-for-bit equality (NaN-safe, unlike torch.equal)."""
    return a.shape == b.shape and torch.equal(a.view(torch.int64), b.view(torch.int64))


def mv_tf(lo, hi):
    """A general (non-ColorTransferFunction) table set: two tables on field
    0, the second weighted by field 1 and by table 0."""
    from yt_gb300.transfer_functions import MultiVariateTransferFunction, TransferFunction

    mv = MultiVariateTransferFunction()
    t0 = TransferFunction((lo, hi), 64)
    t0.add_gaussian(0.5 * (lo + hi), 0.05 * (hi - lo), 1.0)
    t1 = TransferFunction((lo, hi), 200)
    t1.add_gaussian(0.7 * lo + 0.3 * hi, 0.05 * (hi - lo), 0.8)
    mv.add_field_table(t0, 0)
    mv.add_field_table(t1, 0, weight_field_id=1, weight_table_id=0)
    mv.link_channels(1, [0, 1, 2])
    return mv


@pytest.mark.parametrize("blocks", [0, 1])
def test_batch_every_sampler_path(cuda, blocks):
    """Each sampler path of the persistent kernel (colour-table and general
    volume rendering, projection, interpolated projection, MIP) against
    render_kernel, with the tiles spread over many blocks or all in one."""
    grids = testing.amr_blob_grids(root=32, levels=2, patch=8, seed=0)
    kd = AMRKDTree(grids, log_field=False)
    bricks = kd.bricks()
    # a second, positive field for the weighted table
    two = [([d[0], np.sqrt(np.abs(d[0]))], m, le, re, dims) for d, m, le, re, dims in bricks]
    lo = float(min(np.min(d[0]) for d, *_ in bricks))
    hi = float(max(np.max(d[0]) for d, *_ in bricks))
    r_mv = Renderer(two, mv_tf(lo, hi), device=cuda, kdtree=kd)
    r_lin = Renderer(bricks, None, device=cuda, kdtree=kd)
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=32)
    r_ctf = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    cases = [(r_ctf, _lib.VOLUME_RENDER, 1), (r_mv, _lib.VOLUME_RENDER, 2), (r_lin, _lib.PROJECTION, 1),
             (r_lin, _lib.INTERPOLATED_PROJECTION, 3), (r_lin, _lib.MIP, 1), (r_ctf, _lib.LIGHT_SOURCE, 2)]
    light = ((-0.3, 0.8, 0.2), (0.9, 0.5, 0.2, 1.0))
    jobs = [Job(r, cam, kind, n_samples=ns, light=light if kind == _lib.LIGHT_SOURCE else None)
            for (r, kind, ns) in cases for cam in cams(4, seed=7)]
    b = Batch(jobs, device=cuda, blocks=blocks)
    assert len(b.groups) == 6
    b.launch()
    torch.cuda.synchronize()
    b.check()
    for j in jobs:
        alone = j.renderer.render(j.camera, kind=j.kind, n_samples=j.n_samples, light=j.light)
        if j.kind != _lib.LIGHT_SOURCE:
            assert not torch.isnan(alone).any()
        assert same_bits(alone, j.image), (j.kind, j.n_samples)


@pytest.mark.parametrize("tile_shape", [0, 1, 2])
def test_batch_equals_single_views(cuda, tile_shape):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=32)
    r_vr = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    kd_lin = AMRKDTree(testing.amr_blob_grids(root=32, levels=2, patch=8, seed=0), log_field=False)
    r_lin = Renderer(kd_lin.bricks(), None, device=cuda, kdtree=kd_lin)
    jobs = []
    for k, cam in enumerate(cams(9)):
        if k % 3 == 2:
            jobs.append(Job(r_lin, cam, _lib.INTERPOLATED_PROJECTION, n_samples=2))
        else:
            jobs.append(Job(r_vr, cam, _lib.VOLUME_RENDER))
    b = Batch(jobs, device=cuda, tile_shape=tile_shape)
    assert len(b.groups) == 2
    b.launch()
    torch.cuda.synchronize()
    b.check()
    for j in jobs:
        alone = j.renderer.render(j.camera, kind=j.kind, n_samples=j.n_samples,
                                  flags=tile_shape << _lib.FLAG_TILE_SHIFT)
        assert same_bits(alone, j.image)
    g = b.capture()
    snap = [im.clone() for im in b.images]
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    for a, s in zip(b.images, snap):
        assert same_bits(a, s)
    # one view against the oracle
    j = jobs[0]
    p = j.camera.sampler_params()
    s = ocpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                           p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                           camera_data=p["camera_data"], tf=w.tf)
    s.render(ocpu.OracleBricks(w.bricks), r_vr.order(j.camera))
    assert relative_error(j.image.cpu().numpy(), p["image"], channels=(0, 1, 2))[0] <= 1e-5


def test_batch_projection_and_mip(cuda):
    w = workloads.projection_study(n=32, res=48, angles=(0.0, 30.0, 57.0))
    r = Renderer(w.bricks, None, device=cuda)
    jobs = [Job(r, v.camera, v.kind) for v in w.views]
    b = Batch(jobs, device=cuda)
    b.launch()
    torch.cuda.synchronize()
    for j in jobs:
        assert same_bits(r.render(j.camera, kind=j.kind), j.image)


def test_batch_rejects_mixed_layouts():
    e = (_lib.BatchEntry * 2)()
    e[0].args.kind = _lib.PROJECTION
    e[1].args.kind = _lib.MIP
    import ctypes as C

    t, s = C.c_int32(), C.c_int32()
    assert _lib.lib().ytgb_batch_plan(e, 2, 0, C.byref(t), C.byref(s)) != 0


def test_batch_views_with_different_tables(cuda):
    """Views of one sampler class that read different transfer functions:
    the plan asks for no shared memory and the batch reads each view's
    tables from global memory; every image equals the view rendered alone
    (which stages its tables in shared memory), bit for bit, and the
    same views under one shared table take the staged path."""
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=32)
    lg = [float(np.nanmin(b[0][0])) for b in w.bricks] + [float(np.nanmax(b[0][0])) for b in w.bricks]
    lo, hi = min(lg), max(lg)
    r_a = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    r_b = Renderer(r_a.bricks, workloads.color_tf((lo + 0.1, hi - 0.1), 5), device=cuda, kdtree=w.kdtree)
    r_c = Renderer(r_a.bricks, workloads.color_tf((lo, hi), 3, nbins=128), device=cuda, kdtree=w.kdtree)
    views = cams(6, seed=5)
    mixed = Batch([Job([r_a, r_b, r_c][k % 3], cam, _lib.VOLUME_RENDER) for k, cam in enumerate(views)],
                  device=cuda)
    assert len(mixed.groups) == 1 and mixed.groups[0].smem == 0
    shared = Batch([Job(r_b, cam, _lib.VOLUME_RENDER) for cam in views], device=cuda)
    assert shared.groups[0].smem > 0
    for b in (mixed, shared):
        b.launch()
        torch.cuda.synchronize()
        b.check()
        for j in b.jobs:
            alone = j.renderer.render(j.camera, kind=j.kind)
            assert float(alone.abs().max()) > 0
            assert same_bits(alone, j.image)
