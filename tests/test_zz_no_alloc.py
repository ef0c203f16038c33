"""ytgb_batch_render_noalloc against ytgb_batch_render.

The planned batches of a few views (colour-table volume rendering and
interpolated projection) are rendered once through the caller-allocated entry
point, then twice in a row through the static-scratch entry point from the
host copy of the plan; every image matches bit for bit, and the calls leave
the device's free memory unchanged.  Runs last (file name) so that it also
passes after every other GPU test in the same process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from yt_gb300 import _lib, testing, workloads
from yt_gb300.amr_kdtree import AMRKDTree
from yt_gb300.batch import Batch, Job
from yt_gb300.camera import Camera
from yt_gb300.render import Renderer

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    return a.shape == b.shape and torch.equal(a.view(torch.int64), b.view(torch.int64))


def cameras(n, seed=11):
    rng = np.random.default_rng(seed)
    out = []
    for k, p in enumerate(testing.fibonacci_sphere(n, radius=1.4)):
        res = (int(rng.choice([24, 40, 64])), int(rng.choice([32, 48])))
        lens = "perspective" if k % 2 else "plane-parallel"
        out.append(Camera(p, (0.5, 0.5, 0.5), 1.5 if lens == "perspective" else 1.1, res, lens_type=lens))
    return out


def test_noalloc_matches_batch_render(cuda):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=32)
    r_vr = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    kd = AMRKDTree(testing.amr_blob_grids(root=32, levels=2, patch=8, seed=0), log_field=False)
    r_lin = Renderer(kd.bricks(), None, device=cuda, kdtree=kd)
    cams = cameras(6)
    jobs = [Job(r_vr, c, _lib.VOLUME_RENDER) for c in cams] + \
           [Job(r_lin, c, _lib.INTERPOLATED_PROJECTION, n_samples=2) for c in cams]
    b = Batch(jobs, device=cuda)
    b.launch()
    torch.cuda.synchronize()
    b.check()
    ref = [im.clone() for im in b.images]
    assert any(float(r.abs().max()) > 0 for r in ref)

    L = _lib.lib()
    stream = torch.cuda.current_stream(cuda)
    free0 = torch.cuda.mem_get_info(cuda)[0]
    used0 = torch.cuda.memory_allocated(cuda)
    for _ in range(2):
        for im in b.images:
            im.zero_()
        for g in b.groups:
            st = L.ytgb_batch_render_noalloc(g.entries, g.n, g.kind, g.variant, b.tile_shape, g.total_tiles, g.smem, 0,
                                            C.c_void_p(stream.cuda_stream))
            _lib.check(st, "ytgb_batch_render_noalloc")
        torch.cuda.synchronize()
        b.check()
        for got, want in zip(b.images, ref):
            assert same_bits(got, want)
    assert torch.cuda.memory_allocated(cuda) == used0
    assert torch.cuda.mem_get_info(cuda)[0] == free0


def test_noalloc_rejects_oversized_batch():
    e = (_lib.BatchEntry * 1)()
    st = _lib.lib().ytgb_batch_render_noalloc(e, _lib.NOALLOC_MAX_ENTRIES + 1, _lib.PROJECTION, 0, 0, 1, 0, 0, None)
    assert st == _lib.ERR_INVALID
    assert "exceed the static scratch" in _lib.lib().ytgb_last_error().decode()
