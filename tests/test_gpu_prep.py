"""Device brick preparation (ytgb_vertex_bricks) against the host path
(AMRKDTree.brick: numpy vertex centring, log10, slicing): the same arena,
descriptors and boundary tables, and the same images."""
import ctypes as C

import numpy as np
import pytest
import torch

from yt_gb300 import _lib, testing, workloads
from yt_gb300.amr_kdtree import AMRKDTree
from yt_gb300.render import Renderer
from yt_gb300.volume import BrickSet

pytestmark = pytest.mark.gpu


def ulps(a, b):
    ai = a.view(np.int32).astype(np.int64)
    bi = b.view(np.int32).astype(np.int64)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.abs(ai - bi)
    d[both_nan] = 0
    return d


def valid(bs):
    """The arena's brick values (without the alignment padding between
    fields, which neither path writes)."""
    arena = bs.data.cpu().numpy()
    off = bs.desc_host["data_offset"][: bs.n]
    return np.concatenate([arena[o: o + v] for o, v in zip(off, bs.verts[: bs.n])])


@pytest.mark.parametrize("log_field", [False, True])
def test_device_bricks_match_host(cuda, log_field):
    grids = testing.amr_blob_grids(root=32, levels=2, patch=8, seed=3)
    kd = AMRKDTree(grids, log_field=log_field)
    host = BrickSet(kd.bricks(), device=cuda)
    dev = kd.device_brickset(cuda)
    assert dev.n == host.n
    assert np.array_equal(dev.desc.cpu().numpy(), host.desc.cpu().numpy())
    assert torch.equal(dev.bounds, host.bounds)
    a, b = valid(dev), valid(host)
    assert a.size == sum(int((np.asarray(d[4]) + 1).prod()) for d in kd.bricks())
    d = ulps(a, b)
    if not log_field:
        assert np.array_equal(a.view(np.int32), b.view(np.int32))
    else:
        # device log10 against numpy's: at most one float32 ulp, and rarely
        assert d.max() <= 1 and (d > 0).sum() <= max(1, a.size // 100000)


def test_device_bricks_render_like_host(cuda):
    w = workloads.amr_vr(root=32, levels=2, patch=8, res=48)
    host = Renderer(w.bricks, w.tf, device=cuda, kdtree=w.kdtree)
    dev = Renderer(w.kdtree.device_brickset(cuda), w.tf, device=cuda, kdtree=w.kdtree)
    cam = w.views[0].camera
    a = host.render(cam)
    b = dev.render(cam)
    same = np.array_equal(valid(host.bricks).view(np.int32), valid(dev.bricks).view(np.int32))
    if same:
        assert torch.equal(a.view(torch.int64), b.view(torch.int64))
    else:
        assert float((a - b).abs().max()) <= 1e-6 * float(a.abs().max())


def test_device_bricks_reject_bad_slices(cuda):
    """A brick whose grid index is out of range is skipped on the device and
    reported; nothing outside the arrays is read."""
    grids = testing.amr_blob_grids(root=16, levels=1, patch=8, seed=1)
    kd = AMRKDTree(grids, log_field=False)
    lg, li, dims = kd.leaf_slices()
    bs = BrickSet.on_device(dims, kd.leaf_le, kd.leaf_re, cuda)
    cells = torch.zeros(16 ** 3, dtype=torch.float64, device=cuda)
    goff = torch.zeros(1, dtype=torch.int64, device=cuda)
    meta = torch.tensor([16, 16, 16] + [5] * len(lg) + li.ravel().tolist(), dtype=torch.int32, device=cuda)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    L = _lib.lib()
    s = torch.cuda.current_stream(cuda)
    st = L.ytgb_vertex_bricks(cells.data_ptr(), cells.numel(), goff.data_ptr(), meta.data_ptr(), 1,
                              meta.data_ptr() + 12, meta.data_ptr() + 4 * (3 + len(lg)), bs.desc.data_ptr(),
                              len(lg), 0, 0, bs.data.data_ptr(), bs.data.numel(), err.data_ptr(),
                              C.c_void_p(s.cuda_stream), None)
    assert st == _lib.OK
    assert L.ytgb_check_error(err.data_ptr(), C.c_void_p(s.cuda_stream)) == _lib.ERR_DEVICE


def test_device_bricks_low_parts(cuda):
    """The low parts (each value's float32 rounding error) written by the
    device preparation equal the host split packing's."""
    grids = testing.amr_blob_grids(root=32, levels=2, patch=8, seed=3)
    kd = AMRKDTree(grids, log_field=False)
    host = BrickSet(kd.bricks(), device=cuda, with_lo=True)
    dev = kd.device_brickset(cuda, with_lo=True)

    def valid_lo(bs):
        arena = bs.data_lo.cpu().numpy()
        off = bs.desc_host["data_offset"][: bs.n]
        return np.concatenate([arena[o: o + v] for o, v in zip(off, bs.verts[: bs.n])])

    assert np.array_equal(valid(dev).view(np.int32), valid(host).view(np.int32))
    assert np.array_equal(valid_lo(dev).view(np.int32), valid_lo(host).view(np.int32))
