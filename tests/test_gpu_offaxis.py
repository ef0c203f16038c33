"""Octree off-axis projection (ytgb_offaxis_cells) against the reference's
own images (tests/golden/offaxis.npz) and the oracle's, through the drop-in
add_cells_to_image_offaxis and the resident CellSplat.

The device sums each cell's subcells per pixel before one float64 atomic
add per pixel and buffer, so its images differ from the reference's by
summation order only: 1e-12 relative, far inside the 1e-5 bound."""
import numpy as np
import pytest
import torch

from oracle import cpu as ocpu
from yt_gb300 import testing
from yt_gb300.camera import Camera
from yt_gb300.offaxis import CellSplat, add_cells_to_image_offaxis, project_cells

from test_oracle_golden import load, offaxis_case

pytestmark = pytest.mark.gpu

TOL = 1e-12


def close(got, ref, tol=TOL):
    scale = np.max(np.abs(ref))
    assert scale > 0
    err = np.max(np.abs(got - ref)) / scale
    assert err <= tol, f"relative error {err:.3e}"


@pytest.mark.parametrize("i", range(5))
def test_offaxis_matches_reference(cuda, i):
    f = load("offaxis.npz")
    X, D, Q, W, rot, nx, ny = offaxis_case(f, i)
    b, bw = np.zeros((nx, ny)), np.zeros((nx, ny))
    add_cells_to_image_offaxis(Xp=X, dXp=D, qty=Q, weight=W, rotation=rot, buffer=b, buffer_weight=bw, Nx=nx,
                               Ny=ny, device=cuda)
    close(b, f[f"b{i}"])
    close(bw, f[f"bw{i}"])


def octree_cells(base, top, seed):
    _, _, _, cells = testing.octree_cells(base_level=base, max_level=top, seed=seed)
    le, re = cells[:, 8:11], cells[:, 11:14]
    return (le + re) / 2, np.ascontiguousarray((re - le)[:, 0]), cells[:, :8].mean(axis=1)


@pytest.mark.parametrize("res,pos,held", [((256, 256), (0.3, 0.8, -1.1), (1, 1)),
                                          ((256, 256), (0.3, 0.8, -1.1), (0, 1)),
                                          ((256, 256), (-0.9, 0.4, 0.2), (1, 0)),
                                          ((200, 330), (1.4, -0.2, 0.6), (1, 1))])
def test_offaxis_matches_oracle(cuda, res, pos, held):
    """A larger octree (levels 3-7): every stamp level from 16 to 64
    subcells per row, accumulated into buffers that already hold values
    (``held``: which of buffer and buffer_weight do; a zero buffer is the
    launch the drop-in makes first, a held one makes it project again)."""
    ctr, dx, q = octree_cells(3, 7, 5)
    rng = np.random.default_rng(3)
    w = rng.uniform(0.5, 2.0, dx.size)
    nx, ny = res
    cam = Camera(pos, (0.5, 0.5, 0.5), (1, 1, 1), res, lens_type="plane-parallel")
    rot = np.ascontiguousarray(cam.inv_mat.T)
    X = np.ascontiguousarray(ctr - 0.5)
    init = rng.uniform(0, 1, (2, nx, ny)) * np.asarray(held, dtype=np.float64)[:, None, None]
    b, bw = init[0].copy(), init[1].copy()
    add_cells_to_image_offaxis(Xp=X, dXp=dx, qty=q, weight=w, rotation=rot, buffer=b, buffer_weight=bw, Nx=nx,
                               Ny=ny, device=cuda)
    rb, rbw = init[0].copy(), init[1].copy()
    ocpu.add_cells_to_image_offaxis(Xp=X, dXp=dx, qty=q, weight=w, rotation=rot, buffer=rb, buffer_weight=rbw,
                                    Nx=nx, Ny=ny)
    close(b, rb)
    close(bw, rbw)


def test_offaxis_resident_repeats_and_flags_bad_cells(cuda):
    """CellSplat renders the same image on every call, and a cell with a
    non-positive or NaN width is skipped and reported in the error word
    while the other cells are still splatted."""
    ctr, dx, q = octree_cells(2, 5, 2)
    X = np.ascontiguousarray(ctr - 0.5)
    cam = Camera((0.2, 0.4, -1.0), (0.5, 0.5, 0.5), (1, 1, 1), (96, 96), lens_type="plane-parallel")
    rot = np.ascontiguousarray(cam.inv_mat.T)
    s = CellSplat(X, dx, q, device=cuda)
    a = s.project(rot, 96, 96)
    b = s.project(rot, 96, 96)
    torch.cuda.synchronize()
    close(a[0].cpu().numpy(), b[0].cpu().numpy(), 1e-14)
    rb, rbw = np.zeros((96, 96)), np.zeros((96, 96))
    ocpu.add_cells_to_image_offaxis(Xp=X, dXp=dx, qty=q, weight=np.ones_like(dx), rotation=rot, buffer=rb,
                                    buffer_weight=rbw, Nx=96, Ny=96)
    close(a[0].cpu().numpy().reshape(96, 96), rb)
    bad = dx.copy()
    bad[[5, 17]] = [0.0, np.nan]
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    sb = CellSplat(X, bad, q, device=cuda)
    sb.dx_max = s.dx_max  # the same stamps as the clean set
    got = sb.project(rot, 96, 96, error=err)
    torch.cuda.synchronize()
    assert int(err.item()) == 4  # YTGB_DEVERR_BAD_CELL
    keep = np.ones(dx.size, bool)
    keep[[5, 17]] = False
    rb2, rbw2 = np.zeros((96, 96)), np.zeros((96, 96))
    ocpu.add_cells_to_image_offaxis(Xp=X[keep], dXp=dx[keep], qty=q[keep], weight=np.ones(keep.sum()),
                                    rotation=rot, buffer=rb2, buffer_weight=rbw2, Nx=96, Ny=96)
    close(got[0].cpu().numpy().reshape(96, 96), rb2)


def test_offaxis_rejects_wide_images(cuda):
    ctr, dx, q = octree_cells(2, 4, 1)
    with pytest.raises(ValueError):
        add_cells_to_image_offaxis(Xp=ctr - 0.5, dXp=dx, qty=q, weight=np.ones_like(dx), rotation=np.eye(3),
                                   buffer=np.zeros((40, 30)), buffer_weight=np.zeros((40, 30)), Nx=40, Ny=30,
                                   device=cuda)


def test_project_cells_driver(cuda):
    """off_axis_projection's octree branch on plain arrays: the image of a
    constant field is the path length through the domain (times wmax /
    sqrt(3) and the stamp normalisation), identical in the quantity and the
    weight channels when both are 1."""
    ctr, dx, _ = octree_cells(2, 5, 2)
    cam = Camera((0.1, 0.3, -1.2), (0.5, 0.5, 0.5), (1, 1, 1), (64, 64), lens_type="plane-parallel")
    img = project_cells(ctr, dx, np.ones_like(dx), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), cam.inv_mat.T, (64, 64),
                        device=cuda)
    assert img.shape == (64, 64, 2)
    close(img[..., 0], img[..., 1], 1e-14)
    assert img[32, 32, 0] > 0 and img[0, 0, 0] >= 0


def test_offaxis_conserves_each_cells_total_at_full_size(cuda):
    """Size-independent property at the benchmark's scale (217k cells of
    levels 5-9, 1024^2): every cell's stamp sums to one, so a cell lying
    inside the image deposits exactly q * dx^3 * Nx * Ny (and w * dx^3 Nx Ny
    into the weight buffer); the image totals equal those sums."""
    _, _, _, cells = testing.octree_cells(base_level=5, max_level=9, seed=0, percentile=85.0)
    le, re = cells[:, 8:11], cells[:, 11:14]
    # half the image width: every rotated cell stays inside the image
    X = np.ascontiguousarray(((le + re) / 2 - 0.5) / 2)
    dx = np.ascontiguousarray((re - le)[:, 0] / 2)
    q = np.ascontiguousarray(cells[:, :8].mean(axis=1))
    w = np.random.default_rng(1).uniform(0.5, 2.0, dx.size)
    n = 1024
    cam = Camera((0.05, 1.1, -0.16), (0.5, 0.5, 0.5), (1, 1, 1), (n, n), lens_type="plane-parallel")
    b, bw = np.zeros((n, n)), np.zeros((n, n))
    add_cells_to_image_offaxis(Xp=X, dXp=dx, qty=q, weight=w, rotation=np.ascontiguousarray(cam.inv_mat.T),
                               buffer=b, buffer_weight=bw, Nx=n, Ny=n, device=cuda)
    want_q = float(np.sum(q * dx ** 3) * n * n)
    want_w = float(np.sum(w * dx ** 3) * n * n)
    assert abs(b.sum() - want_q) <= 1e-10 * want_q
    assert abs(bw.sum() - want_w) <= 1e-10 * want_w
