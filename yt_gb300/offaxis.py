"""Octree off-axis projection: yt's cell splatting on the device.

For octree datasets seen through a plane-parallel lens, yt's
``off_axis_projection`` (off_axis_projection.py:434-499) does not cast rays:
it splats every cell onto the image with ``add_cells_to_image_offaxis``
(image_utilities.pyx:167-289).  Each cell's projected square is cut into
2^depth x 2^depth subcells weighted by a precomputed *stamp* (the projected
thickness of a unit cube rotated like the camera, one stamp per depth) and
spread bilinearly over the pixels it overlaps.

:func:`offaxis_stamp` computes the stamps on the host exactly as the
reference does (the same float64 operations, vectorised with numpy);
:class:`CellSplat` keeps the cells resident on the device and runs the
``ytgb_offaxis_cells`` launch; :func:`add_cells_to_image_offaxis` is the
drop-in with the reference's keyword signature, and
:func:`project_cells` restates the driver's steps around it (recentring,
periodic wrap, scaling by the image width, the final ``wmax / sqrt(3)``).
"""
from __future__ import annotations

import ctypes as C
import math
import threading

import numpy as np
import torch

from . import _lib


def _integrate_cube(O, u, v, w, nx, ny):
    """direct_integrate_cube (image_utilities.pyx:321-407) over an nx x ny
    grid, vectorised: the depth (zmax - zmin) of the parallelepiped spanned
    by u, v, w from O along z at every pixel centre, and the hit mask.  The
    six faces are tested in the reference's order with its float64
    operations (check_in_parallelogram, :296-318)."""
    Oback = O + u + v + w
    X0 = (np.arange(nx) + 0.5) * (1.0 / nx)
    X1 = (np.arange(ny) + 0.5) * (1.0 / ny)
    front = ((X0 - O[0])[:, None], (X1 - O[1])[None, :])
    back = ((X0 - Oback[0])[:, None], (X1 - Oback[1])[None, :])
    zmin = np.full((nx, ny), np.inf)
    zmax = np.full((nx, ny), -np.inf)
    nhit = np.zeros((nx, ny), dtype=np.int32)
    faces = [(front, v, u, 1, O[2], u[2], v[2]), (front, w, v, 1, O[2], v[2], w[2]),
             (front, w, u, 1, O[2], u[2], w[2]), (back, v, u, -1, Oback[2], u[2], v[2]),
             (back, w, v, -1, Oback[2], v[2], w[2]), (back, w, u, -1, Oback[2], u[2], w[2])]
    for PA, PQ, PR, sign, z0, c0, c1 in faces:
        det = PQ[0] * PR[1] - PQ[1] * PR[0]
        if det == 0:
            continue
        n0 = -(PA[0] * PQ[1] - PA[1] * PQ[0]) / det
        n1 = (PA[0] * PR[1] - PA[1] * PR[0]) / det
        s0, s1 = sign * n0, sign * n1
        within = (0 <= s0) & (s0 <= 1) & (0 <= s1) & (s1 <= 1)
        z = z0 + n0 * c0 + n1 * c1
        zmin = np.where(within & (z < zmin), z, zmin)
        zmax = np.where(within & (z > zmax), z, zmax)
        nhit += within
    if np.any(nhit == 1):
        raise RuntimeError("This should not happen")
    hit = nhit >= 2
    return np.where(hit, zmax - zmin, 0.0), hit


def stamp_extent(dx_max, nx, ny, npix_min=4):
    """(nsx, nsy, max_depth) of the stamps (image_utilities.pyx:220-225)."""
    nsx = max(npix_min, int(math.ceil(2 * dx_max * math.sqrt(3) * nx)))
    nsy = max(npix_min, int(math.ceil(2 * dx_max * math.sqrt(3) * ny)))
    return nsx, nsy, int(math.ceil(math.log2(max(nsx, nsy))))


def offaxis_stamp(rotation, dx_max, nx, ny, npix_min=4, native=True):
    """The stamps and stamp masks of add_cells_to_image_offaxis
    (image_utilities.pyx:204-246): ``(max_depth, nsx, nsy)`` float64 and
    uint8 arrays; level 0 is the single 1, level d >= 1 the integrated cube
    on min(2^d, nsx) x min(2^d, nsy) pixels, normalised to unit sum.  The
    depths come from ``ytgb_offaxis_depths`` (``native``) or from the numpy
    restatement below; both give the same bits."""
    rotation = np.asarray(rotation, dtype=np.float64)
    center = np.array([0.5, 0.5, 0.5])
    w0 = 1 / np.sqrt(3.0)
    a = np.dot(rotation, np.array([1.0, 0, 0]) * w0)
    b = np.dot(rotation, np.array([0, 1.0, 0]) * w0)
    c = np.dot(rotation, np.array([0, 0, 1.0]) * w0)
    o = center - (a + b + c) / 2
    nsx, nsy, max_depth = stamp_extent(dx_max, nx, ny, npix_min)
    stamp = np.zeros((max_depth, nsx, nsy), dtype=float)
    mask = np.zeros((max_depth, nsx, nsy), dtype=np.uint8)
    stamp[0, 0, 0] = 1
    if native:
        # the per-pixel depths natively (the same float64 operations), the
        # normalisation with numpy's own sum as the reference has it
        vec = [np.ascontiguousarray(x, dtype=np.float64) for x in (o, a, b, c)]
        st = _lib.lib().ytgb_offaxis_depths(*[x.ctypes.data for x in vec], nsx, nsy, max_depth, stamp.ctypes.data,
                                            mask.ctypes.data)
        if st != _lib.OK:
            raise RuntimeError(_lib.lib().ytgb_last_error().decode(errors="replace"))
    for depth in range(1, max_depth):
        if not native:
            sx, sy = min(1 << depth, nsx), min(1 << depth, nsy)
            buf, hit = _integrate_cube(o, a, b, c, sx, sy)
            stamp[depth, :sx, :sy] += buf
            mask[depth, :sx, :sy] = hit
        stamp[depth] /= np.sum(stamp[depth])
    return stamp, mask


def _device_stamp(rotation, dx_max, nx, ny, npix_min, device):
    stamp, mask = offaxis_stamp(rotation, dx_max, nx, ny, npix_min)
    # the kernel skips a subcell whose stamp is 0, as the reference skips
    # one whose mask is 0 (a level with no hit divides 0 by 0)
    eff = np.where(mask != 0, stamp, 0.0)
    return torch.from_numpy(np.ascontiguousarray(eff)).to(device), stamp.shape


class CellSplat:
    """Cells resident on the device for repeated off-axis projections.

    ``Xp`` (n, 3) cell centres relative to the image centre and ``dXp`` (n,)
    cell widths, both in units of the image width; ``qty`` and ``weight``
    (n,) as add_cells_to_image_offaxis takes them."""

    def __init__(self, Xp, dXp, qty, weight=None, device="cuda"):
        self.device = torch.device(device)
        Xp = np.ascontiguousarray(Xp, dtype=np.float64).reshape(-1, 3)
        dXp = np.ascontiguousarray(dXp, dtype=np.float64).ravel()
        qty = np.ascontiguousarray(qty, dtype=np.float64).ravel()
        weight = np.ones_like(dXp) if weight is None else np.ascontiguousarray(weight, dtype=np.float64).ravel()
        if not (Xp.shape[0] == dXp.size == qty.size == weight.size):
            raise ValueError("Xp, dXp, qty and weight must describe the same cells")
        self.n = int(dXp.size)
        self.dx_max = float(np.max(dXp))
        self.xp = torch.from_numpy(Xp).to(self.device)
        self.dxp = torch.from_numpy(dXp).to(self.device)
        self.qty = torch.from_numpy(qty).to(self.device)
        self.weight = torch.from_numpy(weight).to(self.device)
        self.upload_bytes = 6 * 8 * self.n
        self._stamps = {}

    def stamp(self, rotation, nx, ny, npix_min=4):
        rotation = np.ascontiguousarray(rotation, dtype=np.float64).reshape(3, 3)
        key = (rotation.tobytes(), nx, ny, npix_min)
        if key not in self._stamps:
            self._stamps[key] = _device_stamp(rotation, self.dx_max, nx, ny, npix_min, self.device)
        return self._stamps[key]

    def project(self, rotation, nx, ny, npix_min=4, out=None, error=None, stream=None):
        """Accumulate every cell into ``out`` = (buffer, buffer_weight), two
        float64 device tensors of nx * ny elements (allocated zeroed when
        None), pixel (i, j) at i * nx + j.  Returns ``out``."""
        nx, ny = int(nx), int(ny)
        if nx > ny:
            raise ValueError("add_cells_to_image_offaxis indexes pixel (i, j) as i * Nx + j, which leaves its "
                             "(Nx, Ny) buffers when Nx > Ny")
        rotation = np.ascontiguousarray(rotation, dtype=np.float64).reshape(3, 3)
        stamp, (max_depth, nsx, nsy) = self.stamp(rotation, nx, ny, npix_min)
        if out is None:
            out = (torch.zeros(nx * ny, dtype=torch.float64, device=self.device),
                   torch.zeros(nx * ny, dtype=torch.float64, device=self.device))
        for t in out:
            if t.dtype != torch.float64 or t.numel() != nx * ny or not t.is_contiguous():
                raise ValueError(f"the buffers must be contiguous float64 tensors of {nx * ny} elements")
        a = _lib.OffaxisArgs()
        a.xp, a.dxp, a.qty, a.weight = (self.xp.data_ptr(), self.dxp.data_ptr(), self.qty.data_ptr(),
                                        self.weight.data_ptr())
        a.stamp = stamp.data_ptr()
        a.buffer, a.buffer_weight = out[0].data_ptr(), out[1].data_ptr()
        for i in range(6):
            a.rot[i] = float(rotation[i // 3, i % 3])
        a.n, a.nx, a.ny, a.nsx, a.nsy, a.max_depth = self.n, nx, ny, nsx, nsy, max_depth
        s = stream or torch.cuda.current_stream(self.device)
        err = None if error is None else error.data_ptr()
        _lib.check(_lib.lib().ytgb_offaxis_cells(C.byref(a), C.c_void_p(err), C.c_void_p(s.cuda_stream)),
                   "ytgb_offaxis_cells")
        return out

    def subcells(self, nx, ny, npix_min=4):
        """The number of stamp subcells the projection visits (jmax * kmax
        summed over the cells, image_utilities.pyx:92-102): the unit of work."""
        nsx, nsy, max_depth = stamp_extent(self.dx_max, nx, ny, npix_min)
        dx = self.dxp.cpu().numpy()
        depth = np.ceil(np.log2(4 * np.sqrt(3) * dx * max(nx, ny))).astype(np.int64)
        depth = np.clip(depth, 1, max_depth - 1)
        return int(np.sum(np.minimum(nsx, 1 << depth) * np.minimum(nsy, 1 << depth)))


def _linear_to_image(lin, nx, ny):
    """The reference's copy-back (image_utilities.pyx:280-285): image[j, k]
    = linear[j * nx + k]."""
    if nx == ny:
        return lin.reshape(nx, ny)
    return np.lib.stride_tricks.as_strided(lin, shape=(nx, ny), strides=(nx * 8, 8))


def add_cells_to_image_offaxis(*, Xp, dXp, qty, weight, rotation, buffer, buffer_weight, Nx, Ny, Npix_min=4,
                               device="cuda"):
    """Drop-in for ``yt.utilities.lib.image_utilities.add_cells_to_image_offaxis``
    (image_utilities.pyx:167-289): adds every cell's splat into ``buffer``
    and ``buffer_weight`` ((Nx, Ny) float64, C order, updated in place)."""
    for b in (buffer, buffer_weight):
        if not isinstance(b, np.ndarray) or b.dtype != np.float64 or b.ndim != 2 or not b.flags.c_contiguous:
            raise ValueError("buffer and buffer_weight must be C-contiguous 2-d float64 arrays")
    dx_max = np.max(dXp)  # raises on no cells, as the reference does
    del dx_max
    nx, ny = int(Nx), int(Ny)
    if buffer.shape != (nx, ny) or buffer_weight.shape != (nx, ny):
        raise ValueError(f"buffer and buffer_weight must have shape ({nx}, {ny})")
    splat = CellSplat(Xp, dXp, qty, weight, device=device)
    if nx != ny:
        # pixel (i, j) lands at i * Nx + j of a linear buffer, read back with
        # the reference's copy-back (Nx < Ny)
        lin, linw = splat.project(rotation, nx, ny, int(Npix_min))
        host = torch.stack([lin, linw]).cpu().numpy()
        buffer += _linear_to_image(host[0], nx, ny)
        buffer_weight += _linear_to_image(host[1], nx, ny)
        return
    # square images: the kernel accumulates straight into device copies of
    # the caller's buffers, which are then copied back.  The projection is
    # launched on buffers of zero bits (the usual new image) while a host
    # thread faults the buffers' pages in and checks that they are zero;
    # otherwise they are uploaded and the projection is run again.
    L = _lib.lib()
    dev = splat.device
    checks = {}

    def host_checks():
        try:
            for b in (buffer, buffer_weight):
                flag = C.c_int32()
                _lib.check(L.ytgb_host_prefault(b.ctypes.data, b.nbytes), "buffer prefault")
                _lib.check(L.ytgb_host_is_uniform(b.ctypes.data, b.size, 0.0, 0, C.byref(flag)), "buffer check")
                checks[id(b)] = bool(flag.value)
        except BaseException as e:  # re-raised on the calling thread
            checks["error"] = e

    outs = tuple(torch.zeros(nx * ny, dtype=torch.float64, device=dev) for _ in range(2))
    checker = threading.Thread(target=host_checks, daemon=True)
    checker.start()
    try:
        splat.project(rotation, nx, ny, int(Npix_min), out=outs)
    finally:
        checker.join()
    if "error" in checks:
        raise checks["error"]
    if not (checks[id(buffer)] and checks[id(buffer_weight)]):
        outs = tuple(torch.zeros(nx * ny, dtype=torch.float64, device=dev) if checks[id(b)] else
                     torch.from_numpy(b).to(dev).reshape(-1) for b in (buffer, buffer_weight))
        splat.project(rotation, nx, ny, int(Npix_min), out=outs)
    torch.from_numpy(buffer).copy_(outs[0].view(nx, ny))
    torch.from_numpy(buffer_weight).copy_(outs[1].view(nx, ny))


def project_cells(positions, dx, qty, center, width, rotation, resolution, weight=None, periodic=(True,) * 3,
                  domain_width=(1.0, 1.0, 1.0), device="cuda"):
    """The octree branch of off_axis_projection (off_axis_projection.py:
    455-497) on plain arrays: cell centres recentred on ``center`` (wrapped
    into [-w/2, w/2] on periodic axes), scaled by the larger image width,
    splatted, and rescaled by ``wmax / sqrt(3)``.  Returns the (nx, ny, 2)
    image of (weighted quantity, weight)."""
    positions = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
    width = np.asarray(width, dtype=np.float64).reshape(-1)
    wmax = float(np.max(width[:2]))
    xyz = np.zeros((positions.shape[0], 3))
    for i in range(3):
        xyz[:, i] = positions[:, i] - center[i]
        if periodic[i]:
            w = float(domain_width[i])
            xyz[:, i] = (xyz[:, i] + w / 2) % w - w / 2
    xyz = xyz / wmax
    dxs = np.asarray(dx, dtype=np.float64) / wmax
    wf = np.ones_like(dxs) if weight is None else np.asarray(weight, dtype=np.float64)
    nx, ny = resolution
    buf, bufw = np.zeros((nx, ny)), np.zeros((nx, ny))
    add_cells_to_image_offaxis(Xp=xyz, dXp=dxs, qty=qty, weight=wf, rotation=rotation, buffer=buf,
                               buffer_weight=bufw, Nx=nx, Ny=ny, device=device)
    buf *= wmax / np.sqrt(3)
    bufw *= wmax / np.sqrt(3)
    return np.stack([buf, bufw], axis=-1)
