"""ctypes binding of the C oracle (``ytoracle.c``) -- TEST INFRASTRUCTURE.

The structures mirror ``yo_vc`` (yt's ``VolumeContainer``,
``yt/utilities/lib/volume_container.pxd:13-33``), ``yo_fit``
(``FieldInterpolationTable``, ``field_interpolation_tables.pxd:27-39``) and
``yo_sampler`` (the fields of ``ImageSampler``,
``yt/utilities/lib/image_samplers.pxd:38-70``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libytoracle.so"

VR, PROJ, IPROJ, MIP, LIGHT = 0, 1, 2, 3, 4
KIND_BY_NAME = {"volume_render": VR, "projection": PROJ, "interpolated_projection": IPROJ, "mip": MIP,
                "light_source": LIGHT}

_dp = C.POINTER(C.c_double)


class YoVC(C.Structure):
    _fields_ = [
        ("left_edge", C.c_double * 3),
        ("right_edge", C.c_double * 3),
        ("dds", C.c_double * 3),
        ("idds", C.c_double * 3),
        ("dims", C.c_int * 3),
        ("n_fields", C.c_int),
        ("data", _dp * 6),
        ("mask", C.POINTER(C.c_uint8)),
    ]


class YoFit(C.Structure):
    _fields_ = [
        ("values", _dp),
        ("bounds", C.c_double * 2),
        ("dbin", C.c_double),
        ("idbin", C.c_double),
        ("d0", _dp),
        ("dy", _dp),
        ("field_id", C.c_int),
        ("weight_field_id", C.c_int),
        ("weight_table_id", C.c_int),
        ("nbins", C.c_int),
    ]


class YoSampler(C.Structure):
    _fields_ = [
        ("nv", C.c_int * 2),
        ("lens", C.c_int),
        ("extent", C.c_int),
        ("kind", C.c_int),
        ("n_samples", C.c_int),
        ("n_fits", C.c_int),
        ("grey_opacity", C.c_int),
        ("field_table_ids", C.c_int * 6),
        ("vp_pos", _dp),
        ("vp_dir", _dp),
        ("center", C.c_double * 3),
        ("bounds", C.c_double * 4),
        ("x_vec", C.c_double * 3),
        ("y_vec", C.c_double * 3),
        ("width", C.c_double * 3),
        ("camera_data", C.c_double * 15),
        ("pdx", C.c_double),
        ("pdy", C.c_double),
        ("image", _dp),
        ("zbuffer", _dp),
        ("fits", YoFit * 6),
        ("light_dir", C.c_double * 3),
        ("light_rgba", C.c_double * 4),
    ]


def build(force: bool = False) -> Path:
    """Compile ``ytoracle.c`` (gcc, OpenMP, no floating-point contraction)."""
    src = HERE / "ytoracle.c"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(
        ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=gnu11",
         str(src), "-o", str(tmp), "-lm"],
        check=True,
    )
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.yo_render.restype = C.c_int64
        _lib.yo_render.argtypes = [C.POINTER(YoSampler), C.POINTER(YoVC), C.POINTER(C.c_int32), C.c_int64, C.c_int]
        _lib.yo_cast_through_kdtree.restype = C.c_int64
        _lib.yo_trace.restype = None
        _lib.yo_trace.argtypes = [C.POINTER(YoSampler), C.POINTER(YoVC), C.POINTER(C.c_int32), C.c_int64,
                                  C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.c_int]
        _lib.yo_fit_init.restype = None
        _lib.yo_fit_init.argtypes = [C.POINTER(YoFit), C.c_int, _dp, C.c_double, C.c_double, C.c_int, C.c_int,
                                     C.c_int, _dp, _dp]
        _lib.yo_padded_rect.restype = None
        _lib.yo_padded_rect.argtypes = [C.POINTER(YoSampler), C.POINTER(YoVC), C.POINTER(C.c_int64)]
        _lib.yo_ghost_zone_interpolate.restype = None
        _lib.yo_ghost_zone_interpolate.argtypes = [C.c_int, _dp, C.POINTER(C.c_int64), _dp, _dp,
                                                   C.POINTER(C.c_int64), _dp]
        _lib.yo_trace_rays.restype = None
        _lib.yo_trace_rays.argtypes = [C.POINTER(YoVC), _dp, _dp, _dp, C.c_int64, C.c_int64,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int32), _dp]
        assert _lib.yo_sizeof_sampler() == C.sizeof(YoSampler), "yo_sampler layout mismatch"
        assert _lib.yo_sizeof_vc() == C.sizeof(YoVC), "yo_vc layout mismatch"
    return _lib


def _ptr(a: np.ndarray, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


class OracleBricks:
    """A list of bricks as ``yo_vc`` records; keeps the numpy arrays alive."""

    def __init__(self, bricks):
        """``bricks``: sequence of (data list of float64 arrays, mask uint8 or
        None, left_edge, right_edge, dims)."""
        self._keep = []
        self.n = len(bricks)
        self.vcs = (YoVC * max(self.n, 1))()
        for k, (data, mask, le, re, dims) in enumerate(bricks):
            vc = self.vcs[k]
            dims = [int(d) for d in dims]
            if mask is None:
                mask = np.ones(dims, dtype=np.uint8)
            mask = np.ascontiguousarray(mask, dtype=np.uint8)
            self._keep.append(mask)
            for i in range(3):
                vc.left_edge[i] = float(le[i])
                vc.right_edge[i] = float(re[i])
                vc.dims[i] = dims[i]
                # partitioned_grid.pyx:54-55
                vc.dds[i] = (vc.right_edge[i] - vc.left_edge[i]) / dims[i]
                vc.idds[i] = 1.0 / vc.dds[i]
            vc.n_fields = len(data)
            for f, d in enumerate(data):
                d = np.ascontiguousarray(d, dtype=np.float64)
                self._keep.append(d)
                vc.data[f] = _ptr(d)
            vc.mask = _ptr(mask, C.c_uint8)


class OracleSampler:
    """The fields of one ``ImageSampler`` (``image_samplers.pyx:59-131``,
    ``:406-446``) as a ``yo_sampler`` record.  ``image`` is rendered into in
    place, like the reference's ``aimage``."""

    def __init__(self, kind, vp_pos, vp_dir, center, bounds, image, x_vec, y_vec, width,
                 lens_type="plane-parallel", camera_data=None, zbuffer=None, n_samples=1, tf=None,
                 light_dir=(1.0, 1.0, 1.0), light_rgba=(1.0, 1.0, 1.0, 1.0)):
        s = YoSampler()
        self._keep = []
        self.image = image
        assert image.dtype == np.float64 and image.flags.c_contiguous and image.shape[2] == 4
        nx, ny = image.shape[:2]
        s.nv[0], s.nv[1] = nx, ny
        s.kind = KIND_BY_NAME[kind] if isinstance(kind, str) else int(kind)
        s.n_samples = int(n_samples)
        vp_pos = np.ascontiguousarray(vp_pos, dtype=np.float64).ravel()
        vp_dir = np.ascontiguousarray(vp_dir, dtype=np.float64).ravel()
        self._keep += [vp_pos, vp_dir]
        if lens_type == "plane-parallel":
            s.lens, s.extent = 0, 0
            assert vp_pos.size == 12 and vp_dir.size == 3
        else:
            s.lens = 1
            s.extent = 1 if (camera_data is not None and lens_type == "perspective") else 2
            assert vp_pos.size == nx * ny * 3 and vp_dir.size == nx * ny * 3
        s.vp_pos = _ptr(vp_pos)
        s.vp_dir = _ptr(vp_dir)
        for i in range(3):
            s.center[i] = float(center[i])
            s.x_vec[i] = float(x_vec[i])
            s.y_vec[i] = float(y_vec[i])
            s.width[i] = float(width[i])
        for i in range(4):
            s.bounds[i] = float(bounds[i])
        s.pdx = (s.bounds[1] - s.bounds[0]) / nx
        s.pdy = (s.bounds[3] - s.bounds[2]) / ny
        if camera_data is not None:
            cd = np.asarray(camera_data, dtype=np.float64).ravel()
            for i in range(15):
                s.camera_data[i] = float(cd[i])
        if zbuffer is None:
            zbuffer = np.ones((nx, ny), dtype=np.float64)
        zbuffer = np.ascontiguousarray(zbuffer, dtype=np.float64)
        self._keep.append(zbuffer)
        s.zbuffer = _ptr(zbuffer)
        s.image = _ptr(image)
        if tf is not None:
            L = lib()
            s.n_fits = int(tf.n_field_tables)
            assert s.n_fits <= 6
            s.grey_opacity = int(getattr(tf, "grey_opacity", 0))
            for i in range(s.n_fits):
                y = np.ascontiguousarray(tf.tables[i].y, dtype=np.float64)
                nb = y.shape[0]
                d0 = np.zeros(nb, dtype=np.float64)
                dy = np.zeros(nb, dtype=np.float64)
                self._keep += [y, d0, dy]
                L.yo_fit_init(C.byref(s.fits[i]), nb, _ptr(y), float(tf.tables[i].x_bounds[0]),
                              float(tf.tables[i].x_bounds[1]), int(tf.field_ids[i]),
                              int(tf.weight_field_ids[i]), int(tf.weight_table_ids[i]), _ptr(d0), _ptr(dy))
            for i in range(6):
                s.field_table_ids[i] = int(tf.field_table_ids[i])
        # LightSourceRenderSampler.__cinit__ (image_samplers.pyx:530-536)
        ld = np.asarray(light_dir, dtype=np.float64)
        ld = ld / np.sqrt(ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2])
        for i in range(3):
            s.light_dir[i] = float(ld[i])
        for i in range(4):
            s.light_rgba[i] = float(light_rgba[i])
        self.s = s

    def render(self, bricks: OracleBricks, order=None, num_threads=0) -> int:
        o = None
        if order is not None:
            order = np.ascontiguousarray(order, dtype=np.int32)
            o = _ptr(order, C.c_int32)
        n = len(order) if order is not None else bricks.n
        return int(lib().yo_render(C.byref(self.s), bricks.vcs, o, n, int(num_threads)))

    def trace(self, bricks: OracleBricks, order=None, num_threads=0):
        nx, ny = self.s.nv[0], self.s.nv[1]
        hashes = np.full(nx * ny, 1469598103934665603, dtype=np.uint64)
        counts = np.zeros(nx * ny, dtype=np.int64)
        o = None
        if order is not None:
            order = np.ascontiguousarray(order, dtype=np.int32)
            o = _ptr(order, C.c_int32)
        n = len(order) if order is not None else bricks.n
        lib().yo_trace(C.byref(self.s), bricks.vcs, o, n, _ptr(hashes, C.c_uint64), _ptr(counts, C.c_int64),
                       int(num_threads))
        return hashes.reshape(nx, ny), counts.reshape(nx, ny)

    def padded_rect(self, bricks: OracleBricks, k: int):
        out = np.zeros(4, dtype=np.int64)
        lib().yo_padded_rect(C.byref(self.s), C.byref(bricks.vcs[k]), _ptr(out, C.c_int64))
        return out


def ghost_zone_vertex_centre(cell: np.ndarray) -> np.ndarray:
    """``grid_patch.py:285-296`` with ``no_ghost=True``: ghost_zone_interpolate
    with rf=1, input_left=[0.5]*3, output_left=[0]*3 onto the (n+1)^3 vertices."""
    cell = np.ascontiguousarray(cell, dtype=np.float64)
    out = np.zeros(tuple(s + 1 for s in cell.shape), dtype=np.float64)
    ish = np.array(cell.shape, dtype=np.int64)
    osh = np.array(out.shape, dtype=np.int64)
    il = np.array([0.5, 0.5, 0.5])
    ol = np.zeros(3)
    lib().yo_ghost_zone_interpolate(1, _ptr(cell), _ptr(ish, C.c_int64), _ptr(il), _ptr(out),
                                    _ptr(osh, C.c_int64), _ptr(ol))
    return out


def trace_rays(brick, pos, dirs, max_t, cap):
    """walk_volume over arbitrary rays through one brick: (counts, cells, ts)."""
    ob = OracleBricks([brick])
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    dirs = np.ascontiguousarray(dirs, dtype=np.float64)
    max_t = np.ascontiguousarray(max_t, dtype=np.float64)
    n = pos.shape[0]
    counts = np.zeros(n, dtype=np.int64)
    cells = np.zeros((n, cap, 3), dtype=np.int32)
    ts = np.zeros((n, cap, 2), dtype=np.float64)
    lib().yo_trace_rays(C.byref(ob.vcs[0]), _ptr(pos), _ptr(dirs), _ptr(max_t), n, cap,
                        _ptr(counts, C.c_int64), _ptr(cells, C.c_int32), _ptr(ts))
    return counts, cells, ts


class OracleOctree:
    """Octree<int> of _octree_raytracing.hpp (yo_octree_build): cells
    inserted at (ipos, lvl) with their keys."""

    def __init__(self, depth, le, re, ipos, lvl, key=None):
        L = lib()
        L.yo_octree_build.restype = C.c_void_p
        L.yo_octree_build.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_int64]
        L.yo_octree_free.argtypes = [C.c_void_p]
        ipos = np.ascontiguousarray(ipos, dtype=np.int32).reshape(-1, 3)
        lvl = np.ascontiguousarray(lvl, dtype=np.int32)
        key = np.arange(ipos.shape[0], dtype=np.int32) if key is None else np.ascontiguousarray(key, dtype=np.int32)
        le = np.ascontiguousarray(le, dtype=np.float64)
        re = np.ascontiguousarray(re, dtype=np.float64)
        self.h = L.yo_octree_build(int(depth), le.ctypes.data, re.ctypes.data, ipos.ctypes.data, lvl.ctypes.data,
                                   key.ctypes.data, ipos.shape[0])

    def __del__(self):
        if getattr(self, "h", None):
            lib().yo_octree_free(self.h)
            self.h = None


def render_octree(sampler: "OracleSampler", cells: np.ndarray, octree: OracleOctree, num_threads=0) -> int:
    """ImageSampler.cast_through_octree (image_samplers.pyx:202-288) into the
    sampler's image; returns the number of cells sampled."""
    L = lib()
    L.yo_cast_through_octree.restype = C.c_int64
    L.yo_cast_through_octree.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    cells = np.ascontiguousarray(cells, dtype=np.float64)
    return int(L.yo_cast_through_octree(C.byref(sampler.s), cells.ctypes.data, octree.h, int(num_threads), None,
                                        None))


def trace_octree(sampler: "OracleSampler", cells: np.ndarray, octree: OracleOctree, num_threads=0):
    """Per pixel: FNV-1a hash over (cell key, enter bits, exit bits) of the
    cells cast_through_octree samples, and their count."""
    L = lib()
    L.yo_cast_through_octree.restype = C.c_int64
    L.yo_cast_through_octree.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    nx, ny = sampler.s.nv[0], sampler.s.nv[1]
    hashes = np.full(nx * ny, 1469598103934665603, dtype=np.uint64)
    counts = np.zeros(nx * ny, dtype=np.int64)
    cells = np.ascontiguousarray(cells, dtype=np.float64)
    L.yo_cast_through_octree(C.byref(sampler.s), cells.ctypes.data, octree.h, int(num_threads),
                             hashes.ctypes.data, counts.ctypes.data)
    return hashes.reshape(nx, ny), counts.reshape(nx, ny)


def _offaxis_lib():
    L = lib()
    L.yo_offaxis_extent.restype = None
    L.yo_offaxis_extent.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.yo_offaxis_stamp.restype = C.c_int
    L.yo_offaxis_stamp.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.yo_add_cells_offaxis.restype = C.c_int
    L.yo_add_cells_offaxis.argtypes = [C.c_void_p] * 4 + [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p] + \
        [C.c_int] * 5 + [C.c_void_p, C.c_void_p]
    return L


def offaxis_stamp(rotation, dx_max, nx, ny, npix_min=4):
    """The stamps and masks of add_cells_to_image_offaxis
    (image_utilities.pyx:204-246), (max_depth, nsx, nsy)."""
    L = _offaxis_lib()
    ext = np.zeros(3, dtype=np.int32)
    L.yo_offaxis_extent(float(dx_max), int(nx), int(ny), int(npix_min), ext.ctypes.data)
    nsx, nsy, max_depth = (int(v) for v in ext)
    rot = np.ascontiguousarray(rotation, dtype=np.float64).reshape(3, 3)
    stamp = np.zeros((max_depth, nsx, nsy))
    mask = np.zeros((max_depth, nsx, nsy), dtype=np.uint8)
    if L.yo_offaxis_stamp(rot.ctypes.data, nsx, nsy, max_depth, stamp.ctypes.data, mask.ctypes.data) != 0:
        raise RuntimeError("This should not happen")
    return stamp, mask


def add_cells_to_image_offaxis(*, Xp, dXp, qty, weight, rotation, buffer, buffer_weight, Nx, Ny, Npix_min=4):
    """add_cells_to_image_offaxis (image_utilities.pyx:167-289), sequential:
    adds into the (Nx, Ny) float64 buffers in place."""
    L = _offaxis_lib()
    Xp = np.ascontiguousarray(Xp, dtype=np.float64).reshape(-1, 3)
    dXp = np.ascontiguousarray(dXp, dtype=np.float64)
    qty = np.ascontiguousarray(qty, dtype=np.float64)
    weight = np.ascontiguousarray(weight, dtype=np.float64)
    rot = np.ascontiguousarray(rotation, dtype=np.float64).reshape(3, 3)
    stamp, mask = offaxis_stamp(rot, np.max(dXp), Nx, Ny, Npix_min)
    max_depth, nsx, nsy = stamp.shape
    assert buffer.flags.c_contiguous and buffer_weight.flags.c_contiguous
    if L.yo_add_cells_offaxis(Xp.ctypes.data, dXp.ctypes.data, qty.ctypes.data, weight.ctypes.data, Xp.shape[0],
                              rot.ctypes.data, stamp.ctypes.data, mask.ctypes.data, nsx, nsy, max_depth, int(Nx),
                              int(Ny), buffer.ctypes.data, buffer_weight.ctypes.data) != 0:
        raise ValueError("Nx > Ny: the reference writes outside its buffers")
