"""Seeded synthetic datasets for the sampler workloads (the role yt's
``yt/testing.py`` fake datasets play for its own tests).

* :func:`blob_grid`    -- one uniform grid of the Gaussian-blob density field.
* :func:`amr_blob_grids` -- the same field refined by factor 2 in patches
  wherever log10(density) exceeds the level's 90th percentile.
* :func:`lognormal_grf` -- a lognormal Gaussian random field with P(k) ~ k^-3.

Every generator draws from ``numpy.random.default_rng(seed)`` in a fixed
order, so a seed names one dataset.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Grid:
    id: int
    level: int
    left_edge: np.ndarray
    right_edge: np.ndarray
    dims: np.ndarray
    data: np.ndarray = field(repr=False)  # cell-centred float64, shape dims

    @property
    def dds(self):
        return (self.right_edge - self.left_edge) / self.dims


@dataclass
class BlobParams:
    centres: np.ndarray
    sigmas: np.ndarray
    amps: np.ndarray


def blob_params(rng, n_blobs=8) -> BlobParams:
    centres = rng.uniform(0.2, 0.8, size=(n_blobs, 3))
    sigmas = rng.uniform(0.03, 0.1, size=n_blobs)
    amps = rng.lognormal(mean=0.0, sigma=1.0, size=n_blobs)
    return BlobParams(centres, sigmas, amps)


def blob_density(p: BlobParams, le, re, dims) -> np.ndarray:
    """1 + sum_k A_k exp(-|x - c_k|^2 / (2 sigma_k^2)) at the cell centres of
    the box [le, re] with ``dims`` cells."""
    dims = [int(d) for d in dims]
    axes = [le[i] + (np.arange(dims[i]) + 0.5) * (re[i] - le[i]) / dims[i] for i in range(3)]
    x, y, z = axes
    rho = np.ones(dims, dtype=np.float64)
    for c, s, a in zip(p.centres, p.sigmas, p.amps):
        gx = np.exp(-((x - c[0]) ** 2) / (2 * s * s))
        gy = np.exp(-((y - c[1]) ** 2) / (2 * s * s))
        gz = np.exp(-((z - c[2]) ** 2) / (2 * s * s))
        rho += a * gx[:, None, None] * gy[None, :, None] * gz[None, None, :]
    return rho


def blob_grid(n=64, seed=0) -> Grid:
    """A single uniform n^3 grid on [0,1]^3: blob field times lognormal noise
    exp(0.1 N(0,1))."""
    rng = np.random.default_rng(seed)
    p = blob_params(rng)
    le, re = np.zeros(3), np.ones(3)
    dims = np.array([n, n, n], dtype=np.int64)
    rho = blob_density(p, le, re, dims) * np.exp(0.1 * rng.standard_normal(tuple(dims)))
    return Grid(0, 0, le, re, dims, rho)


def amr_blob_grids(root=128, levels=3, seed=0, patch=16, block_choices=None, percentile=90.0, stat="mean"):
    """Root grid plus ``levels`` of factor-2 refinement.

    At level l-1 every grid is cut into blocks of b^3 cells (b = patch // 2,
    or drawn per parent grid from ``block_choices``); a block whose mean
    (``stat="mean"``) or maximum log10(density) exceeds the 90th percentile of
    all level-(l-1) cells becomes a level-l grid of (2b)^3 cells over the
    block's extent.  Finer
    data is the same analytic field at the finer cell centres times fresh
    noise drawn in grid order."""
    rng = np.random.default_rng(seed)
    p = blob_params(rng)
    le, re = np.zeros(3), np.ones(3)
    dims = np.array([root] * 3, dtype=np.int64)
    rho = blob_density(p, le, re, dims) * np.exp(0.1 * rng.standard_normal(tuple(dims)))
    grids = [Grid(0, 0, le, re, dims, rho)]
    parents = grids
    for lvl in range(1, levels + 1):
        thresh = np.percentile(np.concatenate([np.log10(g.data).ravel() for g in parents]), percentile)
        children = []
        for g in parents:
            if block_choices is None:
                b = patch // 2
            else:
                opts = [c for c in block_choices if all(int(d) % c == 0 for d in g.dims)]
                b = int(rng.choice(opts))
            lg = np.log10(g.data)
            nb = [int(d) // b for d in g.dims]
            blk6 = lg.reshape(nb[0], b, nb[1], b, nb[2], b)
            blk = blk6.mean(axis=(1, 3, 5)) if stat == "mean" else blk6.max(axis=(1, 3, 5))
            dds = g.dds
            for i, j, k in zip(*np.nonzero(blk > thresh)):
                cle = g.left_edge + np.array([i, j, k]) * b * dds
                cre = cle + b * dds
                cd = np.array([2 * b] * 3, dtype=np.int64)
                children.append((cle, cre, cd))
        if not children:
            break
        new = []
        for cle, cre, cd in children:
            data = blob_density(p, cle, cre, cd) * np.exp(0.1 * rng.standard_normal(tuple(cd)))
            new.append(Grid(len(grids) + len(new), lvl, cle, cre, cd, data))
        grids += new
        parents = new
    return grids


def lognormal_grf(n=512, seed=1, slope=-3.0, dtype=np.float32) -> np.ndarray:
    """exp(g) for a unit-variance Gaussian random field g with P(k) ~ k^slope
    (k = 0 mode removed), from default_rng(seed) white noise."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n, n, n))
    fk = np.fft.rfftn(white)
    kx = np.fft.fftfreq(n)[:, None, None]
    ky = np.fft.fftfreq(n)[None, :, None]
    kz = np.fft.rfftfreq(n)[None, None, :]
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    amp = np.zeros_like(k)
    nz = k > 0
    amp[nz] = k[nz] ** (slope / 2.0)
    fk *= amp
    g = np.fft.irfftn(fk, s=(n, n, n), axes=(0, 1, 2))
    g -= g.mean()
    g /= g.std()
    return np.exp(g).astype(dtype)


def fibonacci_sphere(n, radius=1.5, centre=(0.5, 0.5, 0.5)):
    """n points on a sphere by the Fibonacci lattice."""
    i = np.arange(n) + 0.5
    phi = np.arccos(1.0 - 2.0 * i / n)
    theta = np.pi * (1.0 + 5.0 ** 0.5) * i
    pts = np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], axis=1)
    return np.asarray(centre) + radius * pts


def ctf_layers(x_bounds, n_layers, width=0.01, colormap=None):
    """(location, width, rgba) layers at the positions ColorTransferFunction.
    add_layers uses (transfer_functions.py:874-893): mi = b0 + d/(10N),
    ma = b1 - d/(10N), alpha = logspace(-3, 0, N)."""
    from .transfer_functions import builtin_colormap

    cmap = colormap or builtin_colormap
    b0, b1 = float(x_bounds[0]), float(x_bounds[1])
    dist = b1 - b0
    mi = b0 + dist / (10.0 * n_layers)
    ma = b1 - dist / (10.0 * n_layers)
    alphas = np.logspace(-3, 0, n_layers)
    out = []
    for v, a in zip(np.mgrid[mi: ma: n_layers * 1j], alphas):
        rel = (v - b0) / dist
        r, g, b, _ = cmap(rel)
        out.append((float(v), float(width), (r, g, b, float(a))))
    return out


def blob_point(p: BlobParams, xyz: np.ndarray) -> np.ndarray:
    """The blob field 1 + sum_k A_k exp(-|x - c_k|^2 / (2 sigma_k^2)) at
    points (..., 3)."""
    rho = np.ones(xyz.shape[:-1], dtype=np.float64)
    for c, s, a in zip(p.centres, p.sigmas, p.amps):
        r2 = ((xyz - c) ** 2).sum(axis=-1)
        rho += a * np.exp(-r2 / (2 * s * s))
    return rho


def octree_cells(base_level=3, max_level=6, seed=0, percentile=70.0, log_field=True):
    """An octree dataset on [0,1]^3 in the form yt's octree volume source
    gives its sampler (render_source.py:667-680, octree_raytracing.py:19-41):
    leaf cells from level ``base_level`` down to ``max_level``, a cell refined
    where the blob field at its centre exceeds the ``percentile`` of its
    level.  Returns (depth, ipos (n,3) int32, lvl (n,) int32, cells (n,14)
    float64: the 8 corner values in (i,j,k) C order, left edge, right edge).
    ``ipos = floor(centre * 2^depth)`` as the reference computes it."""
    rng = np.random.default_rng(seed)
    p = blob_params(rng)
    depth = max_level
    n0 = 1 << base_level
    idx = np.stack(np.meshgrid(*[np.arange(n0)] * 3, indexing="ij"), -1).reshape(-1, 3)
    level = base_level
    leaves = []
    while True:
        dx = 1.0 / (1 << level)
        centres = (idx + 0.5) * dx
        val = blob_point(p, centres)
        if level < max_level:
            refine = val > np.percentile(val, percentile)
        else:
            refine = np.zeros(val.size, dtype=bool)
        leaves.append((idx[~refine], level))
        if not refine.any():
            break
        kids = (2 * idx[refine])[:, None, :] + np.stack(np.meshgrid(*[np.arange(2)] * 3, indexing="ij"),
                                                       -1).reshape(1, 8, 3)
        idx = kids.reshape(-1, 3)
        level += 1
    ipos, lvl, cells = [], [], []
    for ix, lv in leaves:
        dx = 1.0 / (1 << lv)
        le = ix * dx
        re = le + dx
        corner = np.stack(np.meshgrid(*[np.arange(2)] * 3, indexing="ij"), -1).reshape(8, 3)
        pts = le[:, None, :] + corner[None, :, :] * dx
        v = blob_point(p, pts)
        if log_field:
            v = np.log10(v)
        centre = (ix + 0.5) * dx
        ipos.append(np.floor(centre * (1 << depth)).astype(np.int32))
        lvl.append(np.full(ix.shape[0], lv, dtype=np.int32))
        cells.append(np.concatenate([v, le, re], axis=1))
    return (depth, np.concatenate(ipos), np.concatenate(lvl),
            np.ascontiguousarray(np.concatenate(cells), dtype=np.float64))


def axis_rays(nx, ny, seed=5):
    """Per-pixel rays ((nx, ny, 3) positions and directions) whose directions
    have zero components (axis-aligned and in-plane), some starting exactly
    on cell faces of [0, 1]^3: their slab t are infinite and their slab
    midpoints NaN."""
    rng = np.random.default_rng(seed)
    dirs = np.array([(0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 0, -1), (-1, 0, 0), (0, 0.6, 0.8), (0.8, 0, -0.6),
                     (0.6, -0.8, 0), (0.3, 0.5, 0.8)], dtype=np.float64)
    d = dirs[rng.integers(0, len(dirs), size=(nx, ny))]
    pos = rng.choice(np.arange(1, 16) / 16.0, size=(nx, ny, 3))
    pos = pos - 1.5 * d + rng.normal(0, 1e-3, size=(nx, ny, 3)) * (rng.random((nx, ny, 1)) < 0.3)
    return np.ascontiguousarray(pos), np.ascontiguousarray(d)
