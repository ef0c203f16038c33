# distutils: language = c++
# cython: language_level=3
"""Visited-cell probe over the reference's ``walk_volume`` -- TEST INFRASTRUCTURE.

Calls yt's compiled ``walk_volume`` (``yt/utilities/lib/grid_traversal.pyx:26-140``)
with a callback that records, per ray, every ``(index[3], enter_t, exit_t)`` the
traversal hands to its sampler.  Used only to pin the oracle's and the GPU
kernel's cell traversal bit for bit against the reference.
"""
cimport numpy as np

import numpy as np

from libc.stdlib cimport free, malloc

from yt.utilities.lib.grid_traversal cimport walk_volume
from yt.utilities.lib.partitioned_grid cimport PartitionedGrid
from yt.utilities.lib.volume_container cimport VolumeContainer


cdef struct Rec:
    np.int64_t n
    np.int64_t cap
    np.int32_t *cells
    np.float64_t *ts


cdef void _record(VolumeContainer *vc, np.float64_t v_pos[3],
                  np.float64_t v_dir[3], np.float64_t enter_t,
                  np.float64_t exit_t, int index[3], void *data) noexcept nogil:
    cdef Rec *r = <Rec *> data
    if r.n < r.cap:
        r.cells[3 * r.n + 0] = index[0]
        r.cells[3 * r.n + 1] = index[1]
        r.cells[3 * r.n + 2] = index[2]
        r.ts[2 * r.n + 0] = enter_t
        r.ts[2 * r.n + 1] = exit_t
    r.n += 1


def trace_rays(PartitionedGrid pg,
               np.float64_t[:, ::1] pos,
               np.float64_t[:, ::1] dirs,
               np.float64_t[::1] max_t,
               int cap):
    """Trace every ray (pos[i], dirs[i], max_t[i]) through brick ``pg``.

    Returns (count int64[n], cells int32[n, cap, 3], ts float64[n, cap, 2]).
    """
    cdef int n = pos.shape[0]
    cdef np.ndarray[np.int64_t, ndim=1] count = np.zeros(n, dtype=np.int64)
    cdef np.ndarray[np.int32_t, ndim=3] cells = np.zeros((n, cap, 3), dtype=np.int32)
    cdef np.ndarray[np.float64_t, ndim=3] ts = np.zeros((n, cap, 2), dtype=np.float64)
    cdef Rec rec
    cdef np.float64_t p[3]
    cdef np.float64_t d[3]
    cdef int i, k
    for i in range(n):
        rec.n = 0
        rec.cap = cap
        rec.cells = <np.int32_t *> &cells[i, 0, 0]
        rec.ts = <np.float64_t *> &ts[i, 0, 0]
        for k in range(3):
            p[k] = pos[i, k]
            d[k] = dirs[i, k]
        walk_volume(pg.container, p, d, _record, <void *> &rec, NULL, max_t[i])
        count[i] = rec.n
    return count, cells, ts
