"""A pure-Python PartitionedGrid with the public attributes of yt's
(``yt/utilities/lib/partitioned_grid.pyx:23-63``, ``partitioned_grid.pxd:19-23``).

The samplers read only ``my_data``, ``source_mask``, ``LeftEdge`` and
``RightEdge`` (and derive ``dims`` from the mask), so yt's own Cython
``PartitionedGrid`` objects work with them just as well.
"""
from __future__ import annotations

import numpy as np


class PartitionedGrid:
    def __init__(self, parent_grid_id, data, mask, left_edge, right_edge, dims, n_fields=-1):
        self.parent_grid_id = int(parent_grid_id)
        self.LeftEdge = np.asarray(left_edge, dtype=np.float64)
        self.RightEdge = np.asarray(right_edge, dtype=np.float64)
        self.dims = np.asarray(dims, dtype=np.int64)
        if n_fields == -1:
            n_fields = len(data)
        self.n_fields = n_fields
        self.my_data = data
        if mask is None:
            mask = np.ones(tuple(int(d) for d in self.dims), dtype=np.uint8)
        self.source_mask = mask
        # partitioned_grid.pyx:54-55
        self.dds = (self.RightEdge - self.LeftEdge) / self.dims
        self.idds = 1.0 / self.dds
