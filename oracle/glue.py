"""numpy restatement of the Python glue around yt's sampler -- TEST INFRASTRUCTURE.

yt cannot be imported here (unyt, matplotlib and friends are absent), so the
pieces of its scene graph that build the sampler's arguments are restated,
each following the cited reference lines:

* ``orientation``          yt/utilities/orientation.py:59-85
* ``Camera``               yt/visualization/volume_rendering/camera.py:112-150,275-281
* ``plane_parallel_params`` lens.py:45-61,83-121
* ``perspective_params``   lens.py:166-240
* ``TransferFunction`` /
  ``ColorTransferFunction`` /
  ``ProjectionTransferFunction`` transfer_functions.py:34-79,268-360,385-408,921-961
* ``KDTree``               yt/utilities/amr_kdtree/amr_kdtree.py:63-118 driving
                           yt/utilities/lib/amr_kdtools.pyx:201-532,612-823
* ``brick_data``           amr_kdtree.py:325-374 with grid_patch.py:270-296
* ``render``               render_source.py:563-616, scene.py:581-625

The compiled sampler arithmetic itself is in ``ytoracle.c`` (see ``cpu.py``).
"""
from __future__ import annotations

import numpy as np

from . import cpu


# ---------------------------------------------------------------- orientation
def orientation(normal_vector, north_vector=None, steady_north=False):
    """Return (unit_vectors (3,3) [east, north, normal], inv_mat)."""
    normal_vector = np.array(normal_vector, dtype="float64")
    if north_vector is not None:
        north_vector = np.array(north_vector, dtype="float64")
        steady_north = True
    normal_vector /= np.sqrt(np.dot(normal_vector, normal_vector))
    if north_vector is None:
        vecs = np.identity(3)
        t = np.cross(normal_vector, vecs).sum(axis=1)
        ax = t.argmax()
        east_vector = np.cross(vecs[ax, :], normal_vector).ravel()
        north_vector = np.cross(normal_vector, east_vector).ravel()
    else:
        if steady_north or (np.dot(north_vector, normal_vector) != 0.0):
            north_vector = north_vector - np.dot(north_vector, normal_vector) * normal_vector
        east_vector = np.cross(north_vector, normal_vector).ravel()
    north_vector /= np.sqrt(np.dot(north_vector, north_vector))
    east_vector /= np.sqrt(np.dot(east_vector, east_vector))
    unit_vectors = np.array([east_vector, north_vector, normal_vector])
    inv_mat = np.linalg.pinv(unit_vectors)
    return unit_vectors, inv_mat


class Camera:
    """The state of a yt ``Camera`` that the sampler sees."""

    def __init__(self, position, focus, width, resolution, north_vector=None, lens_type="plane-parallel",
                 domain_left=(0.0, 0.0, 0.0), domain_right=(1.0, 1.0, 1.0)):
        self.position = np.array(position, dtype="float64")
        self.focus = np.array(focus, dtype="float64")
        self.width = np.array(width, dtype="float64")
        if np.isscalar(resolution):
            resolution = (resolution, resolution)
        self.resolution = tuple(int(r) for r in resolution)
        self.north_vector = north_vector
        self.lens_type = lens_type
        dl = np.array(domain_left, dtype="float64")
        dr = np.array(domain_right, dtype="float64")
        self.domain_center = (dl + dr) / 2.0
        self.domain_width = dr - dl
        self.unit_vectors, self.inv_mat = orientation(self.focus - self.position, north_vector)
        self._setup_box()

    def _setup_box(self):
        uv, w, c = self.unit_vectors, self.width, self.focus
        self.box_vectors = np.array([uv[0] * w[0], uv[1] * w[1], uv[2] * w[2]])
        self.origin = c - 0.5 * w.dot(uv)
        self.back_center = c - 0.5 * w[2] * uv[2]
        self.front_center = c + 0.5 * w[2] * uv[2]
        if self.lens_type == "plane-parallel":
            self.viewpoint = self.front_center + uv[2] * 1.0e6 * w[2]
        else:
            self.viewpoint = self.front_center

    def sampler_params(self):
        """Camera._get_sampler_params (camera.py:275-281) over the lens's own."""
        if self.lens_type == "plane-parallel":
            p = plane_parallel_params(self)
        else:
            p = perspective_params(self)
        p["width"] = self.width.copy()
        p["camera_data"] = np.vstack((self.position, self.width, self.unit_vectors))
        return p


def plane_parallel_params(cam: Camera):
    nx, ny = cam.resolution
    vp_pos = np.concatenate([cam.inv_mat.ravel("F"), cam.back_center.ravel()])
    return {
        "vp_pos": vp_pos,
        "vp_dir": cam.box_vectors[2],
        "center": cam.back_center,
        "bounds": (-cam.width[0] / 2.0, cam.width[0] / 2.0, -cam.width[1] / 2.0, cam.width[1] / 2.0),
        "x_vec": cam.unit_vectors[0],
        "y_vec": cam.unit_vectors[1],
        "image": np.zeros((nx, ny, 4), dtype="float64"),
        "lens_type": "plane-parallel",
    }


def perspective_params(cam: Camera):
    nx, ny = cam.resolution
    cam.width[1] = cam.width[0] * (ny / nx)
    east_vec, north_vec, normal_vec = cam.unit_vectors
    px = np.linspace(-0.5, 0.5, nx)[np.newaxis, :]
    py = np.linspace(-0.5, 0.5, ny)[np.newaxis, :]
    sample_x = cam.width[0] * np.array(east_vec.reshape(3, 1) * px)
    sample_x = sample_x.transpose()
    sample_y = cam.width[1] * np.array(north_vec.reshape(3, 1) * py)
    sample_y = sample_y.transpose()
    sample_x = np.repeat(sample_x.reshape(nx, 1, 3), ny, axis=1)
    sample_y = np.repeat(sample_y.reshape(1, ny, 3), nx, axis=0)
    normal_vecs = np.tile(normal_vec, nx * ny).reshape(nx, ny, 3)
    max_length = np.linalg.norm(cam.position - cam.domain_center) + 0.5 * np.linalg.norm(cam.domain_width)
    vectors = (sample_x + sample_y + normal_vecs * cam.width[2]) * (max_length / cam.width[2])
    positions = np.tile(cam.position, nx * ny).reshape(nx, ny, 3)
    return {
        "vp_pos": positions,
        "vp_dir": vectors,
        "center": cam.back_center,
        "bounds": (0.0, 1.0, 0.0, 1.0),
        "x_vec": np.ones(3, dtype="float64"),
        "y_vec": np.ones(3, dtype="float64"),
        "image": np.zeros((nx, ny, 4), dtype="float64"),
        "lens_type": "perspective",
    }


# ---------------------------------------------------------- transfer functions
class TransferFunction:
    def __init__(self, x_bounds, nbins=256):
        self.nbins = nbins
        self.x_bounds = [np.float64(xb) for xb in x_bounds]
        self.x = np.linspace(self.x_bounds[0], self.x_bounds[1], nbins, dtype="float64")
        self.y = np.zeros(nbins, dtype="float64")

    def add_gaussian(self, location, width, height):
        vals = height * np.exp(-((self.x - location) ** 2.0) / width)
        self.y = np.clip(np.maximum(vals, self.y), 0.0, np.inf)


class MultiVariateTransferFunction:
    def __init__(self, grey_opacity=False):
        self.n_field_tables = 0
        self.tables = []
        self.field_ids = [0] * 6
        self.weight_field_ids = [-1] * 6
        self.field_table_ids = [0] * 6
        self.weight_table_ids = [-1] * 6
        self.grey_opacity = grey_opacity

    def add_field_table(self, table, field_id, weight_field_id=-1, weight_table_id=-1):
        self.tables.append(table)
        self.field_ids[self.n_field_tables] = field_id
        self.weight_field_ids[self.n_field_tables] = weight_field_id
        self.weight_table_ids[self.n_field_tables] = weight_table_id
        self.n_field_tables += 1

    def link_channels(self, table_id, channels=0):
        for c in np.atleast_1d(channels):
            self.field_table_ids[int(c)] = table_id


class ColorTransferFunction(MultiVariateTransferFunction):
    def __init__(self, x_bounds, nbins=256, grey_opacity=False):
        MultiVariateTransferFunction.__init__(self)
        self.x_bounds = [np.float64(xb) for xb in x_bounds]
        self.nbins = nbins
        self.red = TransferFunction(self.x_bounds, nbins)
        self.green = TransferFunction(self.x_bounds, nbins)
        self.blue = TransferFunction(self.x_bounds, nbins)
        self.alpha = TransferFunction(self.x_bounds, nbins)
        self.funcs = (self.red, self.green, self.blue, self.alpha)
        self.grey_opacity = grey_opacity
        for i, tf in enumerate(self.funcs[:3]):
            self.add_field_table(tf, 0, weight_table_id=3)
            self.link_channels(i, i)
        self.add_field_table(self.funcs[3], 0)
        self.link_channels(3, 3)

    def add_gaussian(self, location, width, height):
        for tf, v in zip(self.funcs, height, strict=True):
            tf.add_gaussian(location, width, v)


class ProjectionTransferFunction(MultiVariateTransferFunction):
    def __init__(self, x_bounds=(-1e60, 1e60), n_fields=1):
        MultiVariateTransferFunction.__init__(self)
        self.x_bounds = [np.float64(xb) for xb in x_bounds]
        self.nbins = 2
        self.linear_mapping = TransferFunction(self.x_bounds, 2)
        self.link_channels(0, [0, 1, 2])
        for i in range(n_fields):
            self.add_field_table(self.linear_mapping, i)
            self.link_channels(i, i)
        self.link_channels(n_fields, [3, 4, 5])


def color_tf_from_layers(x_bounds, nbins, layers, grey_opacity=False):
    """A ColorTransferFunction with explicit (location, width, rgba) layers."""
    tf = ColorTransferFunction(x_bounds, nbins=nbins, grey_opacity=grey_opacity)
    for loc, w, rgba in layers:
        tf.add_gaussian(loc, w, list(rgba))
    return tf


# ------------------------------------------------------------------- kd-tree
class KDNode:
    __slots__ = ("parent", "left", "right", "le", "re", "grid", "node_id", "split_dim", "split_pos", "data")

    def __init__(self, parent, le, re, grid, node_id):
        self.parent = parent
        self.left = None
        self.right = None
        self.le = np.array(le, dtype="float64")
        self.re = np.array(re, dtype="float64")
        self.grid = grid
        self.node_id = node_id
        self.split_dim = -1
        self.split_pos = np.nan
        self.data = None

    def is_leaf(self):
        return self.left is None or self.right is None


def _get_choices(gles, gres, l_corner, r_corner):
    """kdtree_get_choices (amr_kdtools.pyx:760-823)."""
    n = gles.shape[0]
    my_max = 0
    my_split = 0
    best_dim = -1
    uniques_by_dim = [[], [], []]
    for dim in range(3):
        uniques = uniques_by_dim[dim]
        for i in range(n):
            for v in (gles[i, dim], gres[i, dim]):
                if not (l_corner[dim] < v and v < r_corner[dim]):
                    continue
                if not any(u == v for u in uniques):
                    uniques.append(v)
        if len(uniques) > my_max:
            best_dim = dim
            my_max = len(uniques)
            my_split = (len(uniques) - 1) // 2
    if best_dim == -1:
        return -1, 0.0, None, None
    tarr = np.array(uniques_by_dim[best_dim][:my_max], dtype="float64")
    tarr.sort()
    split = tarr[my_split]
    less = gles[:, best_dim] < split
    greater = gres[:, best_dim] > split
    return best_dim, split, less, greater


def _divide(node, dim, pos):
    """Node.divide (amr_kdtools.pyx:509-532): children inherit node.grid."""
    node.split_dim = dim
    node.split_pos = pos
    le = node.le.copy()
    re = node.re.copy()
    re[dim] = pos
    node.left = KDNode(node, le, re, node.grid, node.node_id << 1)
    re = node.re.copy()
    le = node.le.copy()
    le[dim] = pos
    node.right = KDNode(node, le, re, node.grid, (node.node_id << 1) + 1)


def _split_grids(node, gles, gres, gids):
    if gles.shape[0] == 0:
        return 0
    best_dim, split, less, greater = _get_choices(gles, gres, node.le, node.re)
    if best_dim == -1:
        return -1
    _divide(node, best_dim, split)
    if less.any():
        _insert_grids(node.left, gles[less], gres[less], gids[less])
    if greater.any():
        _insert_grids(node.right, gles[greater], gres[greater], gids[greater])
    return 0


def _insert_grids(node, gles, gres, gids):
    """Node.insert_grids (amr_kdtools.pyx:278-313) for one rank."""
    n = gles.shape[0]
    if n == 0:
        return
    if n == 1:
        contained = all(gles[0, i] <= node.le[i] and gres[0, i] >= node.re[i] for i in range(3))
        if contained:
            node.grid = int(gids[0])
            return
    if _split_grids(node, gles, gres, gids) == -1:
        node.grid = -1


def _add_grids(node, gles, gres, gids):
    """Node.add_grids (amr_kdtools.pyx:201-265)."""
    if node.is_leaf():
        _insert_grids(node, gles, gres, gids)
        return
    less = gles[:, node.split_dim] < node.split_pos
    greater = gres[:, node.split_dim] > node.split_pos
    if less.any():
        _add_grids(node.left, gles[less], gres[less], gids[less])
    if greater.any():
        _add_grids(node.right, gles[greater], gres[greater], gids[greater])


class KDTree:
    """Tree.build (amr_kdtree.py:63-118): grids added level by level."""

    def __init__(self, grids):
        """``grids``: list of objects with ``id``, ``level``, ``left_edge``,
        ``right_edge`` in index order."""
        self.grids = {g.id: g for g in grids}
        self.trunk = KDNode(None, [-np.inf] * 3, [np.inf] * 3, -1, 1)
        levels = sorted({g.level for g in grids})
        for lvl in range(0, max(levels) + 1 if levels else 0):
            gs = [g for g in grids if g.level == lvl]
            if not gs:
                continue
            gles = np.array([g.left_edge for g in gs], dtype="float64")
            gres = np.array([g.right_edge for g in gs], dtype="float64")
            gids = np.array([g.id for g in gs], dtype="int64")
            _add_grids(self.trunk, gles, gres, gids)

    def _walk(self, node, viewpoint):
        if node.is_leaf():
            if node.grid != -1:
                yield node
            return
        if viewpoint is None or not (viewpoint[node.split_dim] <= node.split_pos):
            first, second = node.left, node.right
        else:
            first, second = node.right, node.left
        yield from self._walk(first, viewpoint)
        yield from self._walk(second, viewpoint)

    def leaves(self, viewpoint=None):
        """kd_traverse (amr_kdtools.pyx:102-111): depth-first left-first
        without a viewpoint, else the viewpoint order of step_viewpoint
        (:708-755): at each split, the child on the far side first."""
        return list(self._walk(self.trunk, viewpoint))


def vertex_centred(cell: np.ndarray, log: bool) -> np.ndarray:
    """get_vertex_centered_data(no_ghost=True) then amr_kdtree.py:346-352."""
    v = cpu.ghost_zone_vertex_centre(cell)
    if log:
        v = v.astype("float64")
        v[v <= 0] = np.nan
        v = np.log10(v)
    return v


def brick_data(node, grid, vertex_data):
    """get_brick_data (amr_kdtree.py:325-374) for one leaf."""
    dds = (grid.right_edge - grid.left_edge) / grid.dims
    gle = grid.left_edge
    nle = node.le
    nre = node.re
    li = np.rint((nle - gle) / dds).astype("int32")
    ri = np.rint((nre - gle) / dds).astype("int32")
    dims = ri - li
    mask = np.ones(dims, dtype="uint8")
    data = [d[li[0]: ri[0] + 1, li[1]: ri[1] + 1, li[2]: ri[2] + 1].copy() for d in vertex_data]
    return data, mask, nle.copy(), nre.copy(), dims.astype("int64")


def render(kind, cam: Camera, bricks, order, tf=None, n_samples=1, num_threads=0, zbuffer=None,
           light_dir=(1.0, 1.0, 1.0), light_rgba=(1.0, 1.0, 1.0, 1.0)):
    """KDTreeVolumeSource.render's brick loop on the C oracle; returns the raw
    sampler image (before finalize_image) and the visited-cell count."""
    p = cam.sampler_params()
    s = cpu.OracleSampler(kind, p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                          p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                          camera_data=p["camera_data"], zbuffer=zbuffer, n_samples=n_samples, tf=tf,
                          light_dir=light_dir, light_rgba=light_rgba)
    ob = bricks if isinstance(bricks, cpu.OracleBricks) else cpu.OracleBricks(bricks)
    visits = s.render(ob, order, num_threads=num_threads)
    return p["image"], visits
