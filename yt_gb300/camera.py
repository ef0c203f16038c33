"""Camera and lens parameters for the samplers, as yt's scene graph builds them.

This is the part of yt's ``Camera`` / ``Lens`` objects that the sampler sees:

* orientation basis          yt/utilities/orientation.py:59-85
* Lens.setup_box_properties  yt/visualization/volume_rendering/lens.py:45-61
* PlaneParallelLens          lens.py:83-121
* PerspectiveLens            lens.py:166-240
* Camera._get_sampler_params camera.py:275-281

``Camera.sampler_params()`` returns exactly the dictionary yt's
``camera._get_sampler_params(render_source)`` does (vp_pos, vp_dir, center,
bounds, x_vec, y_vec, width, image, lens_type, camera_data), and
``Camera.viewpoint`` the point the kd traversal orders bricks from.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def orientation(normal_vector, north_vector=None):
    """Return (unit_vectors [east, north, normal], inv_mat)."""
    normal_vector = np.array(normal_vector, dtype="float64")
    steady_north = north_vector is not None
    if north_vector is not None:
        north_vector = np.array(north_vector, dtype="float64")
    if not np.dot(normal_vector, normal_vector) > 0:
        raise ValueError("normal_vector cannot be the zero vector.")
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
    return unit_vectors, np.linalg.pinv(unit_vectors)


class Camera:
    """A camera looking from ``position`` at ``focus``."""

    def __init__(self, position, focus=(0.5, 0.5, 0.5), width=(1.0, 1.0, 1.0), resolution=(512, 512),
                 north_vector=None, lens_type="plane-parallel", domain_left=(0.0, 0.0, 0.0),
                 domain_right=(1.0, 1.0, 1.0)):
        if lens_type not in ("plane-parallel", "perspective"):
            raise NotImplementedError(f"lens {lens_type!r} is not supported")
        self.position = np.array(position, dtype="float64")
        self.focus = np.array(focus, dtype="float64")
        if np.array_equal(self.position, self.focus):
            raise RuntimeError("Cannot set the camera focus and position to the same value")
        if np.isscalar(width):
            width = (width, width, width)
        self.width = np.array(width, dtype="float64")
        if np.isscalar(resolution):
            resolution = (resolution, resolution)
        self.resolution = (int(resolution[0]), int(resolution[1]))
        self.north_vector = north_vector
        self.lens_type = lens_type
        dl = np.array(domain_left, dtype="float64")
        dr = np.array(domain_right, dtype="float64")
        self.domain_center = (dl + dr) / 2.0
        self.domain_width = dr - dl
        self.unit_vectors, self.inv_mat = orientation(self.focus - self.position, north_vector)
        uv, w, c = self.unit_vectors, self.width, self.focus
        self.box_vectors = np.array([uv[0] * w[0], uv[1] * w[1], uv[2] * w[2]])
        self.origin = c - 0.5 * w.dot(uv)
        self.back_center = c - 0.5 * w[2] * uv[2]
        self.front_center = c + 0.5 * w[2] * uv[2]
        if lens_type == "plane-parallel":
            # lens.py:114-121: a far-away viewpoint makes the kd order parallel
            self.viewpoint = self.front_center + uv[2] * 1.0e6 * w[2]
        else:
            self.viewpoint = self.front_center

    def sampler_params(self):
        if self.lens_type == "plane-parallel":
            p = self._plane_parallel()
        else:
            p = self._perspective()
        p["width"] = self.width.copy()
        p["camera_data"] = np.vstack((self.position, self.width, self.unit_vectors))
        return p

    def _plane_parallel(self):
        nx, ny = self.resolution
        return {
            "vp_pos": np.concatenate([self.inv_mat.ravel("F"), self.back_center.ravel()]),
            "vp_dir": self.box_vectors[2],
            "center": self.back_center,
            "bounds": (-self.width[0] / 2.0, self.width[0] / 2.0, -self.width[1] / 2.0, self.width[1] / 2.0),
            "x_vec": self.unit_vectors[0],
            "y_vec": self.unit_vectors[1],
            "image": np.zeros((nx, ny, 4), dtype="float64"),
            "lens_type": "plane-parallel",
        }

    def _perspective(self):
        nx, ny = self.resolution
        self.width[1] = self.width[0] * (ny / nx)
        east_vec, north_vec, normal_vec = self.unit_vectors
        px = np.linspace(-0.5, 0.5, nx)[np.newaxis, :]
        py = np.linspace(-0.5, 0.5, ny)[np.newaxis, :]
        sample_x = (self.width[0] * np.array(east_vec.reshape(3, 1) * px)).transpose()
        sample_y = (self.width[1] * np.array(north_vec.reshape(3, 1) * py)).transpose()
        sample_x = np.repeat(sample_x.reshape(nx, 1, 3), ny, axis=1)
        sample_y = np.repeat(sample_y.reshape(1, ny, 3), nx, axis=0)
        normal_vecs = np.tile(normal_vec, nx * ny).reshape(nx, ny, 3)
        max_length = np.linalg.norm(self.position - self.domain_center) + 0.5 * np.linalg.norm(self.domain_width)
        vectors = (sample_x + sample_y + normal_vecs * self.width[2]) * (max_length / self.width[2])
        positions = np.tile(self.position, nx * ny).reshape(nx, ny, 3)
        return {
            "vp_pos": positions,
            "vp_dir": vectors,
            "center": self.back_center,
            "bounds": (0.0, 1.0, 0.0, 1.0),
            "x_vec": np.ones(3, dtype="float64"),
            "y_vec": np.ones(3, dtype="float64"),
            "image": np.zeros((nx, ny, 4), dtype="float64"),
            "lens_type": "perspective",
        }

    def device_view(self):
        """The ``ytgb_view`` of this camera with rays generated on the device.

        Plane-parallel views carry yt's 12 + 3 ray parameters.  Perspective
        views carry the camera instead of yt's (nx, ny, 3) ray arrays
        (``YTGB_LENS_PERSPECTIVE``): position, the unit vectors, the width
        (with width[1] = width[0] * ny / nx as ``lens.py:176-178`` sets it)
        and max_length / width[2]; the kernel recomputes yt's per-pixel
        vectors (``lens.py:186-225``) bit for bit."""
        if self.lens_type == "plane-parallel":
            from .image_samplers import make_view

            p = self.sampler_params()
            nx, ny = self.resolution
            v, _, _ = make_view(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], nx, ny, p["x_vec"],
                                p["y_vec"], p["width"], p["lens_type"], p["camera_data"])
            return v
        nx, ny = self.resolution
        self.width[1] = self.width[0] * (ny / nx)
        uv = self.unit_vectors
        v = _lib.View()
        v.nx, v.ny = nx, ny
        v.lens = _lib.LENS_PERSPECTIVE
        v.extent = _lib.EXTENT_PERSPECTIVE
        for i in range(3):
            v.vp_pos[i] = float(self.position[i])
            v.vp_pos[3 + i] = float(uv[0][i])
            v.vp_pos[6 + i] = float(uv[1][i])
            v.vp_pos[9 + i] = float(uv[2][i])
            v.vp_dir[i] = float(self.width[i])
            v.center[i] = float(self.back_center[i])
            v.x_vec[i] = 1.0
            v.y_vec[i] = 1.0
            v.width[i] = float(self.width[i])
        for i, b in enumerate((0.0, 1.0, 0.0, 1.0)):
            v.bounds[i] = b
        v.pdx = (v.bounds[1] - v.bounds[0]) / nx
        v.pdy = (v.bounds[3] - v.bounds[2]) / ny
        max_length = np.linalg.norm(self.position - self.domain_center) + 0.5 * np.linalg.norm(self.domain_width)
        v.ray_scale = float(max_length / self.width[2])
        cd = np.vstack((self.position, self.width, uv)).ravel()
        for i in range(15):
            v.camera_data[i] = float(cd[i])
        return v
