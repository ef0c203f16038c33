"""Known answers the sampler path must reproduce (derived from the code's
definitions, not from fixtures): axis-aligned projection and MIP of a cell
field against numpy, a constant field's projection against the analytic
path length, and volume rendering of a field inside one transfer-function
bin against the closed-form emission-absorption recurrence.  The oracle is
checked here; tests/test_gpu_known_answers.py checks the GPU path."""
import numpy as np
import pytest

from oracle import cpu as ocpu
from yt_gb300.camera import Camera

N = 16      # cells per axis
PIX = 24    # pixels per axis: i/(PIX-1) never falls on an interior cell face (16 i / 23 is an integer
            # only at i = 0 and 23)


def axis_camera(res=PIX):
    # plane-parallel, looking down +z through the unit cube, the back plane at z = 0
    return Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), res, lens_type="plane-parallel")


def field(seed=0):
    return np.random.default_rng(seed).lognormal(0.0, 1.0, (N, N, N))


def ray_origins(cam):
    """Each pixel's ray origin (generate_vector_info_plane_parallel,
    lenses.pyx:179-192)."""
    p = cam.sampler_params()
    vp = p["vp_pos"]
    nx, ny = cam.resolution
    w = cam.width
    out = np.zeros((nx, ny, 3))
    for i in range(nx):
        for j in range(ny):
            px = w[0] * i / (nx - 1) - w[0] / 2
            py = w[1] * j / (ny - 1) - w[1] / 2
            out[i, j] = [vp[0] * px + vp[3] * py + vp[9], vp[1] * px + vp[4] * py + vp[10],
                         vp[2] * px + vp[5] * py + vp[11]]
    return out


def expected_axis(cells, reduce, cam):
    """Rays along +z from (x, y) walk the cells floor(x*N), floor(y*N); rays
    on the cube's right faces (x or y == 1) miss."""
    o = ray_origins(cam)
    out = np.zeros(o.shape[:2])
    for i in range(o.shape[0]):
        for j in range(o.shape[1]):
            x, y = o[i, j, 0], o[i, j, 1]
            if 0 <= x < 1 and 0 <= y < 1:
                out[i, j] = reduce(cells[int(np.floor(x * N)), int(np.floor(y * N)), :])
    return out


def render(kind, cells, cam, tf=None):
    p = cam.sampler_params()
    s = ocpu.OracleSampler(kind, p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"], p["x_vec"],
                           p["y_vec"], p["width"], lens_type=p["lens_type"], camera_data=p["camera_data"], tf=tf)
    s.render(ocpu.OracleBricks([([cells], None, np.zeros(3), np.ones(3), [N] * 3)]), None)
    return p["image"]


def test_axis_projection_is_the_column_sum():
    cells = field()
    cam = axis_camera()
    img = render("projection", cells, cam)
    want = expected_axis(cells, lambda col: np.cumsum(col / N)[-1], cam)
    assert np.allclose(img[..., 0], want, rtol=1e-13, atol=0)


def test_axis_mip_is_the_column_max():
    cells = field(1)
    cam = axis_camera()
    img = render("mip", cells, cam)
    want = expected_axis(cells, np.max, cam)
    assert np.array_equal(img[..., 0], want)


@pytest.mark.parametrize("pos", [(1.3, 0.2, -0.7), (-0.4, 1.1, 1.6)])
def test_constant_field_projection_is_the_path_length(pos):
    """value x (t_exit - t_enter) of each ray through the unit cube, in the
    view's t units (t in [0, 1] spans width[2])."""
    c = 2.5
    cam = Camera(pos, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 20, lens_type="plane-parallel")
    img = render("projection", np.full((N, N, N), c), cam)
    p = cam.sampler_params()
    vp = p["vp_pos"]
    d = np.asarray(p["vp_dir"], dtype=np.float64)
    nx, ny = cam.resolution
    w = cam.width
    for i in range(nx):
        for j in range(ny):
            px = w[0] * i / (nx - 1) - w[0] / 2
            py = w[1] * j / (ny - 1) - w[1] / 2
            o = np.array([vp[0] * px + vp[3] * py + vp[9], vp[1] * px + vp[4] * py + vp[10],
                          vp[2] * px + vp[5] * py + vp[11]])
            with np.errstate(divide="ignore", invalid="ignore"):
                t0 = np.where(d != 0, (0 - o) / d, -np.inf)
                t1 = np.where(d != 0, (1 - o) / d, np.inf)
            lo = max(np.minimum(t0, t1).max(), 0.0)
            hi = min(np.maximum(t0, t1).min(), 1.0)
            want = c * max(hi - lo, 0.0)
            assert abs(img[i, j, 0] - want) <= 1e-12 * max(1.0, want), (i, j)


def test_uniform_field_in_one_bin_follows_the_recurrence():
    """Every sample sees the same value, so every sample has the same
    emission e; with one sample per cell of length dt = 1/N, each colour
    channel follows x <- x + dt e (1 - x): x = 1 - (1 - e/N)^N."""
    from yt_gb300.transfer_functions import ColorTransferFunction

    v = 0.3
    tf = ColorTransferFunction((0.0, 1.0), nbins=64)
    tf.add_gaussian(v, 0.05, [0.9, 0.6, 0.3, 0.8])
    vert = np.full((N + 1,) * 3, v)
    cam = axis_camera()
    p = cam.sampler_params()
    s = ocpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                           p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                           camera_data=p["camera_data"], tf=tf)
    s.render(ocpu.OracleBricks([([vert], None, np.zeros(3), np.ones(3), [N] * 3)]), None)
    img = p["image"]
    # the emission of each channel: table value at v weighted by the alpha table
    ys = [np.interp(v, np.linspace(0, 1, 64), t.y) for t in tf.funcs]
    o = ray_origins(cam)
    hit = (o[..., 0] < 1) & (o[..., 1] < 1)
    for ch in range(3):
        e = ys[ch] * ys[3]
        want = 1 - (1 - e / N) ** N
        assert np.allclose(img[hit, ch], want, rtol=1e-9), ch
        assert np.all(img[~hit, ch] == 0)
