"""Pin the oracle to yt's own compiled sampler through the golden fixtures
(generated by tests/golden/make_golden.py from the reference sources).

Everything here is float64 and bit-exact -- the C oracle reproduces yt's
images, traversal sequences, vertex centring and kd-tree exactly -- except
the off-axis cell splatting, whose reference sums in an unspecified order.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import cpu as ocpu
from oracle import glue
from yt_gb300.amr_kdtree import AMRKDTree, vertex_centred

GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    return np.load(GOLD / name)


CAMS = [((0.5, 0.5, -1.0), (1.0, 1.0, 1.0), (24, 20), "plane-parallel"),
        ((1.3, 0.2, -0.7), (1.0, 1.0, 1.0), (24, 24), "plane-parallel"),
        ((0.4, 0.6, -1.2), (1.5, 1.5, 1.5), (20, 24), "perspective")]


class GoldenTF(glue.ColorTransferFunction):
    """A ColorTransferFunction whose tables are the fixture's."""

    def __init__(self, bounds, ys):
        super().__init__(tuple(bounds), nbins=ys.shape[1])
        for t, y in zip(self.funcs, ys):
            t.y = y.copy()


def test_ghost_zone_interpolate_exact():
    f = load("gz.npz")
    for k in ("a", "lin"):
        assert np.array_equal(ocpu.ghost_zone_vertex_centre(f[k]), f[k + "_out"])
        assert np.array_equal(vertex_centred(f[k]), f[k + "_out"])
    # known answer (test_interpolators.py:107-150): a linear field is reproduced
    i, j, k = np.meshgrid(np.arange(7), np.arange(8), np.arange(6), indexing="ij")
    assert np.allclose(f["lin_out"], 2.0 * i - 3.0 * j + 0.5 * k + 1.0, rtol=0, atol=1e-12)


def test_walk_volume_trace_exact():
    f = load("trace.npz")
    dims = f["dims"]
    brick = ([np.zeros(tuple(dims + 1))], None, f["le"], f["re"], dims)
    cap = f["cells"].shape[1]
    count, cells, ts = ocpu.trace_rays(brick, f["pos"], f["dirs"], f["max_t"], cap)
    assert np.array_equal(count, f["count"])
    assert (f["count"] > 0).sum() > 300
    for i in range(count.size):
        n = min(int(count[i]), cap)
        assert np.array_equal(cells[i, :n], f["cells"][i, :n]), i
        assert np.array_equal(ts[i, :n].view(np.uint64), f["ts"][i, :n].view(np.uint64)), i


NB_CAMS = [((0.3, 0.6, -1.0), (1.5, 1.5, 1.5), (24, 24), "perspective"),
           ((1.2, 0.3, -0.8), (1.0, 1.0, 1.0), (20, 24), "plane-parallel")]


@pytest.mark.parametrize("ci", range(2))
@pytest.mark.parametrize("ns", [1, 3])
def test_near_bound_exact(ci, ns):
    """yt's float64 range test on a field within 1e-9 of a transfer-function
    bound (near_bound.npz): the oracle keeps and drops the same samples."""
    f = load("near_bound.npz")
    tf = GoldenTF(f["tf_bounds"], f["tf_y"])
    pos, width, res, lens = NB_CAMS[ci]
    cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
    n = f["vertex"].shape[0] - 1
    brick = ([f["vertex"]], None, np.zeros(3), np.ones(3), [n, n, n])
    img, visits = glue.render("volume_render", cam, [brick], None, tf=tf, n_samples=ns)
    assert visits > 0
    assert np.array_equal(img, f[f"img_{ci}_{ns}"])


@pytest.mark.parametrize("ci", range(3))
@pytest.mark.parametrize("ns", [1, 3])
def test_volume_render_exact(ci, ns):
    f = load("vr.npz")
    tf = GoldenTF(f["tf_bounds"], f["tf_y"])
    pos, width, res, lens = CAMS[ci]
    cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
    brick = ([f["vertex"]], None, np.zeros(3), np.ones(3), [16, 16, 16])
    img, visits = glue.render("volume_render", cam, [brick], None, tf=tf, n_samples=ns)
    assert visits > 0
    assert np.array_equal(img, f[f"img_{ci}_{ns}"])


@pytest.mark.parametrize("ci", range(3))
def test_projections_exact(ci):
    f = load("proj.npz")
    cell = f["cell"]
    pos, width, res, lens = CAMS[ci]
    img, _ = glue.render("projection", glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens),
                         [([cell], None, np.zeros(3), np.ones(3), [12, 12, 12])], None)
    assert np.array_equal(img, f[f"proj_{ci}"])
    v = ocpu.ghost_zone_vertex_centre(cell)
    img, _ = glue.render("interpolated_projection", glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens),
                         [([v], None, np.zeros(3), np.ones(3), [12, 12, 12])], None, n_samples=2)
    assert np.array_equal(img, f[f"iproj_{ci}"])


class _G:
    def __init__(self, gid, level, le, re, data):
        self.id, self.level, self.left_edge, self.right_edge, self.data = gid, level, le, re, data
        self.dims = np.array(data.shape, dtype=np.int64)

    @property
    def dds(self):
        return (self.right_edge - self.left_edge) / self.dims


def golden_grids():
    f = load("kd.npz")
    return f, [_G(int(i), int(l), a, b, f[f"cell_{int(i)}"])
               for i, l, a, b in zip(f["gids"], f["levels"], f["gles"], f["gres"])]


def test_kdtree_oracle_and_product_exact():
    f, grids = golden_grids()
    ot = glue.KDTree(grids)
    leaves = ot.leaves()
    assert len(leaves) == f["leaf_le"].shape[0]
    for k, n in enumerate(leaves):
        assert np.array_equal(n.le, f["leaf_le"][k]) and np.array_equal(n.re, f["leaf_re"][k])
        assert n.grid == f["leaf_grid"][k]
    kd = AMRKDTree(grids)
    assert np.array_equal(kd.leaf_le, f["leaf_le"]) and np.array_equal(kd.leaf_re, f["leaf_re"])
    assert np.array_equal(kd.leaf_grid, f["leaf_grid"])
    idx = {id(n): k for k, n in enumerate(leaves)}
    for vp, want in zip(f["viewpoints"], f["orders"]):
        assert [idx[id(n)] for n in ot.leaves(vp)] == list(want)
        assert np.array_equal(kd.viewpoint_order(vp), want)


def test_kd_leaves_tile_the_domain():
    """kd_sum_volume (amr_kdtools.pyx:534-543): leaves with a grid tile the
    root grid's domain."""
    f, grids = golden_grids()
    vol = np.prod(f["leaf_re"] - f["leaf_le"], axis=1).sum()
    assert abs(vol - 1.0) < 1e-12


def test_amr_volume_render_exact():
    f, grids = golden_grids()
    g = load("amr_vr.npz")
    tf = GoldenTF(g["tf_bounds"], g["tf_y"])
    ot = glue.KDTree(grids)
    byid = {gr.id: gr for gr in grids}
    vcd = {}
    cam = glue.Camera((0.3, 0.6, -1.1), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), (32, 28), lens_type="perspective")
    assert np.array_equal(cam.viewpoint, g["viewpoint"])
    bricks = []
    for node in ot.leaves(cam.viewpoint):
        gr = byid[node.grid]
        if gr.id not in vcd:
            vcd[gr.id] = [glue.vertex_centred(gr.data, True)]
        bricks.append(glue.brick_data(node, gr, vcd[gr.id]))
    img, _ = glue.render("volume_render", cam, bricks, None, tf=tf)
    assert np.array_equal(img, g["image"])


def amr_cut_bricks():
    """The amr_vr.npz bricks in the golden camera's viewpoint order, built by
    the oracle's kd tree and vertex centring, and that camera."""
    f, grids = golden_grids()
    ot = glue.KDTree(grids)
    byid = {gr.id: gr for gr in grids}
    vcd = {}
    cam = glue.Camera((0.3, 0.6, -1.1), (0.5, 0.5, 0.5), (1.5, 1.5, 1.5), (32, 28), lens_type="perspective")
    bricks = []
    for node in ot.leaves(cam.viewpoint):
        gr = byid[node.grid]
        if gr.id not in vcd:
            vcd[gr.id] = [glue.vertex_centred(gr.data, True)]
        bricks.append(glue.brick_data(node, gr, vcd[gr.id]))
    return bricks, cam


@pytest.mark.parametrize("k", range(3))
def test_amr_cut_bounds_exact(k):
    """Transfer-function bounds cutting through the AMR data (amr_cut.npz):
    the oracle keeps and drops yt's samples and matches its image bit for bit."""
    g = load("amr_cut.npz")
    bricks, cam = amr_cut_bricks()
    assert np.array_equal(cam.viewpoint, g["viewpoint"])
    tf = GoldenTF(g[f"tf_bounds_{k}"], g[f"tf_y_{k}"])
    img, _ = glue.render("volume_render", cam, bricks, None, tf=tf)
    assert np.array_equal(img, g[f"image_{k}"])


LIGHTS = [((1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 1.0), 1), ((-0.3, 0.8, 0.2), (0.9, 0.5, 0.2, 1.0), 3)]


@pytest.mark.parametrize("ci", range(3))
@pytest.mark.parametrize("li", range(2))
@pytest.mark.parametrize("grey", [0, 1])
def test_light_source_exact(ci, li, grey):
    """LightSourceRenderSampler (image_samplers.pyx:496-590, eval_gradient
    fixed_interpolator.cpp:116-148, FIT_eval_transfer_with_light
    field_interpolation_tables.pxd:115-143): oracle == compiled reference,
    bit for bit."""
    f = load("light.npz")
    tf = GoldenTF(f["tf_bounds"], f["tf_y"])
    tf.grey_opacity = grey
    pos, width, res, lens = CAMS[ci]
    ldir, lrgba, ns = LIGHTS[li]
    cam = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
    brick = ([f["vertex"]], None, np.zeros(3), np.ones(3), [16, 16, 16])
    img, visits = glue.render("light_source", cam, [brick], None, tf=tf, n_samples=ns, light_dir=ldir,
                              light_rgba=lrgba)
    assert visits > 0
    assert np.array_equal(img, f[f"img_{ci}_{li}_{ns}_{grey}"])


@pytest.mark.parametrize("name", ["vr1", "vr2", "proj", "iproj"])
def test_octree_exact(name):
    """cast_through_octree (image_samplers.pyx:202-288) over the reference's
    octree ray caster (_octree_raytracing.hpp): oracle == compiled reference,
    bit for bit."""
    f = load("octree.npz")
    oc = ocpu.OracleOctree(int(f["depth"]), np.zeros(3), np.ones(3), f["ipos"], f["lvl"])
    cam = glue.Camera((0.3, 1.45, -0.9), (0.5, 0.5, 0.5), (1.3, 1.3, 1.3), (26, 22), lens_type="perspective")
    p = cam.sampler_params()
    tf = GoldenTF(f["tf_bounds"], f["tf_y"])
    kind, ns, t = {"vr1": ("volume_render", 1, tf), "vr2": ("volume_render", 2, tf), "proj": ("projection", 1, None),
                   "iproj": ("interpolated_projection", 2, None)}[name]
    s = ocpu.OracleSampler(kind, p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"], p["x_vec"],
                           p["y_vec"], p["width"], lens_type=p["lens_type"], camera_data=p["camera_data"],
                           n_samples=ns, tf=t)
    visits = ocpu.render_octree(s, f["cells"], oc)
    assert visits > 0
    assert np.array_equal(p["image"], f[f"img_{name}"])


def offaxis_case(f, i):
    """Inputs of case i of offaxis.npz (make_golden.offaxis_inputs)."""
    nx, ny, ext = (int(v) for v in f[f"view{i}"])
    cells = [f[k] for k in ("X", "D", "Q", "W")]
    if ext:
        cells = [np.ascontiguousarray(np.concatenate([a, f["e" + k]])) for a, k in zip(cells, "XDQW")]
    return (*cells, f[f"rot{i}"], nx, ny)


@pytest.mark.parametrize("i", range(5))
def test_offaxis_oracle(i):
    """add_cells_to_image_offaxis: the oracle against the reference's own
    images.  Both are float64 and differ only in summation order (the
    reference normalises its stamps with numpy's pairwise sum and adds its
    per-thread buffers in any order), hence 1e-12 rather than bit-exact."""
    f = load("offaxis.npz")
    X, D, Q, W, rot, nx, ny = offaxis_case(f, i)
    b, bw = np.zeros((nx, ny)), np.zeros((nx, ny))
    ocpu.add_cells_to_image_offaxis(Xp=X, dXp=D, qty=Q, weight=W, rotation=rot, buffer=b, buffer_weight=bw,
                                    Nx=nx, Ny=ny)
    for got, ref in ((b, f[f"b{i}"]), (bw, f[f"bw{i}"])):
        assert np.max(np.abs(ref)) > 0
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_offaxis_stamp_product_matches_oracle():
    """The product's host stamps (numpy, the reference's operations) and the
    oracle's (C): identical masks, values equal up to the normalising sum."""
    from yt_gb300 import offaxis

    f = load("offaxis.npz")
    for i in range(int(f["n"])):
        X, D, Q, W, rot, nx, ny = offaxis_case(f, i)
        s1, m1 = offaxis.offaxis_stamp(rot, np.max(D), nx, ny)
        s2, m2 = ocpu.offaxis_stamp(rot, np.max(D), nx, ny)
        assert s1.shape == s2.shape and np.array_equal(m1, m2)
        assert np.max(np.abs(s1 - s2)) <= 1e-15
