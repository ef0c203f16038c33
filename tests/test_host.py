"""Host-side pieces of libytgb against the oracle (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import cpu as ocpu
from oracle import glue
from yt_gb300 import _lib, testing, workloads
from yt_gb300.amr_kdtree import AMRKDTree, vertex_centred
from yt_gb300.camera import Camera
from yt_gb300.image_samplers import make_view
from yt_gb300.transfer_functions import ColorTransferFunction, pack
from yt_gb300.volume import BrickSet

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol():
    hdr = (ROOT / "include" / "ytgb.h").read_text()
    names = set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(ytgb_\w+)\s*\(", hdr, flags=re.M))
    assert len(names) >= 12
    L = _lib.lib()
    for n in sorted(names):
        assert hasattr(L, n), n
    assert set(_lib.SIGNATURES) == names


CAMS = [
    ((0.5, 0.5, -1.0), (1.0, 1.0, 1.0), 64, "plane-parallel"),
    ((1.3, 0.2, -0.7), (1.0, 1.0, 1.0), (64, 50), "plane-parallel"),
    ((-0.4, 1.1, 1.6), (0.7, 0.7, 0.7), 33, "plane-parallel"),
    ((0.5, 0.5, -1.0), (1.5, 1.5, 1.5), 96, "perspective"),
    ((1.6, 1.4, 1.9), (1.5, 1.5, 1.5), (80, 64), "perspective"),
    ((0.45, 0.52, 0.55), (1.5, 1.5, 1.5), 48, "perspective"),
]


@pytest.mark.parametrize("pos,width,res,lens", CAMS)
def test_camera_params_match_oracle(pos, width, res, lens):
    a = Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens).sampler_params()
    b = glue.Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens).sampler_params()
    for k in ("vp_pos", "vp_dir", "center", "x_vec", "y_vec", "width", "camera_data"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    assert tuple(a["bounds"]) == tuple(b["bounds"])
    assert a["lens_type"] == b["lens_type"]


@pytest.fixture(scope="module")
def amr_small():
    return workloads.amr_vr(root=32, levels=2, patch=8, res=64)


@pytest.mark.parametrize("pos,width,res,lens", CAMS)
def test_brick_rects_match_oracle(amr_small, pos, width, res, lens):
    w = amr_small
    cam = Camera(pos, (0.5, 0.5, 0.5), width, res, lens_type=lens)
    p = cam.sampler_params()
    nx, ny = cam.resolution
    view, _, _ = make_view(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], nx, ny, p["x_vec"], p["y_vec"],
                           p["width"], p["lens_type"], p["camera_data"])
    bs = BrickSet(w.bricks, device="cpu")
    order = w.order(cam)
    rects = bs.rects(view, order)
    s = ocpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                           p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                           camera_data=p["camera_data"], tf=w.tf)
    ob = ocpu.OracleBricks(w.bricks)
    for k, b in enumerate(order):
        assert np.array_equal(rects[k], s.padded_rect(ob, int(b))), k


def test_vertex_centring_matches_oracle():
    g = testing.blob_grid(18, seed=2)
    assert np.array_equal(vertex_centred(g.data), ocpu.ghost_zone_vertex_centre(g.data))


def test_kdtree_matches_oracle_restatement():
    grids = testing.amr_blob_grids(root=32, levels=2, patch=8, seed=4)
    kd = AMRKDTree(grids)
    ot = glue.KDTree(grids)
    leaves = ot.leaves()
    assert kd.num_bricks == len(leaves)
    for k, n in enumerate(leaves):
        assert np.array_equal(kd.leaf_le[k], n.le) and np.array_equal(kd.leaf_re[k], n.re)
        assert kd.leaf_grid[k] == n.grid
    rng = np.random.default_rng(0)
    for _ in range(6):
        vp = rng.uniform(-1.0, 2.0, 3)
        want = [(tuple(n.le), n.grid) for n in ot.leaves(vp)]
        got = [(tuple(kd.leaf_le[k]), kd.leaf_grid[k]) for k in kd.viewpoint_order(vp)]
        assert got == want
    many = kd.viewpoint_orders(np.array([[0.1, 0.2, 3.0], [2.0, -1.0, 0.5]]))
    assert np.array_equal(many[1], kd.viewpoint_order([2.0, -1.0, 0.5]))


def test_bricks_match_oracle_slicing():
    grids = testing.amr_blob_grids(root=32, levels=2, patch=8, seed=1)
    kd = AMRKDTree(grids)
    ot = glue.KDTree(grids)
    byid = {g.id: g for g in grids}
    vcd = {}
    for k, node in enumerate(ot.leaves()):
        g = byid[node.grid]
        if g.id not in vcd:
            vcd[g.id] = [glue.vertex_centred(g.data, True)]
        want = glue.brick_data(node, g, vcd[g.id])
        got = kd.brick(k)
        np.testing.assert_array_equal(got[0][0], want[0][0])
        assert np.array_equal(got[4], want[4])


def test_tf_pack_ctf_layout():
    tf = ColorTransferFunction((-0.2, 1.3), nbins=256)
    for loc, w, rgba in testing.ctf_layers((-0.2, 1.3), 4):
        tf.add_gaussian(loc, w, list(rgba))
    pk = pack(tf)
    h = pk.header
    assert h.n_fits == 4 and h.ctf_fast == 1 and h.nbins_max == 256
    assert list(h.weight_table_id)[:4] == [3, 3, 3, -1]
    assert list(h.field_table_ids) == [0, 1, 2, 3, 0, 0]
    # exclusive bounds: the float nearest outside each float64 bound
    assert np.float32(h.lo_excl[0]) <= -0.2 and np.float64(np.nextafter(np.float32(h.lo_excl[0]), np.float32(1))) > -0.2
    assert np.float32(h.hi_excl[0]) >= 1.3 and np.float64(np.nextafter(np.float32(h.hi_excl[0]), np.float32(-2))) < 1.3
    tab = pk.tables.reshape(4, 256, 4)
    y = tf.funcs[1].y
    assert np.array_equal(tab[1, :, 0], y.astype(np.float32))
    dbin = (1.3 - -0.2) / 255
    d0 = -0.2 + np.arange(255) * dbin
    assert np.allclose(tab[1, :255, 2].astype(np.float64) + tab[1, :255, 3], d0, rtol=0, atol=1e-14)


def test_tf_pack_rejects_bad_input():
    class Bad:
        n_field_tables = 1
        tables = [type("T", (), {"y": np.zeros(1), "x_bounds": (0.0, 1.0)})()]
        field_ids = [0] * 6
        weight_field_ids = [-1] * 6
        weight_table_ids = [-1] * 6
        field_table_ids = [0] * 6
        grey_opacity = 0

    with pytest.raises(_lib.YtgbError):
        pack(Bad())


def test_tf_pack_out_of_float32_range():
    """Tables whose bounds overflow float32 pack only when all-zero (they
    evaluate to 0 everywhere, as yt's float64 lookup does)."""
    from yt_gb300.transfer_functions import MultiVariateTransferFunction, TransferFunction

    def one_table(t):
        mv = MultiVariateTransferFunction()
        mv.add_field_table(t, 0)
        mv.link_channels(0, [0, 1, 2])
        return mv

    pk = pack(one_table(TransferFunction((-1e60, 1e60), 2)))
    assert pk.header.hi_excl[0] == -np.inf and pk.header.lo_excl[0] == np.inf
    nonzero = TransferFunction((-1e60, 1e60), 4)
    nonzero.y[:] = 1.0
    with pytest.raises(_lib.YtgbError, match="float32 range"):
        pack(one_table(nonzero))


def test_brick_rects_rejects_bad_order(amr_small):
    w = amr_small
    cam = w.views[0].camera
    p = cam.sampler_params()
    view, _, _ = make_view(p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], 64, 64, p["x_vec"], p["y_vec"],
                           p["width"], p["lens_type"], p["camera_data"])
    bs = BrickSet(w.bricks[:3], device="cpu")
    with pytest.raises(_lib.YtgbError):
        bs.rects(view, np.array([0, 5], dtype=np.int32))


def test_sampler_constructor_errors():
    from yt_gb300.image_samplers import ProjectionSampler

    img = np.zeros((4, 5, 4))
    with pytest.raises(RuntimeError, match="Bad lens shape"):
        ProjectionSampler(np.zeros((4, 4, 3)), np.zeros((4, 5, 3)), np.zeros(3), (0, 1, 0, 1), img, np.ones(3),
                          np.ones(3), np.zeros(3), "KDTree", 1, lens_type="perspective")
    s = ProjectionSampler(np.atleast_3d(np.zeros(12)), np.atleast_3d(np.ones(3)), np.zeros(3), (0, 1, 0, 1), img,
                          np.ones(3), np.ones(3), np.ones(3), "Nope", 1, lens_type="plane-parallel")
    with pytest.raises(NotImplementedError):
        s(None)


def _args_for(view, n_order=1):
    a = _lib.RenderArgs()
    a.kind = _lib.PROJECTION
    a.n_samples = 1
    a.n_order = n_order
    a.view = view
    buf = np.zeros(64, dtype=np.float64)
    base = buf.ctypes.data
    a.bricks = base
    a.order = base
    a.rects = base
    a.data = base
    a.bounds = base
    a.image = base
    return a, buf


def test_render_rejects_misaligned_pointers_before_launch():
    """Host-side guards: a misaligned rects table (read as 16-byte int4) is
    rejected before any device work (so this runs without a GPU)."""
    cam = Camera((0.5, 0.5, -1.0), 0.5, 1.0, 8)
    a, buf = _args_for(cam.device_view())
    a.rects = buf.ctypes.data + 4
    st = _lib.lib().ytgb_render(C.byref(a), None)
    assert st == _lib.ERR_INVALID and b"misaligned" in _lib.lib().ytgb_last_error()
    a.rects = buf.ctypes.data
    a.bounds = None
    assert _lib.lib().ytgb_render(C.byref(a), None) == _lib.ERR_INVALID


def test_batch_plan_rejects_misaligned_and_counts_tiles():
    cam = Camera((0.5, 0.5, -1.0), 0.5, 1.0, (20, 33))
    e = (_lib.BatchEntry * 2)()
    a, buf = _args_for(cam.device_view())
    e[0].args = a
    e[1].args = a
    t, s = C.c_int32(), C.c_int32()
    assert _lib.lib().ytgb_batch_plan(e, 2, 0, C.byref(t), C.byref(s)) == 0
    per = ((20 + 7) // 8) * ((33 + 15) // 16)
    assert t.value == 2 * per and e[1].tile_begin == per and e[1].tiles_y == 3
    e[1].args.rects = buf.ctypes.data + 8
    assert _lib.lib().ytgb_batch_plan(e, 2, 0, C.byref(t), C.byref(s)) == _lib.ERR_INVALID


def test_batch_tables_are_aligned_for_every_view():
    """Batch packs every view's rects + order into one buffer; each view's
    rects must start on a 16-byte boundary (ytgb_batch_plan checks it)."""
    from yt_gb300.batch import Batch, Job
    from yt_gb300.render import Renderer

    w = workloads.amr_vr(root=32, levels=2, patch=8, res=16)
    r = Renderer(w.bricks, w.tf, device="cpu", kdtree=w.kdtree)
    sub = Renderer(w.bricks[:7], w.tf, device="cpu")  # 7 bricks: 35-int tables
    jobs = [Job(sub, Camera((0.5, 0.5, -1.0), 0.5, 1.2, 12)), Job(r, Camera((1.3, 0.4, -0.6), 0.5, 1.5, 16,
                                                                           lens_type="perspective")),
            Job(sub, Camera((0.2, 1.4, 0.3), 0.5, 1.2, (9, 14)))]
    b = Batch(jobs, device="cpu")
    for g in b.groups:
        for k in range(g.n):
            assert g.entries[k].args.rects % 16 == 0


def test_leaf_slices_match_brick():
    from yt_gb300.amr_kdtree import AMRKDTree

    kd = AMRKDTree(testing.amr_blob_grids(root=32, levels=2, patch=8, seed=3), log_field=True)
    lg, li, dims = kd.leaf_slices()
    for k in range(0, kd.num_bricks, 7):
        data, mask, le, re, d = kd.brick(k)
        g = kd.grids[lg[k]]
        assert g.id == kd.leaf_grid[k]
        assert np.array_equal(d, dims[k])
        v = kd._vertex(g)
        s = v[li[k][0]: li[k][0] + d[0] + 1, li[k][1]: li[k][1] + d[1] + 1, li[k][2]: li[k][2] + d[2] + 1]
        assert np.array_equal(s, data[0], equal_nan=True)


def test_native_brick_scan_matches_python():
    """_ytgb_marshal.scan flattens a sampler's bricks exactly as the Python
    scan does, and declines bricks that need converting."""
    from yt_gb300 import volume
    from yt_gb300.partitioned_grid import PartitionedGrid
    from yt_gb300.image_samplers import brick_tuple

    if volume._marshal() is None:
        pytest.skip("_ytgb_marshal not built")
    rng = np.random.default_rng(3)
    bricks = []
    for k in range(30):
        dims = rng.integers(1, 7, 3)
        data = [rng.random(tuple(int(d) + 1 for d in dims)) for _ in range(int(rng.integers(1, 4)))]
        mask = None if k % 4 == 0 else np.ones(tuple(int(d) for d in dims), np.uint8)
        le = rng.random(3)
        bricks.append((data, mask, le if k % 3 else list(le), le + 1.0, tuple(int(d) for d in dims)))
    pg = PartitionedGrid(0, [rng.random((3, 4, 5))], np.ones((2, 3, 4), np.uint8), np.zeros(3), np.ones(3),
                         np.array([2, 3, 4]))
    bricks.append(brick_tuple(pg))
    bricks.append(pg)  # the object itself: its attributes are read
    n = len(bricks)

    def arrays():
        return np.ones((n, 3), np.int64), np.zeros((n, 3)), np.ones((n, 3)), np.zeros(n, np.int64)

    a = arrays()
    got = volume._scan(bricks, n, *a)
    assert got is not None
    b = arrays()
    ref = volume.BrickSet.__new__(volume.BrickSet)._scan_python(bricks, n, *b)
    for x, y in zip(got + a, ref + b):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    # a Fortran-ordered field, a float32 field or a bool mask: left to Python
    for bad in ([np.asfortranarray(rng.random((3, 3, 3)))], [rng.random((3, 3, 3)).astype(np.float32)]):
        odd = list(bricks) + [(bad, None, np.zeros(3), np.ones(3), (2, 2, 2))]
        assert volume._scan(odd, len(odd), *[np.resize(v, (len(odd),) + v.shape[1:]) for v in arrays()]) is None
    odd = list(bricks) + [([rng.random((3, 3, 3))], np.ones((2, 2, 2), bool), np.zeros(3), np.ones(3), (2, 2, 2))]
    assert volume._scan(odd, len(odd), *[np.resize(v, (len(odd),) + v.shape[1:]) for v in arrays()]) is None


def test_native_brick_layout_matches_numpy():
    """ytgb_brick_layout's descriptors and cell-boundary tables equal the
    numpy elementwise formulas (PartitionedGrid.__cinit__'s dds = (RE-LE)/dims,
    idds = 1/dds; the tables k*dds + le) bit for bit."""
    from yt_gb300.volume import BrickSet

    rng = np.random.default_rng(8)
    n = 25
    dims = rng.integers(1, 20, (n, 3)).astype(np.int64)
    le = rng.uniform(-1, 1, (n, 3))
    re = le + rng.uniform(1e-3, 2, (n, 3))
    nfields = rng.integers(1, 4, n).astype(np.int64)
    sizes = (dims + 1).prod(axis=1)
    bs = BrickSet.__new__(BrickSet)
    bs.n = n
    desc, stride, data_off, total, bounds = bs._layout(dims, le, re, nfields, sizes, sizes)
    dds = (re - le) / dims
    assert np.array_equal(desc["dds"], dds) and np.array_equal(desc["idds"], 1.0 / dds)
    assert np.array_equal(desc["snap"], 1e-10 * dds)
    assert np.array_equal(desc["lef"], le.astype(np.float32)) and np.array_equal(desc["iddsf"],
                                                                                  (1.0 / dds).astype(np.float32))
    st = (sizes + 3) & ~3
    assert np.array_equal(stride, st) and np.array_equal(data_off, np.concatenate([[0], np.cumsum(st * nfields)])[:n])
    assert total == int((st * nfields).sum())
    cnt = (dims + 1).ravel()
    starts = np.concatenate([[0], np.cumsum(cnt)])
    kk = np.arange(starts[-1], dtype=np.float64) - np.repeat(starts[:-1], cnt)
    ref = kk * np.repeat(dds.ravel(), cnt) + np.repeat(le.ravel(), cnt)
    assert np.array_equal(bounds, ref)
    assert np.array_equal(desc["bounds_offset"], starts[:-1].reshape(n, 3)[:, 0])
    assert (desc["mask_offset"] == -1).all()


def test_native_offaxis_stamp_matches_numpy():
    """ytgb_offaxis_depths (direct_integrate_cube natively) gives the numpy
    restatement's stamps and masks bit for bit."""
    from yt_gb300 import offaxis
    from yt_gb300.camera import Camera

    for pos, dxm, n in [((0.1, 0.3, -1.2), 0.05, 64), ((1.3, 0.2, 0.4), 0.2, 96), ((0.5, 0.5, -1.0), 0.02, 200),
                        ((-0.4, 1.1, 0.3), 0.11, 48)]:
        rot = Camera(pos, (0.5, 0.5, 0.5), (1, 1, 1), (n, n), lens_type="plane-parallel").inv_mat.T
        s1, m1 = offaxis.offaxis_stamp(rot, dxm, n, n)
        s2, m2 = offaxis.offaxis_stamp(rot, dxm, n, n, native=False)
        assert np.array_equal(s1.view(np.int64), s2.view(np.int64)) and np.array_equal(m1, m2)


def test_range_eps_is_the_largest_finite_value():
    """BrickSet(with_lo=True).range_eps = 2^-24 * the largest finite |value|
    of the arena (NaN and infinite values excluded, the padding between
    fields zeroed); 0 without the rounding errors."""
    from yt_gb300.volume import BrickSet

    rng = np.random.default_rng(2)
    a = rng.normal(0.0, 3.0, (5, 5, 5))
    b = rng.normal(0.0, 1.0, (3, 4, 6))
    a[0, 0, 0], a[1, 1, 1], b[0, 0, 0] = np.nan, np.inf, -np.inf
    bricks = [([a], None, np.zeros(3), np.ones(3), np.array([4, 4, 4])),
              ([b], None, np.zeros(3), np.ones(3), np.array([2, 3, 5]))]
    bs = BrickSet(bricks, device="cpu", with_lo=True)
    finite = np.concatenate([a[np.isfinite(a)], b[np.isfinite(b)]]).astype(np.float32)
    assert bs.range_eps == float(np.abs(finite).max()) * 2.0 ** -24
    assert BrickSet(bricks, device="cpu").range_eps == 0.0
    bs.data[0] = 1e30
    assert bs.range_eps == float(np.abs(finite).max()) * 2.0 ** -24  # kept until data_changed()
    bs.data_changed()
    assert bs.range_eps == float(np.float32(1e30)) * 2.0 ** -24
