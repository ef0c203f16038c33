"""The render server: each request's image is the same alone and in the mix
(bit for bit, and within 1e-5 of the oracle on an audit sample); admission
respects the HBM budget; latencies are recorded."""
import numpy as np
import pytest
import torch

from oracle import cpu as ocpu
from yt_gb300 import _lib, testing, workloads
from yt_gb300.amr_kdtree import AMRKDTree
from yt_gb300.camera import Camera
from yt_gb300.render import relative_error
from yt_gb300.serve import RenderServer, Request, latency_summary

pytestmark = pytest.mark.gpu


def make_server(cuda, **kw):
    w1 = workloads.amr_vr(root=32, levels=2, patch=8, res=32)
    w2 = workloads.uniform_vr(n=24, res=32, seed=3)
    tfs = {"a": w1.tf, "b": w2.tf, "c": workloads.color_tf((-0.2, 1.4), 5, nbins=128)}
    vols = {"amr": (w1.bricks, w1.kdtree), "uni": (w2.bricks, w2.kdtree)}
    return RenderServer(vols, tfs, device=cuda, **kw), w1, w2


def requests(n, seed=0, rate=None):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        if rate:
            t += rng.exponential(1.0 / rate)
        p = testing.fibonacci_sphere(1, radius=1.5)[0] + rng.normal(0, 0.3, 3)
        res = int(rng.choice([24, 32, 48]))
        lens = "perspective" if rng.random() < 0.5 else "plane-parallel"
        cam = Camera(p, (0.5, 0.5, 0.5), 1.5 if lens == "perspective" else 1.2, res, lens_type=lens)
        out.append(Request(i, str(rng.choice(["amr", "uni"])), str(rng.choice(["a", "b", "c"])), cam,
                           arrival=t))
    return out


@pytest.mark.parametrize("batch_pixels", [0, 40 * 40, 1 << 30])
def test_alone_equals_mixed(cuda, batch_pixels):
    """Every request's image is the same alone and in the mix, whether the
    group renders through the batch kernel (all small), the single-view
    kernel (all large) or both."""
    srv, w1, w2 = make_server(cuda, keep_images=True, slots=3, max_batch=8, batch_pixels=batch_pixels)
    reqs = requests(24)
    done = srv.run(reqs, realtime=False)
    assert len(done) == 24 and all(q.done >= q.arrival for q in done)
    assert all(q.done >= q.launched for q in done)
    for q in done:
        alone = srv.renderer(q.volume, q.tf).render(q.camera)
        assert torch.equal(alone.view(torch.int64), q.image.view(torch.int64)), q.rid
    # audit one request against the oracle
    q = done[0]
    bricks = w1.bricks if q.volume == "amr" else w2.bricks
    kd = w1.kdtree if q.volume == "amr" else w2.kdtree
    tf = srv.tfs[q.tf][0]
    p = q.camera.sampler_params()
    s = ocpu.OracleSampler("volume_render", p["vp_pos"], p["vp_dir"], p["center"], p["bounds"], p["image"],
                           p["x_vec"], p["y_vec"], p["width"], lens_type=p["lens_type"],
                           camera_data=p["camera_data"], tf=tf)
    s.render(ocpu.OracleBricks(bricks), kd.viewpoint_order(q.camera.viewpoint))
    assert relative_error(q.image.cpu().numpy(), p["image"], channels=(0, 1, 2))[0] <= 1e-5


def test_budget_admission_and_latency(cuda):
    # budget of about three 48^2 images: requests wait for memory, all finish
    srv, _, _ = make_server(cuda, hbm_budget=3 * 48 * 48 * 32, slots=2, max_batch=4)
    reqs = requests(20, seed=1, rate=2000.0)
    done = srv.run(reqs, realtime=True)
    assert len(done) == 20
    assert srv.in_use == 0
    s = latency_summary(done)
    assert s["p99_ms"] >= s["p50_ms"] > 0
    for q in done:
        assert q.admitted >= q.arrival - 1e-9 and q.launched >= q.admitted and q.done >= q.launched


def test_cancellation_and_slow_producer(cuda):
    """Requests cancelled while waiting are dropped without rendering and
    release their budget; a stalled loop turn (a simulated slow host) delays
    but does not lose requests."""
    import time as _time

    srv, _, _ = make_server(cuda, hbm_budget=2 * 48 * 48 * 32, slots=1, max_batch=2)
    reqs = requests(16, seed=4, rate=5000.0)
    state = {"turns": 0}

    def tick(server, now):
        state["turns"] += 1
        if state["turns"] == 3:
            for q in reqs[8:12]:
                q.cancelled = True
        if state["turns"] == 5:
            _time.sleep(0.02)

    srv.on_tick = tick
    done = srv.run(reqs, realtime=True)
    cancelled = {q.rid for q in srv.cancelled}
    assert {q.rid for q in done} | cancelled == {q.rid for q in reqs}
    assert not ({q.rid for q in done} & cancelled)
    assert srv.in_use == 0
    assert all(q.image is None for q in srv.cancelled)
