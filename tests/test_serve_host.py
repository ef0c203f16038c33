"""Host logic of the render server, without a GPU: the priority level of
each launch (first come, first served among batches in flight)."""
from yt_gb300.camera import Camera
from yt_gb300.serve import PRIORITY_LEVELS, Request, launch_level, split_group


def test_launch_level_is_below_every_batch_in_flight():
    assert launch_level([]) == 0
    assert launch_level([0]) == 1
    assert launch_level([1, 0]) == 2
    assert launch_level([2]) == 3
    # the lowest level is shared once reached
    assert launch_level([PRIORITY_LEVELS - 1]) == PRIORITY_LEVELS - 1
    # an idle GPU starts again at the top
    assert launch_level(iter(())) == 0


def _req(i, res):
    return Request(i, "v", "t", Camera((0.5, 0.5, -1.0), (0.5, 0.5, 0.5), 1.0, res), arrival=0.01 * i)


def test_split_group_batches_only_small_requests():
    reqs = [_req(0, 256), _req(1, 2048), _req(2, 256), _req(3, 512), _req(4, 128)]
    small, large = split_group(reqs, 512 * 512)
    assert [q.rid for q in small] == [0, 2, 4] and [q.rid for q in large] == [1, 3]
    # a lone small request takes the single-view kernel, first
    small, large = split_group([_req(0, 2048), _req(1, 256)], 512 * 512)
    assert small == [] and [q.rid for q in large] == [1, 0]
    # 0 batches nothing; a huge threshold batches everything
    assert split_group(reqs, 0)[0] == []
    assert len(split_group(reqs, 1 << 30)[0]) == 5


def test_latency_summary_p99_interval():
    from yt_gb300.serve import latency_summary

    reqs = []
    for i, ms in enumerate(list(range(1, 200)) + [1000]):
        q = _req(i, 64)
        q.arrival, q.done = 0.0, ms / 1e3
        reqs.append(q)
    s = latency_summary(reqs)
    assert s["n"] == 200 and abs(s["p50_ms"] - 100.5) < 1e-9
    lo, hi = s["p99_ci95_ms"]
    assert lo <= s["p99_ms"] <= hi and hi <= 1000.0


def test_bench_p99_flags():
    """The per-rate comparison bench.py writes from two latency summaries."""
    import importlib.util
    from pathlib import Path

    spec = importlib.util.spec_from_file_location("bench", Path(__file__).resolve().parent.parent / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    a = {"p99_ms": 10.0, "p99_ci95_ms": [9.0, 12.0]}
    b = {"p99_ms": 11.0, "p99_ci95_ms": [10.5, 13.0]}
    c = {"p99_ms": 20.0, "p99_ci95_ms": [18.0, 25.0]}
    assert bench.p99_flags(a, b) == {"served_beats_plain_p99": True, "p99_intervals_overlap": True}
    assert bench.p99_flags(b, a) == {"served_beats_plain_p99": False, "p99_intervals_overlap": True}
    assert bench.p99_flags(a, c) == {"served_beats_plain_p99": True, "p99_intervals_overlap": False}
