"""Host logic of the render server, without a GPU: the priority level of
each launch (first come, first served among batches in flight)."""
from yt_gb300.serve import PRIORITY_LEVELS, launch_level


def test_launch_level_is_below_every_batch_in_flight():
    assert launch_level([]) == 0
    assert launch_level([0]) == 1
    assert launch_level([1, 0]) == 2
    assert launch_level([2]) == 3
    # the lowest level is shared once reached
    assert launch_level([PRIORITY_LEVELS - 1]) == PRIORITY_LEVELS - 1
    # an idle GPU starts again at the top
    assert launch_level(iter(())) == 0
