"""Lane assignment of gls_raw_batch (CPU only): frames by decreasing pixel count, each to the
lane with the fewest pixels so far, ties to the lower frame index and lane."""
import pytest

from climage_gb300 import gls


def test_equal_frames_round_robin():
    assert gls.batch_plan([(4032, 3024)] * 6, 3) == [0, 1, 2, 0, 1, 2]


def test_largest_first_to_least_loaded():
    sizes = [(4032, 3024), (1920, 1080), (8064, 6048), (2016, 1512), (4032, 3024)]
    # 8064x6048 -> lane 0; the two 12 Mpx frames -> lanes 1, 2; 2016x1512 -> lane 1; 1920x1080 -> lane 2
    assert gls.batch_plan(sizes, 3) == [1, 2, 0, 1, 2]


def test_loads_balanced_for_a_burst():
    import random
    rnd = random.Random(4)
    choices = [(1920, 1080), (2016, 1512), (4032, 3024), (8064, 6048)]
    sizes = [rnd.choice(choices) for _ in range(64)]
    lanes = 4
    plan = gls.batch_plan(sizes, lanes)
    load = [0] * lanes
    for (w, h), l in zip(sizes, plan):
        load[l] += w * h
    # LPT is within 4/3 of the optimum; the optimum is at least the mean and the largest frame
    bound = max(sum(load) / lanes, max(w * h for w, h in sizes))
    assert max(load) <= 4 / 3 * bound
    assert gls.batch_plan(sizes, lanes) == plan  # deterministic


def test_degenerate_inputs():
    assert gls.batch_plan([(64, 48)] * 3, 1) == [0, 0, 0]
    assert gls.batch_plan([], 2) == []
    with pytest.raises(gls.GlsError):
        gls.batch_plan([(64, 48)], 0)
