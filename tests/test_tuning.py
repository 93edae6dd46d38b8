"""The persistent query kernel's autotuner: its search logic on the host, with synthetic cost functions (no device).

The device side (every schedule gives identical results; the autotuner keeps the fastest) is in test_hibf_gpu.py."""

import ctypes

import pytest

from hibf_gb300 import _build, _native as N
from hibf_gb300.hibf import tune_search

VARIANTS = {(1, 8, 7), (2, 8, 7), (1, 8, 5), (2, 8, 5), (1, 16, 7), (1, 16, 5)}


@pytest.fixture(scope="module", autouse=True)
def lib():
    _build.build()
    return N.lib()


def kernel(t):
    return t["values_per_lane"], t["fetch_bytes"], t["counter_bits"]


def test_default_schedule():
    t = N.Tuning()
    N.lib().hibf_gpu_tuning_default(ctypes.byref(t))
    assert t.as_dict() == dict(values_per_lane=1, fetch_bytes=8, counter_bits=7, blocks_per_sm=0, early_exit_first=0,
                               early_exit_step=32, early_exit_stages=N.EARLY_EXIT_ADAPTIVE, early_exit_min=256,
                               block_queries=8192, schedule=N.SCHEDULE_QUEUE, level_values_per_lane=0)


def cost(t):
    # fastest: 16-byte fetch, 5-bit counters, all blocks resident, checkpoints from 20% every 10%, tasks >= 128
    c = 10.0
    c -= 2.0 * (t["fetch_bytes"] == 16) + 0.5 * (t["counter_bits"] == 5) - 0.3 * (t["values_per_lane"] == 2)
    c += 0.7 * (t["blocks_per_sm"] == 1)
    c += 0.0 if t["early_exit_stages"] == 0 else abs(t["early_exit_first"] - 20) / 100 + t["early_exit_step"] / 1000
    c += 0.5 if t["early_exit_stages"] == 0 else 0.0
    c += abs(t["early_exit_min"] - 128) / 10000
    c -= 0.25 * (t["schedule"] == N.SCHEDULE_LEVELS)
    return c


def test_search_finds_the_minimum_over_all_stages():
    best, trials = tune_search(2, 4, cost)
    assert kernel(best) == (1, 16, 5) and best["blocks_per_sm"] == 0
    assert (best["early_exit_first"], best["early_exit_step"], best["early_exit_min"]) == (20, 10, 128)
    assert best["early_exit_stages"] == 8  # checkpoints 20, 30, ..., 90 percent
    assert best["schedule"] == N.SCHEDULE_LEVELS
    assert min(tr["kernel_ms"] for tr in trials) == pytest.approx(cost(best))
    # stage 1: all six kernels at two occupancies (the default adaptive schedule); then the level schedule with the
    # fastest; stage 2: ten fixed checkpoint schedules and the other adaptive step; stage 3: four minimums
    assert {kernel(tr) for tr in trials[:12]} == VARIANTS
    assert trials[12]["schedule"] == N.SCHEDULE_LEVELS and kernel(trials[12]) == (1, 16, 5)
    assert len(trials) == 12 + 1 + 11 + 4
    assert trials[0] == dict(best | dict(values_per_lane=1, fetch_bytes=8, counter_bits=7, early_exit_first=0,
                                         early_exit_step=32, early_exit_stages=N.EARLY_EXIT_ADAPTIVE,
                                         early_exit_min=256, schedule=N.SCHEDULE_QUEUE,
                                         level_values_per_lane=0),
                             kernel_ms=trials[0]["kernel_ms"])


def test_search_respects_what_the_hierarchy_admits():
    _, trials = tune_search(2, 1, cost)  # one-word rows: no 16-byte fetch
    assert {kernel(tr) for tr in trials} == {(1, 8, 7), (2, 8, 7), (1, 8, 5), (2, 8, 5)}
    for h, words in ((4, 1), (5, 4), (2, 8), (3, 16)):  # more hashes or wider rows: the default kernel only
        _, trials = tune_search(h, words, cost)
        assert {kernel(tr) for tr in trials} == {(1, 8, 7)}
        assert len(trials) == 2 + 1 + 11 + 4


def test_search_without_early_exit_skips_its_minimum():
    best, trials = tune_search(3, 4, lambda t: 1.0 if t["early_exit_stages"] == 0 else 2.0)
    assert best["early_exit_stages"] == 0
    # the level schedule, then its two values per lane below the root (the default kernel has one)
    assert len(trials) == 12 + 2 + 11  # no minimum-length stage when early exit is off
    assert trials[13]["schedule"] == N.SCHEDULE_LEVELS and trials[13]["level_values_per_lane"] == 2


def test_search_reports_measurement_failures():
    def boom(t):
        raise RuntimeError("device busy")

    with pytest.raises(RuntimeError, match="device busy"):
        tune_search(2, 4, boom)
    with pytest.raises(N.InvalidArgument):
        tune_search(6, 4, cost)
