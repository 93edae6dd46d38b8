"""GPU parity of the single-level IBF (interleaved_bloom_filter) through the C ABI.

Bit-exact against the reference's golden vectors (tests/golden/ibf_cases.npz), the reference's snippet/unit-test
known answers, and the C oracle on larger seeded cases.
"""

import numpy as np
import pytest

import hibf_gb300 as hg
from hibf_gb300 import synthetic as S
from tests import golden_io as G

pytestmark = pytest.mark.gpu


def _ibf(bins, bsz, h=2, track=False):
    return hg.interleaved_bloom_filter(hg.bin_count(bins), hg.bin_size(bsz), hg.hash_function_count(h), track)


@pytest.mark.parametrize("case", G.ibf_cases(), ids=lambda c: f"ibf{c['index']}")
def test_ibf_matches_reference_golden(gpu_lib, case):
    bins, bsz, h, track = (int(x) for x in case["params"])
    ibf = _ibf(bins, bsz, h, bool(track))
    ibf.emplace_many(case["values"], case["bins"])
    assert S.digest(ibf.words().tolist()) == int(case["digest"][0])
    q = case["queries"]
    np.testing.assert_array_equal(ibf.containment_agent().bulk_contains_words(q), case["contains"])
    for w in (1, 2, 4, 8):
        np.testing.assert_array_equal(ibf.counting_agent(w).bulk_count(q), case[f"count{w}"])
    for t in (0, 1, 2, 3, 50):
        np.testing.assert_array_equal(ibf.membership_agent().membership_for(q, t), case[f"member{t}"])
    ibf.clear(hg.bin_index(bins // 2))
    np.testing.assert_array_equal(ibf.counting_agent(4).bulk_count(q), case["after_clear"])
    ibf.clear([hg.bin_index(int(b)) for b in case["clear_range_bins"]])
    np.testing.assert_array_equal(ibf.counting_agent(4).bulk_count(q), case["after_clear_range"])
    ibf.increase_bin_number_to(hg.bin_count(int(case["widened_bins"][0])))
    assert S.digest(ibf.words().tolist()) == int(case["widened_digest"][0])
    np.testing.assert_array_equal(ibf.counting_agent(2).bulk_count(q), case["widened_count"])


def test_ibf_snippets_gpu(gpu_lib):
    # test/snippet/ibf/counting_agent.cpp/.out and interleaved_bloom_filter_clear.cpp/.out
    ibf = _ibf(8, 8192, 2)
    for v in range(0, 20):
        ibf.emplace(v, hg.bin_index(0))
    for v in range(10, 30):
        ibf.emplace(v, hg.bin_index(4))
    for v in range(25, 35):
        ibf.emplace(v, hg.bin_index(7))
    agent = ibf.counting_agent()
    assert agent.bulk_count(np.arange(20)).tolist() == [20, 0, 0, 0, 10, 0, 0, 0]
    assert agent.bulk_count([92, 1238, 812, 81273]).tolist() == [0] * 8
    assert agent.bulk_count(np.arange(1024)).tolist() == [20, 0, 0, 0, 20, 0, 0, 10]
    assert ibf.counting_agent(1).bulk_count(np.arange(20)).tolist() == [20, 0, 0, 0, 10, 0, 0, 0]
    ibf.clear(hg.bin_index(0))
    assert agent.bulk_count(np.arange(20)).tolist() == [0, 0, 0, 0, 10, 0, 0, 0]
    assert agent.bulk_count(np.arange(1024)).tolist() == [0, 0, 0, 0, 20, 0, 0, 10]
    ibf.clear([hg.bin_index(4), hg.bin_index(7)])
    assert agent.bulk_count(np.arange(1024)).tolist() == [0] * 8
    # membership_agent_membership_for.cpp/.out: [3,5,7]
    ibf = _ibf(12, 8192)
    q = [126, 712, 237]
    ibf.emplace(165, hg.bin_index(0))
    for v in q:
        ibf.emplace(v, hg.bin_index(3))
        ibf.emplace(v, hg.bin_index(5))
    ibf.emplace(126, hg.bin_index(7))
    ibf.emplace(712, hg.bin_index(7))
    ibf.emplace(956, hg.bin_index(9))
    assert ibf.membership_agent().membership_for(q, 2).tolist() == [3, 5, 7]
    # containment_agent_bulk_contains.cpp/.out and increase_bin_number_to.cpp/.out
    ibf = _ibf(12, 8192)
    ibf.emplace(126, hg.bin_index(0))
    ibf.emplace(712, hg.bin_index(3))
    ibf.emplace(237, hg.bin_index(9))
    assert ibf.containment_agent().bulk_contains(712).astype(int).tolist() == [0, 0, 0, 1] + [0] * 8
    ibf.increase_bin_number_to(hg.bin_count(18))
    a = ibf.containment_agent()
    assert a.bulk_contains(126).astype(int).tolist() == [1] + [0] * 17
    assert a.bulk_contains(237).astype(int).tolist() == [0] * 9 + [1] + [0] * 8
    # try_increase_bin_number_to.cpp/.out
    ibf = _ibf(73, 1024)
    assert ibf.try_increase_bin_number_to(hg.bin_count(73)) and ibf.bin_count() == 73
    assert not ibf.try_increase_bin_number_to(hg.bin_count(50)) and ibf.bin_count() == 73
    assert ibf.try_increase_bin_number_to(hg.bin_count(128)) and ibf.bin_count() == 128
    assert not ibf.try_increase_bin_number_to(hg.bin_count(129)) and ibf.bin_count() == 128


def test_ibf_errors_gpu(gpu_lib):
    with pytest.raises(hg.LogicError):
        _ibf(0, 1024)
    with pytest.raises(hg.LogicError):
        _ibf(8, 1024, 6)
    ibf = _ibf(8, 1024)
    with pytest.raises(hg.InvalidArgument):
        ibf.increase_bin_number_to(hg.bin_count(7))


@pytest.mark.parametrize("bins,bsz,h", [(1024, 1 << 16, 3), (64, 1 << 18, 2), (256, 50000, 3), (4096, 3000, 2)])
def test_ibf_large_vs_oracle(gpu_lib, oracle, bins, bsz, h):
    """Seeded larger filters: build on both sides from the same inserts; bit stores and query results equal."""
    rng = np.random.default_rng(bins * 7 + h)
    n_ins = 400_000
    vals = S.stream_range(bins, 0, n_ins)
    bns = rng.integers(0, bins, n_ins).astype(np.uint64)
    g = _ibf(bins, bsz, h)
    g.emplace_many(vals, bns)
    o = oracle.ibf(bins, bsz, h)
    o.emplace(vals, bns)
    np.testing.assert_array_equal(g.words(), o.words())
    q = np.concatenate([vals[::7][:50_000], S.stream_range(99, 0, 50_000)])
    np.testing.assert_array_equal(g.counting_agent(2).bulk_count(q), o.bulk_count(q, 2))
    np.testing.assert_array_equal(g.counting_agent(1).bulk_count(q), o.bulk_count(q, 1))
    np.testing.assert_array_equal(g.containment_agent().bulk_contains_words(q[:20_000]), o.bulk_contains(q[:20_000]))


def test_ibf_empty_and_ragged_inputs(gpu_lib, oracle):
    ibf = _ibf(100, 999, 3)
    assert ibf.counting_agent().bulk_count(np.zeros(0, np.uint64)).tolist() == [0] * 100
    assert ibf.membership_agent().membership_for(np.zeros(0, np.uint64), 0).tolist() == list(range(100))
    assert ibf.membership_agent().membership_for(np.zeros(0, np.uint64), 1).tolist() == []
    o = oracle.ibf(100, 999, 3)
    for n in (1, 31, 32, 33, 127, 128, 129, 1000):
        v = S.stream_range(n, 0, n)
        ibf.emplace_many(v, n % 100)
        o.emplace(v, np.full(n, n % 100, np.uint64))
        np.testing.assert_array_equal(ibf.counting_agent().bulk_count(v), o.bulk_count(v, 2))


@pytest.mark.parametrize("binned", [False, True])
def test_occupancy_in_insertion_order(gpu_lib, oracle, binned):
    """track_occupancy counts a value when one of its bits was not set yet, in insertion order (the reference's
    sequential emplace); a small filter makes values of a bin share bits, and a 3e6-value call spans chunks."""
    rng = np.random.default_rng(12)
    bins, size = 70, 64
    ibf = _ibf(bins, size, 3, True)
    O = oracle.ibf(bins, size, 3, True)
    assert ibf.track_occupancy and not _ibf(bins, size, 3, False).track_occupancy
    for n in (5, 1000, 3_000_000):
        v = rng.integers(0, 1 << 62, n, dtype=np.uint64)
        if binned:
            b = rng.integers(0, bins, n).astype(np.uint64)
            ibf.emplace_many(v, b)
            O.emplace(v, b)
        else:
            ibf.emplace_many(v, np.full(n, 7, np.uint64))
            O.emplace(v, 7)
        np.testing.assert_array_equal(ibf.occupancy, O.occupancy())
    np.testing.assert_array_equal(ibf.words(), O.words())
