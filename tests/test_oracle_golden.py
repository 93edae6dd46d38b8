"""Pins the C restatement (oracle/hibf_oracle.c) against the reference's own outputs and known answers.

CPU only.  Golden vectors come from the reference itself (tests/golden/make_golden.py); the known answers are the
expectations of the reference's unit tests and documentation snippets:
  test/unit/hibf/interleaved_bloom_filter_test.cpp, test/unit/hibf/hierarchical_interleaved_bloom_filter_test.cpp,
  test/unit/hibf/counting_vector_test.cpp, test/snippet/**/*.out
"""

import numpy as np
import pytest

from hibf_gb300 import synthetic as S
from tests import golden_io as G


def _build_ibf(oracle, c):
    bins, bsz, h, track = (int(x) for x in c["params"])
    ibf = oracle.ibf(bins, bsz, h, bool(track))
    ibf.emplace(c["values"], c["bins"])
    return ibf


@pytest.mark.parametrize("case", G.ibf_cases(), ids=lambda c: f"ibf{c['index']}")
def test_ibf_case_matches_reference(oracle, case):
    ibf = _build_ibf(oracle, case)
    assert S.digest(ibf.words().tolist()) == int(case["digest"][0])
    q = case["queries"]
    np.testing.assert_array_equal(ibf.bulk_contains(q), case["contains"])
    for w in (1, 2, 4, 8):
        np.testing.assert_array_equal(ibf.bulk_count(q, w), case[f"count{w}"])
    for t in (0, 1, 2, 3, 50):
        np.testing.assert_array_equal(ibf.membership_for(q, t), case[f"member{t}"])
    bins = int(case["params"][0])
    ibf.clear(bins // 2)
    np.testing.assert_array_equal(ibf.bulk_count(q, 4), case["after_clear"])
    ibf.clear_range(case["clear_range_bins"])
    np.testing.assert_array_equal(ibf.bulk_count(q, 4), case["after_clear_range"])
    ibf.increase_bin_number_to(int(case["widened_bins"][0]))
    assert S.digest(ibf.words().tolist()) == int(case["widened_digest"][0])
    np.testing.assert_array_equal(ibf.bulk_count(q, 2), case["widened_count"])


def test_ibf_unit_known_answers(oracle):
    # interleaved_bloom_filter_test.cpp:296-331 counting: 128 bins x 128 values -> 128 per bin
    ibf = oracle.ibf(128, 1024, 2)
    vals = np.tile(np.arange(128, dtype=np.uint64), 128)
    ibf.emplace(vals, np.repeat(np.arange(128, dtype=np.uint64), 128))
    np.testing.assert_array_equal(ibf.bulk_count(np.arange(128), 8), np.full(128, 128))
    # :181 emplace -> every hash in every bin
    ibf = oracle.ibf(64, 1024, 2)
    ibf.emplace(np.tile(np.arange(64, dtype=np.uint64), 64), np.repeat(np.arange(64, dtype=np.uint64), 64))
    assert (ibf.bulk_contains(np.arange(64)) == np.uint64(2**64 - 1)).all()
    # :241 clear bin 17
    ibf.clear(17)
    w = ibf.bulk_contains(np.arange(64))
    assert ((w >> np.uint64(17)) & np.uint64(1) == 0).all()
    # :355 counting_no_ub (bins 63 and 127) and :383 with 127 bins
    for bins, ub in ((128, (63, 127)), (127, (63, 126))):
        ibf = oracle.ibf(bins, 1024, 2)
        for b in ub:
            ibf.emplace(np.arange(128, dtype=np.uint64), b)
        exp = np.zeros(bins, np.uint64)
        exp[list(ub)] = 128
        np.testing.assert_array_equal(ibf.bulk_count(np.arange(128), 8), exp)
    # :145 empty filter
    assert (oracle.ibf(64, 1024, 2).bulk_contains(np.arange(64)) == 0).all()


def test_ibf_snippets(oracle):
    # test/snippet/ibf/counting_agent.cpp/.out
    ibf = oracle.ibf(8, 8192, 2)
    ibf.emplace(np.arange(0, 20), 0)
    ibf.emplace(np.arange(10, 30), 4)
    ibf.emplace(np.arange(25, 35), 7)
    assert ibf.bulk_count(np.arange(20)).tolist() == [20, 0, 0, 0, 10, 0, 0, 0]
    assert ibf.bulk_count([92, 1238, 812, 81273]).tolist() == [0] * 8
    assert ibf.bulk_count(np.arange(1024)).tolist() == [20, 0, 0, 0, 20, 0, 0, 10]
    assert ibf.bulk_count(np.arange(20), 1).tolist() == [20, 0, 0, 0, 10, 0, 0, 0]
    # test/snippet/ibf/interleaved_bloom_filter_clear.cpp/.out
    ibf.clear(0)
    assert ibf.bulk_count(np.arange(20)).tolist() == [0, 0, 0, 0, 10, 0, 0, 0]
    assert ibf.bulk_count(np.arange(1024)).tolist() == [0, 0, 0, 0, 20, 0, 0, 10]
    ibf.clear_range([4, 7])
    assert ibf.bulk_count(np.arange(1024)).tolist() == [0] * 8
    # test/snippet/ibf/membership_agent_membership_for.cpp/.out
    ibf = oracle.ibf(12, 8192, 2)
    q = [126, 712, 237]
    ibf.emplace([165], 0)
    ibf.emplace(q, 3)
    ibf.emplace(q, 5)
    ibf.emplace([126, 712], 7)
    ibf.emplace([956], 9)
    assert ibf.membership_for(q, 2).tolist() == [3, 5, 7]
    # test/snippet/ibf/containment_agent_bulk_contains.cpp and increase_bin_number_to.cpp
    ibf = oracle.ibf(12, 8192, 2)
    ibf.emplace([126], 0)
    ibf.emplace([712], 3)
    ibf.emplace([237], 9)
    assert int(ibf.bulk_contains([712])[0, 0]) == 1 << 3
    ibf.increase_bin_number_to(18)
    assert [int(x) for x in ibf.bulk_contains([126, 712, 237])[:, 0]] == [1, 8, 512]
    # try_increase_bin_number_to snippet: 73 -> 73 true, 50 false, 128 true, 129 false
    ibf = oracle.ibf(73, 1024, 2)
    assert ibf.try_increase_bin_number_to(73) and ibf.bins == 73
    assert not ibf.try_increase_bin_number_to(50) and ibf.bins == 73
    assert ibf.try_increase_bin_number_to(128) and ibf.bins == 128
    assert not ibf.try_increase_bin_number_to(129) and ibf.bins == 128


def test_counting_wraparound(oracle):
    # counting_vector_test.cpp:172-190: counters wrap modulo 2^bits
    ibf = oracle.ibf(64, 256, 1)
    ibf.emplace([7], 5)
    q = np.full(300, 7, np.uint64)
    assert int(ibf.bulk_count(q, 1)[5]) == 300 - 256
    assert int(ibf.bulk_count(q, 2)[5]) == 300
    q = np.full(70000, 7, np.uint64)
    assert int(ibf.bulk_count(q, 2)[5]) == 70000 - 65536


def test_ibf_invalid_arguments(oracle):
    # IBF.cpp:41-46 logic errors
    for args in ((0, 10, 2), (8, 10, 0), (8, 10, 6), (8, 0, 2)):
        with pytest.raises(ValueError):
            oracle.ibf(*args)
    ibf = oracle.ibf(8, 10, 2)
    with pytest.raises(ValueError):
        ibf.increase_bin_number_to(7)


@pytest.mark.parametrize("name", G.HIBF_CASES)
def test_hibf_case_matches_reference(oracle, name):
    d = G.hibf_case(name)
    H = oracle.hibf(G.tables(d))
    qs = G.queries(d)
    unsorted = G.mem_lists(d, "mem_unsorted")
    sorted_ = G.mem_lists(d, "mem_sorted")
    widths = [w for w in (1, 2, 4, 8) if f"count{w}" in d]
    for i, q in enumerate(qs):
        np.testing.assert_array_equal(H.membership_for(q, int(d["mem_t"][i]), sort=False), unsorted[i])
        np.testing.assert_array_equal(H.membership_for(q, int(d["mem_t"][i]), sort=True), sorted_[i])
        for w in widths:
            np.testing.assert_array_equal(H.bulk_count(q, int(d["cnt_t"][i]), w), d[f"count{w}"][i])


def test_hibf_unit_expectations(oracle):
    # hierarchical_interleaved_bloom_filter_test.cpp:23-45 and :297-332 (copy_agents)
    d = G.hibf_case("snippet")
    H = oracle.hibf(G.tables(d))
    assert H.membership_for([1, 2, 3, 4, 5], 2).tolist() == [0, 1]
    assert H.membership_for([1, 2, 3, 4, 5], 6).tolist() == []
    assert H.bulk_count([1, 2, 3, 4, 5], 1).tolist() == [5, 5]
    assert H.bulk_count([1, 2, 3, 4, 5], 6).tolist() == [0, 0]
    # test/snippet/readme.cpp/.out: "2 0" unsorted, then "0 1" sorted
    d = G.hibf_case("readme")
    H = oracle.hibf(G.tables(d))
    assert H.membership_for([3, 9, 12, 14], 2, sort=False).tolist() == [2, 0]
    assert H.membership_for(np.arange(15), 5, sort=True).tolist() == [0, 1]
    # :112 three_level: overlap query -> {ub, ub+1}; unique query -> {ub}
    d = G.hibf_case("three_level")
    H = oracle.hibf(G.tables(d))
    assert d["bins"].size > 64 + 1  # three levels
    for ub in range(0, 4096, 100):
        s = ub * 16
        assert H.membership_for(np.arange(s + 16, s + 20), 4).tolist() == [ub, ub + 1]
        assert H.membership_for(np.arange(s + 5, s + 9), 4).tolist() == [ub]
    # :233 counting_agent_same_bins: 500 <= count <= 502
    d = G.hibf_case("same")
    H = oracle.hibf(G.tables(d))
    c = H.bulk_count(np.arange(500), 1, 4)
    assert (c >= 500).all() and (c <= 502).all()
    # :264 counting_agent_different_bins: count >= size of the user bin
    d = G.hibf_case("uneven")
    H = oracle.hibf(G.tables(d))
    c = H.bulk_count(np.arange(1, 251000), 1, 4)
    assert all(int(c[ub]) >= 2 * ub + 2 for ub in range(500))


def test_c1_oracle_answers_like_the_reference(oracle):
    """The 64-user-bin workload (h = 2, fpr 0.05, tmax 64; user bins of 1e3-1e5 values): the oracle's HIBF with the reference's tables, filled in the
    builder's insertion order, holds the reference's bits in every IBF, and answers all 10,000 queries
    (membership_for + sort_results at t = 125, counting_agent<uint16_t>::bulk_count at t = 125) with the
    reference's per-query lengths and digests (hierarchical_interleaved_bloom_filter.hpp:424-439, 549-566)."""
    from hibf_gb300 import build as B
    from hibf_gb300 import synthetic as S

    d = G.c1_reference()
    offs = d["ub_offsets"]
    ubs = [S.user_bin_values(1, offs, u) for u in range(64)]
    cfg = B.config(input_fn=lambda u, it: it.push(ubs[u]), number_of_user_bins=64, number_of_hash_functions=2,
                   maximum_fpr=0.05)
    o2, vals = B.build_inputs(cfg, d["layout_text"])
    t = dict(n_user_bins=64, bins=d["bins"], bin_size=d["bin_size"], hash_funs=d["hash_funs"],
             next_ibf=d["next_ibf"], user_bin=d["user_bin"])
    O = G.oracle_hibf_from_inputs(oracle, t, o2, vals)
    for k in range(d["bins"].size):
        assert S.digest(O.words(k).tolist()) == int(d["digests"][k]), f"IBF {k}"
    r = O.query_batch(d["q_values"], d["q_offsets"], d["thresholds"], d["thresholds"], threads=4)
    for key in ("mem_len", "mem_digest", "cnt_nnz", "cnt_digest"):
        np.testing.assert_array_equal(r[key], d[key], err_msg=key)


def test_c1_reference_fixture_shape():
    z = np.load(G.GOLDEN / "c1_reference.npz")
    assert z["bins"].size == 3 and z["mem_len"].size == 10000
    layout = bytes(z["layout"]).decode()
    assert layout.startswith("#TOP_LEVEL_IBF fullest_technical_bin_idx:")
