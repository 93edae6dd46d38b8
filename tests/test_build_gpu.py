"""GPU build from a layout (hibf_gpu_hibf_build / _build_synthetic) against the reference's own builds.

For the layouts the reference computed (tests/golden), the device build must reproduce, for every IBF matched by its
path of merged bins: the bin count, bin size and bin-to-user-bin table, and the exact bit words (digest), split user
bins included (both builds chunk them in the reference's hash-set order, through a split table); query results are
also checked against the C oracle run on the downloaded bits.  The benchmark workloads are checked the same way at
reduced scale against the reference's own builds of them (tests/golden/ref_c3_*.npz, ref_c4_*.npz).
"""

import numpy as np
import pytest

import hibf_gb300 as hg
from hibf_gb300 import build as B
from hibf_gb300 import synthetic as S
from tests import golden_io as G
from tests.hibf_canon import canonical, split_free

pytestmark = pytest.mark.gpu


def _cfg(d, input_fn=None):
    h, tmax, sketch = (int(x) for x in d["config"])
    fpr, rfpr, alpha, ratio = (float(x) for x in d["fpr"])
    return B.config(input_fn=input_fn, number_of_user_bins=d["n_ub"], number_of_hash_functions=h, maximum_fpr=fpr,
                    relaxed_fpr=rfpr)


def _compare_with_reference(H, d, every_ibf=False):
    """Same IBFs (matched by path of merged bins), sizes and tables; bit stores equal for every IBF holding no split
    user bin, or for every IBF (`every_ibf`: builds that chunk split user bins in the reference's order)."""
    ref_t = G.tables(d)
    ref = canonical(ref_t)
    got = canonical(H.tables())
    assert set(ref) == set(got)
    n_exact = 0
    for path, (bins, size, row, k_ref) in ref.items():
        gb, gs, grow, k_got = got[path]
        assert (bins, size, row) == (gb, gs, grow), path
        if every_ibf or split_free(ref_t, k_ref):
            assert S.digest(H.words(k_got).tolist()) == int(d["digests"][k_ref]), path
            n_exact += 1
    return n_exact


def _queries_vs_oracle(H, oracle, d):
    t = H.tables()
    t["words"] = [H.words(k) for k in range(H.n_ibfs)]
    O = oracle.hibf(t)
    qv, qo = d["q_values"], d["q_offsets"]
    offs, ids, _ = H.membership_agent().query_batch(qv, qo, d["mem_t"])
    o_off, o_ids = O.membership_batch(qv, qo, d["mem_t"], threads=4)
    np.testing.assert_array_equal(offs, o_off)
    np.testing.assert_array_equal(ids, o_ids)


@pytest.mark.parametrize("name", ["synth64", "synth600", "synth_t128", "synth_t256"])
def test_build_synthetic_matches_reference(gpu_lib, oracle, name):
    d = G.hibf_case(name)
    seed = int(d["synthetic_seed"][0])
    H = B.build_synthetic(_cfg(d), d["layout_text"], seed, d["ub_offsets"])
    assert _compare_with_reference(H, d, every_ibf=True) == len(d["bins"])
    _queries_vs_oracle(H, oracle, d)
    # the same build from an exported and re-imported split table
    table = B.split_table.from_arrays(B.split_table.synthetic(_cfg(d), d["layout_text"], seed, d["ub_offsets"]).arrays())
    H2 = B.build_synthetic(_cfg(d), d["layout_text"], seed, d["ub_offsets"], table)
    np.testing.assert_array_equal(H2.digests(), H.digests())
    # no false negatives: every value of every user bin is counted in its user bin
    offs = d["ub_offsets"]
    ca = H.counting_agent(4)
    for ub in range(0, d["n_ub"], max(1, d["n_ub"] // 20)):
        v = S.user_bin_values(seed, offs, ub)
        assert int(ca.bulk_count(v, 1)[ub]) >= v.size


@pytest.mark.parametrize("name", ["snippet", "readme", "three_level", "uneven", "similar", "same", "simple", "synth64",
                                  "synth600", "synth_t128", "synth_t256"])
def test_build_input_fn_matches_reference(gpu_lib, oracle, name):
    """hierarchical_interleaved_bloom_filter(config&, layout) through input_fn: every IBF's bit store equals the
    reference's, split user bins included."""
    d = G.hibf_case(name)
    if "ub_values" in d:
        vals, offs = d["ub_values"], d["ub_offsets"]
        ubs = [vals[offs[u]:offs[u + 1]] for u in range(d["n_ub"])]
    else:
        seed = int(d["synthetic_seed"][0])
        ubs = [S.user_bin_values(seed, d["ub_offsets"], u) for u in range(d["n_ub"])]

    def input_fn(ub, it):
        it.push(ubs[ub])

    H = hg.hierarchical_interleaved_bloom_filter(_cfg(d, input_fn), d["layout_text"])
    assert _compare_with_reference(H, d, every_ibf=True) == len(d["bins"])
    _queries_vs_oracle(H, oracle, d)


def test_build_matches_reference_unit_expectations(gpu_lib):
    # hierarchical_interleaved_bloom_filter_test.cpp:112 three_level_hibf, built here from the reference's layout
    d = G.hibf_case("three_level")
    vals, offs = d["ub_values"], d["ub_offsets"]
    H = hg.hierarchical_interleaved_bloom_filter(
        _cfg(d, lambda ub, it: it.push(vals[offs[ub]:offs[ub + 1]])), d["layout_text"])
    a = H.membership_agent()
    for ub in range(0, 4096, 100):
        s = ub * 16
        a.membership_for(np.arange(s + 16, s + 20), 4)
        assert a.sort_results().tolist() == [ub, ub + 1]
        assert a.membership_for(np.arange(s + 5, s + 9), 4).tolist() == [ub]


def test_build_timers(gpu_lib, tmp_path):
    """The build's phase timers (hierarchical_interleaved_bloom_filter.hpp:283-290): an input_fn build reads every
    user bin once (one user_bin_io interval each, plus the upload of the distinct values), sizes unions and replays
    split orders (merge_kmers), allocates once and fills once; a synthetic build generates its values in the fill
    kernel (no user_bin_io) and replays split orders only without a table; a loaded HIBF holds no timers."""
    d = G.hibf_case("synth600")
    seed = int(d["synthetic_seed"][0])
    ubs = [S.user_bin_values(seed, d["ub_offsets"], u) for u in range(d["n_ub"])]

    def check(t, counts):
        assert {n: v["count"] for n, v in t.items()} == counts
        for n, v in t.items():
            assert v["seconds"] >= v["max_seconds"] >= 0.0, n
            assert (v["seconds"] > 0.0) == (v["count"] > 0), n

    H = hg.hierarchical_interleaved_bloom_filter(_cfg(d, lambda ub, it: it.push(ubs[ub])), d["layout_text"])
    check(H.build_timers(), dict(index_allocation=1, user_bin_io=d["n_ub"] + 1, merge_kmers=3, fill_ibf=1))
    cfg = _cfg(d)
    check(B.build_synthetic(cfg, d["layout_text"], seed, d["ub_offsets"]).build_timers(),
          dict(index_allocation=1, user_bin_io=0, merge_kmers=1, fill_ibf=1))
    table = B.split_table.synthetic(cfg, d["layout_text"], seed, d["ub_offsets"])
    check(B.build_synthetic(cfg, d["layout_text"], seed, d["ub_offsets"], table).build_timers(),
          dict(index_allocation=1, user_bin_io=0, merge_kmers=0, fill_ibf=1))
    H.save(tmp_path / "h.bin")
    L = hg.hierarchical_interleaved_bloom_filter.load(tmp_path / "h.bin")
    check(L.build_timers(), dict(index_allocation=0, user_bin_io=0, merge_kmers=0, fill_ibf=0))


def _digests_by_path(t, digests):
    return {path: int(digests[k]) for path, (_b, _s, _r, k) in canonical(t).items()}


def _same_index_as_reference(H, ref):
    """Every IBF of H (tables and bit words, matched by path of merged bins) equals the reference build `ref`."""
    rt = dict(bins=ref["bins"], bin_size=ref["bin_size"], next_ibf=ref["next_ibf"], user_bin=ref["user_bin"])
    want, got = canonical(rt), canonical(H.tables())
    assert {p: v[:3] for p, v in want.items()} == {p: v[:3] for p, v in got.items()}
    assert _digests_by_path(H.tables(), H.digests()) == _digests_by_path(rt, ref["digests"])


def test_c1_matches_reference(gpu_lib):
    """The 64-user-bin workload (h = 2, fpr 0.05, tmax 64; user bins of 1e3-1e5 values), built from the reference's layout both through input_fn and
    from the generator: every IBF holds the reference's bits, and all 10,000 queries answer as the reference did --
    membership_for + sort_results at t = 125 and counting_agent<uint16_t>::bulk_count at t = 125, compared per query
    by length and digest (hierarchical_interleaved_bloom_filter.hpp:424-439, 549-566)."""
    d = G.c1_reference()
    offs = d["ub_offsets"]
    cfg = B.config(number_of_user_bins=64, number_of_hash_functions=2, maximum_fpr=0.05)
    ubs = [S.user_bin_values(1, offs, u) for u in range(64)]
    H1 = hg.hierarchical_interleaved_bloom_filter(
        B.config(input_fn=lambda u, it: it.push(ubs[u]), number_of_user_bins=64, number_of_hash_functions=2,
                 maximum_fpr=0.05), d["layout_text"])
    H2 = B.build_synthetic(cfg, d["layout_text"], 1, offs)
    qv, qo, thr = d["q_values"], d["q_offsets"], d["thresholds"]
    for H in (H1, H2):
        _same_index_as_reference(H, d)
        m_off, m_ids, _ = H.membership_agent().query_batch(qv, qo, thr)
        mem_digest, mem_len = G.fold_digests(m_off, m_ids)
        np.testing.assert_array_equal(mem_len, d["mem_len"])
        np.testing.assert_array_equal(mem_digest, d["mem_digest"])
        c_off, c_ids, c_cnt = H.counting_agent(2).query_batch(qv, qo, thr)
        cnt_digest, cnt_nnz = G.fold_digests(c_off, c_ids, c_cnt)
        np.testing.assert_array_equal(cnt_nnz, d["cnt_nnz"])
        np.testing.assert_array_equal(cnt_digest, d["cnt_digest"])


@pytest.mark.parametrize("name,fixture", [("hibf8192", "ref_c3_0.05.npz"), ("hibf65536", "ref_c4_0.02.npz")])
def test_benchmark_layout_matches_reference_build(gpu_lib, name, fixture):
    """The benchmark workloads' layouts with every user bin at reduced scale: the device build (split user bins
    chunked by the replayed split table) equals the reference's own build of the same user bins in every IBF."""
    from hibf_gb300.workloads import WORKLOADS

    wl = WORKLOADS[name]
    ref = dict(np.load(G.GOLDEN / fixture))
    offs = ref["ub_offsets"]
    table, _ = wl.split_table(offs)
    cfg = B.config(number_of_user_bins=wl.n_user_bins, number_of_hash_functions=wl.h, maximum_fpr=wl.fpr)
    H = B.build_synthetic(cfg, wl.layout_text(), wl.query.seed, offs, table)
    _same_index_as_reference(H, ref)


@pytest.mark.parametrize("case", G.ibf_config_cases(), ids=lambda c: f"ibfcfg{c['index']}")
def test_ibf_from_config_matches_reference(gpu_lib, case):
    """interleaved_bloom_filter(config&, max_bin_elements): same bins, size, bit store, counts and memberships."""
    ubs = case["user_bins"]
    cfg = B.config(input_fn=lambda ub, it: it.push(ubs[ub]), **case["config"])
    ibf = B.ibf_from_config(cfg, case["max_bin_elements"])
    bins, size, h = (int(x) for x in case["params"])
    assert (ibf.bin_count(), ibf.bin_size(), ibf.hash_function_count()) == (bins, size, h)
    assert S.digest(ibf.words().tolist()) == int(case["digest"][0])
    q = case["queries"]
    np.testing.assert_array_equal(ibf.counting_agent(2).bulk_count(q), case["count2"])
    np.testing.assert_array_equal(ibf.membership_agent().membership_for(q[:200], 2), case["member"])


def test_ibf_from_config_unit_expectation(gpu_lib):
    """interleaved_bloom_filter_test.cpp:65-98 (construction_from_config): 2 is in both user bins, 8 only in the first,
    0 only in the second."""
    ubs = [list(range(1, 11)), [0, 2, 3, 4, 5]]
    ibf = B.ibf_from_config(B.config(input_fn=lambda ub, it: it.push(ubs[ub]), number_of_user_bins=2))
    agent = ibf.containment_agent()
    assert agent.bulk_contains(2).tolist() == [True, True]
    assert agent.bulk_contains(8).tolist() == [True, False]
    assert agent.bulk_contains(0).tolist() == [False, True]


def test_ibf_from_config_membership_for(gpu_lib):
    """interleaved_bloom_filter_test.cpp:410-431 (membership_for): querying 1..5 with threshold 2 hits both bins."""
    ubs = [list(range(1, 11)), list(range(1, 6))]
    ibf = B.ibf_from_config(B.config(input_fn=lambda ub, it: it.push(ubs[ub]), number_of_user_bins=2))
    got = ibf.membership_agent().membership_for(np.arange(1, 6, dtype=np.uint64), 2)
    assert got.tolist() == [0, 1]


@pytest.mark.parametrize("name", ["three_level", "uneven", "similar", "same", "synth600", "synth_t256", "dups",
                                  "synth_h4", "synth_h5"])
def test_device_set_materialisation_reproduces_reference_bits(gpu_lib, oracle, name):
    """With a device present the builder's front end materialises every user bin's distinct set (first-appearance
    order) and sizes the merged-bin unions by sorts on the device; the insertion order it returns must rebuild every
    IBF of the reference bit-exactly, split user bins and repeated values included (the same check the CPU test makes
    of the host front end)."""
    from tests.test_build_plan import test_insertion_order_reproduces_reference_bits as check

    check(oracle, name)
