"""GPU parity of the HIBF query path (membership_for / bulk_count) through the C ABI.

The HIBFs here were built by the reference itself (tables + bit words in tests/golden/hibf_*.npz); the GPU answers
every stored query and must reproduce the reference's outputs bit-exactly: traversal-order and sorted membership
lists, and dense counting vectors for uint8/uint16/uint32/uint64 counters (wraparound included).  The batched
persistent launch, the plain one-launch-per-query form and the single-query agent calls must all agree.
"""

import ctypes

import numpy as np
import pytest

import hibf_gb300 as hg
from hibf_gb300 import _native as N
from tests import golden_io as G

pytestmark = pytest.mark.gpu


def _gpu_hibf(d):
    t = G.tables(d)
    return hg.hierarchical_interleaved_bloom_filter.from_tables(t["n_user_bins"], t["bins"], t["bin_size"],
                                                                t["hash_funs"], t["next_ibf"], t["user_bin"],
                                                                words=t["words"])


def _split(offs, ids):
    return [ids[offs[i]:offs[i + 1]] for i in range(offs.size - 1)]


@pytest.mark.parametrize("mode", ["warp", "block"])
@pytest.mark.parametrize("name", G.HIBF_CASES)
def test_hibf_batch_matches_reference(gpu_lib, name, mode):
    """Every golden HIBF's queries, one task per warp and one task per block of eight warps (latency mode)."""
    d = G.hibf_case(name)
    H = _gpu_hibf(d)
    for k, w in enumerate(G.tables(d)["words"]):
        np.testing.assert_array_equal(H.words(k), w)
    agent = H.membership_agent()
    agent.tuning = dict(agent.tuning, block_queries=0 if mode == "warp" else 1 << 30)
    qv, qo = d["q_values"], d["q_offsets"]
    offs, ids, _ = agent.query_batch(qv, qo, d["mem_t"], mode=N.QUERY_MEMBERSHIP)
    got = _split(offs, ids)
    exp = G.mem_lists(d, "mem_sorted")
    assert len(got) == len(exp)
    for i, (g, e) in enumerate(zip(got, exp)):
        np.testing.assert_array_equal(g, e, err_msg=f"query {i}")
    for w in (1, 2, 4, 8):
        if f"count{w}" not in d:
            continue
        offs, ids, cnts = agent.query_batch(qv, qo, d["cnt_t"], mode=N.QUERY_COUNT, width=w)
        dense = np.zeros_like(d[f"count{w}"])
        for i in range(offs.size - 1):
            dense[i, ids[offs[i]:offs[i + 1]].astype(np.int64)] = cnts[offs[i]:offs[i + 1]]
        np.testing.assert_array_equal(dense, d[f"count{w}"])


@pytest.mark.parametrize("name", ["snippet", "readme", "three_level", "uneven", "similar", "synth64", "synth600",
                                  "synth_t256", "dups"])
def test_hibf_single_query_agents_match_reference(gpu_lib, name):
    d = G.hibf_case(name)
    H = _gpu_hibf(d)
    ma = H.membership_agent()
    unsorted = G.mem_lists(d, "mem_unsorted")
    qs = G.queries(d)
    for i, q in enumerate(qs[:60]):
        np.testing.assert_array_equal(ma.membership_for(q, int(d["mem_t"][i])), unsorted[i])
        np.testing.assert_array_equal(ma.sort_results(), np.sort(unsorted[i]))
    widths = [w for w in (1, 2, 4, 8) if f"count{w}" in d]
    for w in widths:
        ca = H.counting_agent(w)
        for i, q in enumerate(qs[:30]):
            np.testing.assert_array_equal(ca.bulk_count(q, int(d["cnt_t"][i])), d[f"count{w}"][i])


def test_readme_snippet_gpu(gpu_lib):
    # test/snippet/readme.out: "2 0" (unsorted), then "0 1" (sorted)
    H = _gpu_hibf(G.hibf_case("readme"))
    a = H.membership_agent()
    assert a.membership_for([3, 9, 12, 14], 2).tolist() == [2, 0]
    a.membership_for(np.arange(15), 5)
    assert a.sort_results().tolist() == [0, 1]
    # hierarchical_interleaved_bloom_filter_test.cpp copy_agents: counts {5,5} / {0,0}
    H = _gpu_hibf(G.hibf_case("snippet"))
    assert H.counting_agent().bulk_count([1, 2, 3, 4, 5], 1).tolist() == [5, 5]
    assert H.counting_agent().bulk_count([1, 2, 3, 4, 5], 6).tolist() == [0, 0]


@pytest.mark.parametrize("name", ["three_level", "synth600"])
def test_plain_form_equals_batch(gpu_lib, name):
    import torch

    d = G.hibf_case(name)
    H = _gpu_hibf(d)
    a = H.membership_agent()
    qv, qo = d["q_values"], d["q_offsets"]
    offs_b, ids_b, _ = a.query_batch(qv, qo, d["mem_t"])
    dv = torch.from_numpy(qv.view(np.int64)).cuda()
    torch.cuda.synchronize()
    a.query_plain_device(dv.data_ptr(), qo, d["mem_t"])
    offs_p, ids_p, _ = a.fetch_results(qo.size - 1)
    np.testing.assert_array_equal(offs_b, offs_p)
    np.testing.assert_array_equal(ids_b, ids_p)


def test_batch_vs_oracle_many_thresholds(gpu_lib, oracle):
    """Every threshold from 0 (descend everywhere) upwards on the 600-user-bin HIBF, against the C oracle."""
    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    O = oracle.hibf(G.tables(d))
    qs = G.queries(d)
    vals = np.concatenate(qs[:100])
    qo = np.zeros(101, np.uint64)
    np.cumsum([q.size for q in qs[:100]], out=qo[1:])
    for t in (0, 1, 2, 5, 20):
        thr = np.full(100, t, np.uint64)
        offs, ids, _ = H.membership_agent().query_batch(vals, qo, thr)
        o_off, o_ids = O.membership_batch(vals, qo, thr, threads=4)
        np.testing.assert_array_equal(offs, o_off)
        np.testing.assert_array_equal(ids, o_ids)


def test_empty_queries_and_empty_batch(gpu_lib):
    d = G.hibf_case("synth64")
    H = _gpu_hibf(d)
    a = H.membership_agent()
    qo = np.array([0, 0, 0], np.uint64)
    offs, ids, _ = a.query_batch(np.zeros(0, np.uint64), qo, [0, 1])
    # threshold 0 with no values: every user bin reaches 0 >= 0, as in the reference
    assert int(offs[1] - offs[0]) == d["n_ub"] and int(offs[2] - offs[1]) == 0
    offs, ids, _ = a.query_batch(np.zeros(0, np.uint64), np.array([0], np.uint64), np.zeros(0, np.uint64))
    assert offs.tolist() == [0] and ids.size == 0


def test_invalid_thresholds(gpu_lib):
    H = _gpu_hibf(G.hibf_case("snippet"))
    a = H.membership_agent()
    with pytest.raises(hg.InvalidArgument):
        a.query_batch([1, 2], [0, 2], [70000])
    with pytest.raises(hg.InvalidArgument):
        a.query_batch([1, 2], [0, 2], [0], mode=N.QUERY_COUNT)


def test_large_batch_checks_every_slice(gpu_lib):
    """A large batch's host checks run in slices on several threads: a decreasing offset or a bad threshold in the
    last slice is still an invalid argument, and a valid batch of the same size answers."""
    H = _gpu_hibf(G.hibf_case("snippet"))
    a = H.membership_agent()
    nq = 300_000
    qo = np.zeros(nq + 1, np.uint64)  # every query empty
    thr = np.ones(nq, np.uint64)
    offs, ids, _ = a.query_batch(np.zeros(0, np.uint64), qo, thr)
    assert offs.size == nq + 1 and ids.size == 0
    bad = qo.copy()
    bad[-2] = 5  # qoff[nq - 1] > qoff[nq]
    with pytest.raises(hg.InvalidArgument, match="non-decreasing"):
        a.query_batch(np.zeros(5, np.uint64), bad, thr)
    t = thr.copy()
    t[-1] = 70000
    with pytest.raises(hg.InvalidArgument, match="uint16"):
        a.query_batch(np.zeros(0, np.uint64), qo, t)
    t[-1] = 0
    with pytest.raises(hg.InvalidArgument, match="> 0"):
        a.query_batch(np.zeros(0, np.uint64), qo, t, mode=N.QUERY_COUNT)
    offs, ids, _ = a.query_batch(np.zeros(0, np.uint64), qo, thr)  # the agent still answers
    assert offs.size == nq + 1 and ids.size == 0


def test_work_counters(gpu_lib):
    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    a = H.membership_agent()
    qv, qo = d["q_values"], d["q_offsets"]
    a.query_batch(qv, qo, d["mem_t"])
    tasks, visits = a.last_work()
    assert tasks >= qo.size - 1
    assert visits >= int(qo[-1])


KERNELS = [(1, 8, 7), (2, 8, 7), (1, 8, 5), (2, 8, 5), (1, 16, 7), (1, 16, 5)]
EARLY_EXIT = [dict(early_exit_first=30, early_exit_step=10, early_exit_stages=7, early_exit_min=256),
              dict(early_exit_stages=0),
              dict(early_exit_first=10, early_exit_step=10, early_exit_stages=9, early_exit_min=16),
              dict(early_exit_first=0, early_exit_step=32, early_exit_stages=N.EARLY_EXIT_ADAPTIVE, early_exit_min=16),
              dict(early_exit_first=0, early_exit_step=1, early_exit_stages=N.EARLY_EXIT_ADAPTIVE, early_exit_min=1)]


@pytest.mark.parametrize("name", ["synth600", "synth_t128", "synth_t256"])
def test_every_schedule_gives_the_reference_results(gpu_lib, name):
    """Each kernel variant (values per lane, fetch width, counter width) and early-exit schedule: bit-exact
    membership lists and uint16 counts against the reference."""
    d = G.hibf_case(name)
    H = _gpu_hibf(d)
    a = H.membership_agent()
    qv, qo = d["q_values"], d["q_offsets"]
    exp = G.mem_lists(d, "mem_sorted")
    for vpl, fb, cb in KERNELS:
        for ee in EARLY_EXIT:
            for bps in (0, 1):
                a.tuning = dict(values_per_lane=vpl, fetch_bytes=fb, counter_bits=cb, blocks_per_sm=bps,
                                block_queries=0, **ee)
                offs, ids, _ = a.query_batch(qv, qo, d["mem_t"])
                got = _split(offs, ids)
                for i, (g, e) in enumerate(zip(got, exp)):
                    np.testing.assert_array_equal(g, e, err_msg=f"{(vpl, fb, cb, bps, ee)} query {i}")
        offs, ids, cnts = a.query_batch(qv, qo, d["cnt_t"], mode=N.QUERY_COUNT, width=2)
        dense = np.zeros_like(d["count2"])
        for i in range(offs.size - 1):
            dense[i, ids[offs[i]:offs[i + 1]].astype(np.int64)] = cnts[offs[i]:offs[i + 1]]
        np.testing.assert_array_equal(dense, d["count2"], err_msg=str((vpl, fb, cb)))


def test_tuning_validation(gpu_lib):
    a = _gpu_hibf(G.hibf_case("synth_t256")).membership_agent()
    default = a.tuning
    for bad in (dict(values_per_lane=2, fetch_bytes=16), dict(counter_bits=6), dict(blocks_per_sm=33),
                dict(early_exit_first=95, early_exit_step=10, early_exit_stages=2),
                dict(early_exit_first=0, early_exit_stages=3)):
        with pytest.raises(hg.InvalidArgument):
            a.tuning = dict(default, **bad)
    assert a.tuning == default


@pytest.mark.parametrize("name", ["synth600", "synth_t256"])
def test_autotune_keeps_the_fastest_and_the_results(gpu_lib, name):
    import torch

    d = G.hibf_case(name)
    H = _gpu_hibf(d)
    a = H.membership_agent()
    qv, qo, t = d["q_values"], d["q_offsets"], d["mem_t"]
    dv = torch.from_numpy(qv.view(np.int64)).cuda()
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(t.astype(np.uint64).view(np.int64)).cuda()
    torch.cuda.synchronize()
    trials = a.autotune(dv.data_ptr(), dq.data_ptr(), qo.size - 1, dt.data_ptr(), reps=1)
    assert len(trials) >= 12
    best = min(trials, key=lambda tr: tr["kernel_ms"])
    assert a.tuning == {k: v for k, v in best.items() if k != "kernel_ms"}
    offs, ids, _ = a.query_batch(qv, qo, t)
    for i, (g, e) in enumerate(zip(_split(offs, ids), G.mem_lists(d, "mem_sorted"))):
        np.testing.assert_array_equal(g, e, err_msg=f"query {i}")


def test_claim_order_work_counters_and_features(gpu_lib):
    """A permuted claim order gives the same results; per-query work sums to the batch's executed visits; the
    scheduler's features are well-formed."""
    import torch

    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    a = H.membership_agent()
    qv, qo, t = d["q_values"], d["q_offsets"], d["mem_t"]
    nq = qo.size - 1
    dv = torch.from_numpy(qv.view(np.int64)).cuda()
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(t.astype(np.uint64).view(np.int64)).cuda()
    perm = np.random.default_rng(1).permutation(nq).astype(np.uint32)
    dperm = torch.from_numpy(perm.view(np.int32)).cuda()
    work = torch.zeros(nq, dtype=torch.int64, device="cuda")
    a.set_work_out(work.data_ptr(), nq)
    a.set_order(dperm.data_ptr(), nq)
    offs, ids, _ = a.query_batch(qv, qo, t)
    for i, (g, e) in enumerate(zip(_split(offs, ids), G.mem_lists(d, "mem_sorted"))):
        np.testing.assert_array_equal(g, e, err_msg=f"query {i}")
    w = work.cpu().numpy().view(np.uint64)
    assert int(w.sum()) == a.last_work_executed()
    assert np.all(w >= np.minimum(np.diff(qo), 1))  # every query reads at least one value at the root (if any)
    bad = perm.copy()
    bad[5] = nq + 7
    dbad = torch.from_numpy(bad.view(np.int32)).cuda()
    a.set_order(dbad.data_ptr(), nq)
    with pytest.raises(hg.InvalidArgument):
        a.query_batch(qv, qo, t)
    a.set_order(dperm.data_ptr(), nq - 1)
    with pytest.raises(hg.InvalidArgument, match="different length"):
        a.query_batch(qv, qo, t)
    a.set_order(None)
    a.set_work_out(None)
    offs, ids, _ = a.query_batch(qv, qo, t)
    assert np.array_equal(_split(offs, ids)[-1], G.mem_lists(d, "mem_sorted")[-1])
    feats = torch.zeros(nq * 6, dtype=torch.float32, device="cuda")
    a.query_features(dv.data_ptr(), dq.data_ptr(), nq, dt.data_ptr(), 16, feats.data_ptr())
    torch.cuda.synchronize()
    f = feats.cpu().numpy().reshape(nq, 6)
    n = np.diff(qo).astype(np.float64)
    np.testing.assert_allclose(f[:, 0], np.log2(1 + n) / 16, rtol=1e-6)
    np.testing.assert_allclose(f[:, 5], np.minimum(n, 16) / 16, rtol=1e-6)
    assert np.all((f[:, 2] >= 0) & (f[:, 2] <= 1)) and np.all((f[:, 3] >= 0) & (f[:, 3] <= 1))


@pytest.mark.parametrize("name", G.HIBF_CASES)
@pytest.mark.parametrize("schedule", ["fixed", "adaptive"])
def test_early_decisions_on_every_case(gpu_lib, name, schedule):
    """Checkpoints after every 10% of every task's values, or adaptive checks at most one value apart (no minimum
    length): the hopeless and the decided exits fire as often as they can, and membership lists and counts stay the
    reference's."""
    d = G.hibf_case(name)
    H = _gpu_hibf(d)
    a = H.membership_agent()
    if schedule == "fixed":
        a.tuning = dict(a.tuning, block_queries=0, early_exit_first=10, early_exit_step=10, early_exit_stages=9,
                        early_exit_min=1)
    else:
        a.tuning = dict(a.tuning, block_queries=0, early_exit_first=0, early_exit_step=1,
                        early_exit_stages=N.EARLY_EXIT_ADAPTIVE, early_exit_min=1)
    qv, qo = d["q_values"], d["q_offsets"]
    offs, ids, _ = a.query_batch(qv, qo, d["mem_t"])
    for i, (g, e) in enumerate(zip(_split(offs, ids), G.mem_lists(d, "mem_sorted"))):
        np.testing.assert_array_equal(g, e, err_msg=f"query {i}")
    w = 2 if "count2" in d else 8
    offs, ids, cnts = a.query_batch(qv, qo, d["cnt_t"], mode=N.QUERY_COUNT, width=w)
    dense = np.zeros_like(d[f"count{w}"])
    for i in range(offs.size - 1):
        dense[i, ids[offs[i]:offs[i + 1]].astype(np.int64)] = cnts[offs[i]:offs[i + 1]]
    np.testing.assert_array_equal(dense, d[f"count{w}"])


def _long_batch(d, n_queries, rng, odd=True):
    """n_queries queries cut from the golden queries' values, lengths in [301, 799] (odd lengths when `odd`)."""
    qs = [q for q in G.queries(d) if q.size]
    lens = rng.integers(150, 400, n_queries) * 2 + (1 if odd else 0)
    parts = []
    for i, n in enumerate(lens):
        q = qs[i % len(qs)]
        parts.append(np.resize(q, int(n)))
    qo = np.zeros(n_queries + 1, np.uint64)
    np.cumsum(lens, out=qo[1:])
    thr = np.floor(lens * rng.uniform(0.3, 0.8, n_queries)).astype(np.uint64)
    return np.concatenate(parts).astype(np.uint64), qo, thr


def test_streamed_host_batch_equals_resident_batch(gpu_lib, oracle):
    """A host batch of at least 64 MiB of values is copied in chunks while the kernel answers the chunks already
    copied.  Its results equal the device-resident batch's and the oracle's, for odd query lengths (chunks start only
    where a query's first value starts a 32-byte sector) and for counts as well as membership."""
    import torch

    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    rng = np.random.default_rng(11)
    vals, qo, thr = _long_batch(d, 24000, rng)
    assert vals.size * 8 >= 64 << 20
    a = H.membership_agent()
    offs, ids, _ = a.query_batch(vals, qo, thr)
    assert a.input_chunks() > 2
    dv = torch.from_numpy(vals.view(np.int64)).cuda()
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(thr.view(np.int64)).cuda()
    r = H.membership_agent()
    nq = qo.size - 1
    r.reserve(nq, vals.size, nq * 8 + 65536, nq * 16 + 65536)
    r.query_batch_device(dv.data_ptr(), dq.data_ptr(), nq, dt.data_ptr())
    offs_r, ids_r, _ = r.fetch_results(nq)
    np.testing.assert_array_equal(offs, offs_r)
    np.testing.assert_array_equal(ids, ids_r)
    O = oracle.hibf(G.tables(d))
    o_off, o_ids = O.membership_batch(vals, qo, thr, threads=8)
    np.testing.assert_array_equal(offs, o_off)
    np.testing.assert_array_equal(ids, o_ids)
    c = H.counting_agent(2)
    cthr = np.maximum(thr, 1)
    c_offs, c_ids, c_cnt = c.query_batch(vals, qo, cthr, mode=N.QUERY_COUNT, width=2)
    assert c.input_chunks() > 2
    c.reserve(nq, vals.size, nq * 8 + 65536, nq * 16 + 65536)
    c.query_batch_device(dv.data_ptr(), dq.data_ptr(), qo.size - 1,
                         torch.from_numpy(cthr.view(np.int64)).cuda().data_ptr(), mode=N.QUERY_COUNT, width=2)
    r_offs, r_ids, r_cnt = c.fetch_results(qo.size - 1, mode=N.QUERY_COUNT, width=2)
    np.testing.assert_array_equal(c_offs, r_offs)
    np.testing.assert_array_equal(c_ids, r_ids)
    np.testing.assert_array_equal(c_cnt, r_cnt)


def test_host_batch_without_sector_aligned_query_starts_is_copied_whole(gpu_lib):
    """Query offsets that never start a 32-byte sector after the first query: no chunk boundary exists, the batch is
    copied whole before the launch, with the same results."""
    import torch

    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    rng = np.random.default_rng(12)
    vals, qo, thr = _long_batch(d, 18000, rng, odd=False)
    lens = np.diff(qo)
    lens = lens - lens % 4  # every length a multiple of 4 ...
    lens[0] = 1             # ... after a first query of one value: every later query starts at 1 mod 4
    qo = np.zeros(lens.size + 1, np.uint64)
    np.cumsum(lens, out=qo[1:])
    vals = vals[:int(qo[-1])]
    thr = np.minimum(thr, lens)
    assert vals.size * 8 >= 64 << 20 and np.all(qo[1:] % 4 == 1)
    a = H.membership_agent()
    offs, ids, _ = a.query_batch(vals, qo, thr)
    assert a.input_chunks() == 0
    dv = torch.from_numpy(vals.view(np.int64)).cuda()
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(thr.view(np.int64)).cuda()
    r = H.membership_agent()
    nq = qo.size - 1
    r.reserve(nq, vals.size, nq * 8 + 65536, nq * 16 + 65536)
    r.query_batch_device(dv.data_ptr(), dq.data_ptr(), nq, dt.data_ptr())
    offs_r, ids_r, _ = r.fetch_results(nq)
    np.testing.assert_array_equal(offs, offs_r)
    np.testing.assert_array_equal(ids, ids_r)


@pytest.mark.parametrize("schedule", ["fixed", "adaptive"])
def test_early_exit_bounds_a_split_user_bins_sum_by_its_bin_count(gpu_lib, oracle, schedule):
    """A user bin split over w technical bins sums w counts, so one value can add up to w to its sum: the early exit
    must bound the final sum by x + w * remaining, not x + remaining.  All-ones rows make every value count in every
    bin: user bin 0 (4 bins) sums 4 per value and reaches a threshold of 3 x the query length; the others sum 1."""
    tb = 64
    user_bin = np.array([0, 0, 0, 0] + list(range(1, tb - 3)), np.uint64)
    t = dict(n_user_bins=int(user_bin.max()) + 1, bins=np.array([tb], np.uint64), bin_size=np.array([1024], np.uint64),
             hash_funs=np.array([2], np.uint64), next_ibf=np.zeros(tb, np.uint64), user_bin=user_bin)
    words = np.full(1024 * (tb // 64), np.uint64(~np.uint64(0)), np.uint64)
    H = hg.hierarchical_interleaved_bloom_filter.from_tables(t["n_user_bins"], t["bins"], t["bin_size"],
                                                             t["hash_funs"], t["next_ibf"], t["user_bin"],
                                                             words=[words])
    O = oracle.hibf(dict(t, words=[words]))
    rng = np.random.default_rng(3)
    lens = [1000, 2000, 700, 3000]
    vals = rng.integers(0, 2**63, sum(lens), dtype=np.uint64)
    qo = np.zeros(len(lens) + 1, np.uint64)
    np.cumsum(lens, out=qo[1:])
    thr = np.array([3 * n for n in lens], np.uint64)
    a = H.membership_agent()
    tune = dict(a.tuning, early_exit_min=64)
    if schedule == "adaptive":
        tune.update(early_exit_stages=N.EARLY_EXIT_ADAPTIVE, early_exit_step=32)
    a.tuning = tune
    offs, ids, _ = a.query_batch(vals, qo, thr)
    o_off, o_ids = O.membership_batch(vals, qo, thr, threads=2)
    np.testing.assert_array_equal(offs, o_off)
    np.testing.assert_array_equal(ids, o_ids)
    assert list(ids) == [0] * len(lens)
    c = H.counting_agent(2)
    c.tuning = tune
    c_offs, c_ids, c_cnt = c.query_batch(vals, qo, thr, mode=N.QUERY_COUNT, width=2)
    assert list(c_ids) == [0] * len(lens) and list(c_cnt) == [4 * n for n in lens]


def test_streamed_host_batch_with_empty_queries_and_zero_thresholds(gpu_lib):
    """Streamed host batch whose queries include empty ones (some at chunk boundaries, since a chunk may start at any
    query whose first value starts a sector) and zero thresholds (every segment reached, every merged bin descended):
    the same results as the device-resident batch."""
    import torch

    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    rng = np.random.default_rng(13)
    vals, qo, thr = _long_batch(d, 20000, rng)
    lens = np.diff(qo).astype(np.int64)
    lens[rng.random(lens.size) < 0.2] = 0  # a fifth of the queries empty
    lens[:3] = 0
    lens[-3:] = 0
    keep = np.concatenate([np.arange(qo[i], qo[i] + lens[i]) for i in range(lens.size)]).astype(np.int64)
    vals = vals[keep]
    qo = np.zeros(lens.size + 1, np.uint64)
    np.cumsum(lens, out=qo[1:])
    thr = np.minimum(thr, np.maximum(lens, 1).astype(np.uint64))  # empty queries: threshold 1, no result
    thr[rng.random(thr.size) < 0.01] = 0  # threshold 0: every user bin, every merged bin descended
    assert vals.size * 8 >= 64 << 20
    a = H.membership_agent()
    offs, ids, _ = a.query_batch(vals, qo, thr)
    assert a.input_chunks() > 2
    nq = qo.size - 1
    r = H.membership_agent()
    r.reserve(nq, vals.size, nq * 16 + 65536, nq * 128 + 65536)
    dv = torch.from_numpy(vals.view(np.int64)).cuda()
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(thr.view(np.int64)).cuda()
    r.query_batch_device(dv.data_ptr(), dq.data_ptr(), nq, dt.data_ptr())
    offs_r, ids_r, _ = r.fetch_results(nq)
    np.testing.assert_array_equal(offs, offs_r)
    np.testing.assert_array_equal(ids, ids_r)
    empty = (lens == 0) & (thr > 0)
    assert empty.sum() > 1000 and np.all(np.diff(offs)[empty] == 0)
    zero = thr == 0
    assert zero.sum() > 50 and np.all(np.diff(offs)[zero] == d["n_ub"])


@pytest.mark.parametrize("name", G.HIBF_CASES)
def test_implied_visits_equal_the_oracles(gpu_lib, oracle, name):
    """The work the roofline counts: the (query, IBF) tasks and value visits the reference's traversal implies, as the
    kernel reports them (hibf_gpu_agent_last_work), equal the oracle's walk of the same queries (every IBF it counts,
    times the query's length), under the work queue and the level schedule."""
    d = G.hibf_case(name)
    qv, qo = d["q_values"], d["q_offsets"]
    nq = qo.size - 1
    if nq == 0:
        return
    O = oracle.hibf(G.tables(d))
    walks = O.query_batch(qv, qo, d["mem_t"], d["cnt_t"], threads=4)["visits"].astype(np.int64)
    lengths = np.diff(qo).astype(np.int64)
    H = _gpu_hibf(d)
    a = H.membership_agent()
    for schedule in (N.SCHEDULE_QUEUE, N.SCHEDULE_LEVELS):
        a.tuning = dict(a.tuning, block_queries=0, schedule=schedule)
        a.query_batch(qv, qo, d["mem_t"])
        tasks, visits = a.last_work()
        assert tasks == int(walks.sum()) and visits == int((walks * lengths).sum()), schedule


@pytest.mark.parametrize("name", G.HIBF_CASES)
def test_level_schedule_gives_the_reference_results(gpu_lib, name):
    """HIBF_GPU_SCHEDULE_LEVELS (one launch per level, each level's tasks grouped by IBF): membership lists and
    counts equal the reference's with the adaptive early exit and without one, read in place from page-locked host
    memory (roots staging the values for the lower levels), in a permuted claim order, and from a graph-captured batch
    replayed twice."""
    import torch

    d = G.hibf_case(name)
    H = _gpu_hibf(d)
    a = H.membership_agent()
    qv, qo = d["q_values"], d["q_offsets"]
    nq = qo.size - 1
    exp = G.mem_lists(d, "mem_sorted")
    w = 2 if "count2" in d else 8
    for ee in (dict(), dict(early_exit_stages=0), dict(level_values_per_lane=2)):
        try:
            a.tuning = dict(a.tuning, block_queries=0, schedule=N.SCHEDULE_LEVELS, **ee)
        except hg.InvalidArgument:
            assert "level_values_per_lane" in ee  # more than 3 hashes or rows wider than 4 words: default kernel
            continue
        offs, ids, _ = a.query_batch(qv, qo, d["mem_t"])
        for i, (g, e) in enumerate(zip(_split(offs, ids), exp)):
            np.testing.assert_array_equal(g, e, err_msg=f"{ee} query {i}")
        # per-level work adds up to the batch's; the roots visit every value once
        lw = a.level_work()
        if nq == 0:
            assert lw == []
        else:
            tasks, visits = a.last_work()
            assert len(lw) == H.info()["max_depth"] + 1
            assert sum(x["tasks"] for x in lw) == tasks and sum(x["value_visits"] for x in lw) == visits
            assert sum(x["value_visits_executed"] for x in lw) == a.last_work_executed()
            assert lw[0]["tasks"] == nq and lw[0]["value_visits"] == int(qo[-1])
            assert all(x["value_visits_executed"] <= x["value_visits"] for x in lw)
        offs, ids, cnts = a.query_batch(qv, qo, d["cnt_t"], mode=N.QUERY_COUNT, width=w)
        dense = np.zeros_like(d[f"count{w}"])
        for i in range(nq):
            dense[i, ids[offs[i]:offs[i + 1]].astype(np.int64)] = cnts[offs[i]:offs[i + 1]]
        np.testing.assert_array_equal(dense, d[f"count{w}"], err_msg=str(ee))
    if nq == 0:
        return
    # the same batch read in place from page-locked memory (the roots stage the values for the lower levels)
    if qv.size:
        a.tuning = dict(a.tuning, early_exit_stages=N.EARLY_EXIT_ADAPTIVE, level_values_per_lane=0)
        pinned = torch.from_numpy(qv.view(np.int64)).pin_memory().numpy().view(np.uint64)
        offs, ids, _ = a.query_batch(pinned, qo, d["mem_t"])
        assert a.last_in_place()
        for i, (g, e) in enumerate(zip(_split(offs, ids), exp)):
            np.testing.assert_array_equal(g, e, err_msg=f"in place query {i}")
        offs, ids, cnts = a.query_batch(pinned, qo, d["cnt_t"], mode=N.QUERY_COUNT, width=w)
        dense = np.zeros_like(d[f"count{w}"])
        for i in range(nq):
            dense[i, ids[offs[i]:offs[i + 1]].astype(np.int64)] = cnts[offs[i]:offs[i + 1]]
        np.testing.assert_array_equal(dense, d[f"count{w}"], err_msg="in place counts")
    dv = torch.from_numpy(qv.view(np.int64)).cuda() if qv.size else torch.zeros(1, dtype=torch.int64, device="cuda")
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(d["mem_t"].astype(np.uint64).view(np.int64)).cuda()
    perm = np.random.default_rng(3).permutation(nq).astype(np.uint32)
    dperm = torch.from_numpy(perm.view(np.int32)).cuda()
    a.set_order(dperm.data_ptr(), nq)
    offs, ids, _ = a.query_batch(qv, qo, d["mem_t"])
    for i, (g, e) in enumerate(zip(_split(offs, ids), exp)):
        np.testing.assert_array_equal(g, e, err_msg=f"ordered query {i}")
    a.set_order(None)
    a.reserve(nq, max(qv.size, 1), nq * 8 + 65536, nq * 64 + 65536)
    a.capture_batch_device(dv.data_ptr(), dq.data_ptr(), nq, dt.data_ptr())
    for _ in range(2):
        a.replay()
        offs, ids, _ = a.fetch_results(nq)
        for i, (g, e) in enumerate(zip(_split(offs, ids), exp)):
            np.testing.assert_array_equal(g, e, err_msg=f"replayed query {i}")
    levels = a.level_ms()
    assert len(levels) == H.info()["max_depth"] + 1 and all(x >= 0 for x in levels)


def test_level_schedule_streamed_host_batch(gpu_lib, oracle):
    """A streamed host batch (values copied in chunks while the root level waits for them) under the level
    schedule: the oracle's results."""
    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    vals, qo, thr = _long_batch(d, 24000, np.random.default_rng(17))
    a = H.membership_agent()
    a.tuning = dict(a.tuning, schedule=N.SCHEDULE_LEVELS)
    offs, ids, _ = a.query_batch(vals, qo, thr)
    assert a.input_chunks() > 2
    O = oracle.hibf(G.tables(d))
    o_off, o_ids = O.membership_batch(vals, qo, thr, threads=8)
    np.testing.assert_array_equal(offs, o_off)
    np.testing.assert_array_equal(ids, o_ids)
    t = a.last_timeline()
    assert len(t) == a.input_chunks() + 3 and t[-1] >= t[-2] >= t[-3]


def test_host_batch_read_in_place(gpu_lib, oracle):
    """A large host batch in page-locked memory is read in place by the kernel by default (no copy, the configured
    schedule from the first root): the oracle's results, membership and counts; pageable values, or page-locked ones
    with in-place reads switched off, are copied (streamed)."""
    import torch

    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    vals, qo, thr = _long_batch(d, 24000, np.random.default_rng(31))
    pinned = torch.from_numpy(vals.view(np.int64)).pin_memory().numpy().view(np.uint64)
    O = oracle.hibf(G.tables(d))
    o_off, o_ids = O.membership_batch(vals, qo, thr, threads=8)
    for schedule in (N.SCHEDULE_LEVELS, N.SCHEDULE_QUEUE):
        a = H.membership_agent()
        a.tuning = dict(a.tuning, schedule=schedule)
        offs, ids, _ = a.query_batch(pinned, qo, thr)  # in place is the default
        assert a.last_in_place() and a.input_chunks() == 0
        np.testing.assert_array_equal(offs, o_off)
        np.testing.assert_array_equal(ids, o_ids)
        c = H.counting_agent(2)
        c.set_host_read(True)
        c_off, c_ids, c_cnt = c.query_batch(pinned, qo, thr, mode=N.QUERY_COUNT, width=2)
        np.testing.assert_array_equal(c_ids, o_ids)
        assert c.last_in_place()
        # results as views of the agents' page-locked buffers: the same arrays
        v_off, v_ids, _ = a.query_batch(pinned, qo, thr, copy=False)
        np.testing.assert_array_equal(v_off, o_off)
        np.testing.assert_array_equal(v_ids, o_ids)
        w_off, w_ids, w_cnt = c.query_batch(pinned, qo, thr, mode=N.QUERY_COUNT, width=2, copy=False)
        assert w_cnt.dtype == np.uint16 and not w_cnt.flags.owndata
        np.testing.assert_array_equal(w_ids, c_ids)
        np.testing.assert_array_equal(w_cnt, c_cnt)
        offs, ids, _ = a.query_batch(vals, qo, thr)  # pageable: copied
        assert not a.last_in_place()
        np.testing.assert_array_equal(ids, o_ids)
        a.set_host_read(False)  # page-locked but copied first: streamed in chunks
        offs, ids, _ = a.query_batch(pinned, qo, thr)
        assert not a.last_in_place() and a.input_chunks() > 2
        np.testing.assert_array_equal(ids, o_ids)


def test_autotune_on_a_throughput_batch_tries_the_level_schedule(gpu_lib, oracle):
    """A batch above block_queries runs the persistent kernel, so the search times the level schedule too; whichever
    it keeps, the results are the oracle's."""
    import torch

    d = G.hibf_case("synth600")
    H = _gpu_hibf(d)
    vals, qo, thr = _long_batch(d, 12000, np.random.default_rng(23))
    nq = qo.size - 1
    a = H.membership_agent()
    dv = torch.from_numpy(vals.view(np.int64)).cuda()
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(thr.view(np.int64)).cuda()
    a.reserve(nq, vals.size, nq * 8 + 65536, nq * 16 + 65536)
    torch.cuda.synchronize()
    trials = a.autotune(dv.data_ptr(), dq.data_ptr(), nq, dt.data_ptr(), reps=1)
    assert any(t["schedule"] == N.SCHEDULE_LEVELS for t in trials)
    offs, ids, _ = a.query_batch(vals, qo, thr)
    O = oracle.hibf(G.tables(d))
    o_off, o_ids = O.membership_batch(vals, qo, thr, threads=8)
    np.testing.assert_array_equal(offs, o_off)
    np.testing.assert_array_equal(ids, o_ids)
