"""Continuous-batching server (hibf_gpu_server_*): every request's results equal the same queries answered alone,
whatever else shares its batch; admission control; the open-loop driver.  GPU tests."""

import random
import threading

import numpy as np
import pytest

import hibf_gb300 as hg
from hibf_gb300 import _native as N
from hibf_gb300.serve import server
from tests import golden_io as G

pytestmark = pytest.mark.gpu


def _hibf(name="synth600"):
    d = G.hibf_case(name)
    t = G.tables(d)
    H = hg.hierarchical_interleaved_bloom_filter.from_tables(t["n_user_bins"], t["bins"], t["bin_size"],
                                                             t["hash_funs"], t["next_ibf"], t["user_bin"],
                                                             words=t["words"])
    return H, d


def _requests(d, n, seed):
    rng = random.Random(seed)
    qs = G.queries(d)
    out = []
    for _ in range(n):
        k = rng.randint(1, 24)
        first = rng.randrange(0, len(qs) - k)
        sel = qs[first:first + k]
        qo = np.zeros(k + 1, np.uint64)
        np.cumsum([q.size for q in sel], out=qo[1:])
        f = rng.uniform(0.5, 0.9)
        thr = np.array([int(np.ceil(f * q.size)) for q in sel], np.uint64)
        out.append((np.concatenate(sel), qo, thr))
    return out


def test_results_same_alone_and_in_the_mix(gpu_lib):
    H, d = _hibf()
    reqs = _requests(d, 150, 1)
    alone = [H.membership_agent().query_batch(v, qo, t)[:2] for v, qo, t in reqs]
    srv = server(H, slots=3, max_batch_queries=48, max_batch_values=30000, admission_bytes=1 << 30)
    ids = [None] * len(reqs)

    def client(part):
        for i in part:
            v, qo, t = reqs[i]
            ids[i] = srv.submit(v, qo, t)

    threads = [threading.Thread(target=client, args=(range(j, len(reqs), 4),)) for j in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for i, (v, qo, t) in enumerate(reqs):
        st, offs, rid, lat = srv.wait_result(ids[i], qo.size - 1, timeout_ms=60000)
        assert st == N.OK
        np.testing.assert_array_equal(offs, alone[i][0])
        np.testing.assert_array_equal(rid, alone[i][1])
        assert lat >= 0
    s = srv.stats()
    assert s["batches"] >= 2 and s["batches"] < len(reqs)  # requests were coalesced
    srv.close()


def test_admission_rejects_oversized_request(gpu_lib):
    H, d = _hibf()
    srv = server(H, slots=2, max_batch_queries=8, max_batch_values=1000, admission_bytes=1 << 28)
    v = np.arange(5000, dtype=np.uint64)
    rid = srv.submit(v, [0, 5000], [10])
    st, offs, ids, _ = srv.wait_result(rid, 1, timeout_ms=60000)
    assert st == N.ERR_ADMISSION and offs is None
    # the server keeps serving
    rid = srv.submit(v[:100], [0, 100], [10])
    st, offs, ids, _ = srv.wait_result(rid, 1, timeout_ms=60000)
    assert st == N.OK
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_open_loop_driver(gpu_lib):
    H, d = _hibf()
    srv = server(H, slots=4, max_batch_queries=4096, max_batch_values=1 << 22, admission_bytes=1 << 30)
    r = srv.open_loop(d["q_values"], d["q_offsets"], offered_qps=20000, duration_s=0.3, max_request_queries=64)
    assert r["requests"] > 0 and r["rejected"] == 0
    assert 0 < r["p50_ms"] <= r["p99_ms"] <= r["p999_ms"]
    # the load generator's lateness, and latency from the actual submission, which the lateness can only shorten
    assert 0 <= r["generator_late_p999_ms"] <= r["generator_late_max_ms"]
    assert 0 <= r["generator_late_over_1ms"] <= r["requests"]
    assert 0 < r["p99_from_submit_ms"] <= r["p99_ms"] + 1e-6
    assert r["p99_from_submit_ms"] <= r["p999_from_submit_ms"] <= r["p999_ms"] + 1e-6
    srv.close()


def test_bounded_wait_expires_into_status(gpu_lib):
    """Failure detection: a work-queue wait that nothing satisfies ends after its limit with a TIMEOUT status read by
    the host, and the same agent and context answer correctly afterwards."""
    H, d = _hibf()
    a = H.membership_agent()
    N.call("hibf_gpu_agent_selftest_wait_limit", a._a, 50.0)
    offs, ids, _ = a.query_batch(d["q_values"], d["q_offsets"], d["mem_t"])
    exp = G.mem_lists(d, "mem_sorted")
    got = [ids[offs[i]:offs[i + 1]] for i in range(offs.size - 1)]
    assert all(np.array_equal(g, e) for g, e in zip(got, exp))


def test_allocation_failure_is_a_status(gpu_lib):
    """A device allocation that cannot succeed returns OUT_OF_MEMORY; nothing else breaks."""
    with pytest.raises(MemoryError):
        hg.interleaved_bloom_filter(hg.bin_count(64), hg.bin_size(1 << 46), hg.hash_function_count(2))
    ibf = hg.interleaved_bloom_filter(hg.bin_count(64), hg.bin_size(1024), hg.hash_function_count(2))
    ibf.emplace(5, hg.bin_index(3))
    assert ibf.counting_agent().bulk_count([5])[3] == 1


def test_pinned_borrowed_requests_match(gpu_lib):
    """Requests whose values sit in page-locked memory go to the device without staging; mixed with staged ones in
    the same batches, every result equals the query answered alone."""
    import torch

    H, d = _hibf()
    reqs = _requests(d, 40, seed=5)
    agent = H.membership_agent()
    expect = [agent.query_batch(v, qo, t)[:2] for v, qo, t in reqs]
    srv = server(H, slots=2, max_batch_queries=4096, max_batch_values=1 << 22, admission_bytes=1 << 30)
    keep, ids = [], []
    for i, (v, qo, t) in enumerate(reqs):
        if i % 2 == 0:
            pv = torch.from_numpy(v.view(np.int64)).pin_memory()
            srv.register_host(pv.data_ptr(), max(8, pv.numel() * 8), already_pinned=True)
            keep.append((pv, qo, t))
            ids.append(srv.submit_borrowed(pv.data_ptr(), qo, t))
        else:
            ids.append(srv.submit(v, qo, t))
    for rid, (v, qo, t), (eo, ei) in zip(ids, reqs, expect):
        st, offs, res, _ = srv.wait_result(rid, qo.size - 1)
        assert st == 0
        np.testing.assert_array_equal(offs, eo)
        np.testing.assert_array_equal(res, ei)
    # the batch log: every value once, and only the copied requests' values staged through the slots' buffers
    log = srv.batch_log()
    assert log.shape[1] == 12 and int(log[:, 6].sum()) == sum(qo.size - 1 for _, qo, _ in reqs)
    assert int(log[:, 7].sum()) == sum(v.size for v, _, _ in reqs)
    assert int(log[:, 10].sum()) == sum(v.size for i, (v, _, _) in enumerate(reqs) if i % 2)
    srv.close()


def test_zero_copy_batches_match(gpu_lib):
    """Back-to-back borrowed requests in one mapped page-locked range are answered without copying their values (the
    kernel reads them in place), in memory the caller page-locked and in pageable memory the server page-locks on
    registration; with zero copy off they are copied first.  Every result equals the query answered alone."""
    import torch

    H, d = _hibf()
    qs = G.queries(d)
    agent = H.membership_agent()
    pool = torch.from_numpy(np.concatenate(qs).view(np.int64)).pin_memory()
    starts = np.zeros(len(qs) + 1, np.int64)
    np.cumsum([q.size for q in qs], out=starts[1:])
    # consecutive slices of the pool, so that a batch of several of them is one contiguous run
    reqs = []
    k0 = 0
    rng = np.random.default_rng(3)
    while k0 < len(qs) - 1:
        k1 = min(len(qs), k0 + int(rng.integers(1, 12)))
        qo = (starts[k0:k1 + 1] - starts[k0]).astype(np.uint64)
        thr = np.array([int(np.ceil(0.6 * q.size)) for q in qs[k0:k1]], np.uint64)
        reqs.append((k0, k1, qo, thr))
        k0 = k1
    pageable = np.concatenate(qs).astype(np.uint64)  # page-locked by the server on registration
    for zc, base, pinned in ((True, pool.data_ptr(), True), (False, pool.data_ptr(), True),
                             (True, pageable.ctypes.data, False)):
        srv = server(H, slots=2, max_batch_queries=4096, max_batch_values=1 << 22, admission_bytes=1 << 30)
        srv.set_zero_copy(zc)
        srv.register_host(base, starts[-1] * 8, already_pinned=pinned)
        ids = [srv.submit_borrowed(base + 8 * int(starts[a]), qo, thr) for a, b, qo, thr in reqs]
        for rid, (a, b, qo, thr) in zip(ids, reqs):
            st, offs, res, _ = srv.wait_result(rid, qo.size - 1)
            assert st == 0
            eo, ei, _ = agent.query_batch(pool.numpy()[starts[a]:starts[b]].view(np.uint64), qo, thr)
            np.testing.assert_array_equal(offs, eo)
            np.testing.assert_array_equal(res, ei)
        log = srv.batch_log()
        assert int(log[:, 10].sum()) == 0
        assert (log[:, 11].sum() > 0) == zc
        if not pinned:
            srv.unregister_host(base)
        srv.close()


def test_open_loop_reads_a_page_locked_pool_without_staging(gpu_lib):
    """The open-loop driver registers a page-locked request pool, so its borrowed requests go to the device by DMA
    from the pool: no value is staged through a slot's buffer."""
    import torch

    H, d = _hibf()
    pool = torch.from_numpy(d["q_values"].view(np.int64)).pin_memory()
    srv = server(H, slots=2, max_batch_queries=4096, max_batch_values=1 << 22, admission_bytes=1 << 30)
    r = srv.open_loop(pool.numpy().view(np.uint64), d["q_offsets"], offered_qps=20000, duration_s=0.3,
                      max_request_queries=64)
    log = srv.batch_log()
    assert r["requests"] > 0 and log.shape[0] > 0
    assert int(log[:, 10].sum()) == 0
    srv.close()
