"""The seeded synthetic workloads agree across their three statements: hibf_gb300.synthetic (Python), the C header
on the host (C ABI synth entry points) and the CUDA generator (GPU test)."""

import ctypes

import numpy as np
import pytest

from hibf_gb300 import _build, _native as N
from hibf_gb300 import synthetic as S


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return N.lib()


SPECS = [
    S.query_spec(1, S.QUERIES_HALF_ONE_BIN, 250, 250, 0, 0, 1, 2, 64),
    S.query_spec(3, S.QUERIES_MIXED, 20, 2000, 70, 2, 7, 10, 8192),
    S.query_spec(5, S.QUERIES_MIXED, 50, 5000, 70, 2, 6, 10, 300),
]


def _c_offsets(spec, first, n):
    qo = np.zeros(n + 1, np.uint64)
    thr = np.zeros(n, np.uint64)
    N.call("hibf_gpu_synth_query_offsets", spec.seed, spec.law, spec.len_lo, spec.len_hi, spec.mix_pct,
           spec.noise_pct, spec.thr_num, spec.thr_den, spec.n_user_bins, first, n, qo.ctypes.data, thr.ctypes.data)
    return qo, thr


def test_user_bin_sizes_match(lib):
    for args in ((1, S.SIZES_LOG_UNIFORM, 0.0, 0.0, 1000, 100000, 64),
                 (1, S.SIZES_LOG_NORMAL, 200000.0, 1.5, 1000, 50000000, 8192)):
        off = np.zeros(args[-1] + 1, np.uint64)
        N.call("hibf_gpu_synth_user_bin_offsets", *args, off.ctypes.data)
        seed, law, p0, p1, lo, hi, n = args
        np.testing.assert_array_equal(off, S.offsets_of(S.user_bin_sizes(seed, n, law, p0, p1, lo, hi)))


@pytest.mark.parametrize("spec", SPECS, ids=["half", "mixed2000", "mixed5000"])
def test_queries_match(lib, spec):
    sizes = S.user_bin_sizes(spec.seed, spec.n_user_bins, S.SIZES_LOG_UNIFORM, 0, 0, 10, 5000)
    offs = S.offsets_of(sizes)
    first, n = 17, 40
    qv, qo, thr = S.queries(spec, offs, first, n)
    c_qo, c_thr = _c_offsets(spec, first, n)
    np.testing.assert_array_equal(qo, c_qo)
    np.testing.assert_array_equal(thr, c_thr)
    vals = np.zeros(int(c_qo[-1]), np.uint64)
    N.call("hibf_gpu_synth_queries", spec.seed, spec.law, spec.len_lo, spec.len_hi, spec.mix_pct, spec.noise_pct,
           spec.thr_num, spec.thr_den, spec.n_user_bins, offs.ctypes.data, first, n, c_qo.ctypes.data,
           vals.ctypes.data)
    np.testing.assert_array_equal(vals, qv)


def test_user_bin_values_distinct():
    offs = S.offsets_of(S.user_bin_sizes(1, 64, S.SIZES_LOG_UNIFORM, 0, 0, 1000, 100000))
    allv = S.stream_range(1, 0, int(offs[-1]))
    assert np.unique(allv).size == allv.size
    np.testing.assert_array_equal(S.user_bin_values(1, offs, 5), allv[offs[5]:offs[6]])


@pytest.mark.gpu
@pytest.mark.parametrize("spec", SPECS, ids=["half", "mixed2000", "mixed5000"])
def test_device_queries_match(gpu_lib, spec):
    import torch

    sizes = S.user_bin_sizes(spec.seed, spec.n_user_bins, S.SIZES_LOG_UNIFORM, 0, 0, 10, 5000)
    offs = S.offsets_of(sizes)
    first, n = 1000, 3000
    qo, _ = _c_offsets(spec, first, n)
    host = np.zeros(int(qo[-1]), np.uint64)
    N.call("hibf_gpu_synth_queries", spec.seed, spec.law, spec.len_lo, spec.len_hi, spec.mix_pct, spec.noise_pct,
           spec.thr_num, spec.thr_den, spec.n_user_bins, offs.ctypes.data, first, n, qo.ctypes.data,
           host.ctypes.data)
    d_offs = torch.from_numpy(offs.view(np.int64)).cuda()
    d_qo = torch.from_numpy(qo.view(np.int64)).cuda()
    d_v = torch.empty(int(qo[-1]), dtype=torch.int64, device="cuda")
    N.call("hibf_gpu_synth_queries_d", spec.seed, spec.law, spec.len_lo, spec.len_hi, spec.mix_pct, spec.noise_pct,
           spec.thr_num, spec.thr_den, spec.n_user_bins, d_offs.data_ptr(), first, n, d_qo.data_ptr(),
           d_v.data_ptr(), None)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_v.cpu().numpy().view(np.uint64), host)


def test_ibf_workload_queries_match(lib):
    seed, bins, vpb, first, n = 1, 1024, 5_000_000, 12345, 20000
    c = np.zeros(n, np.uint64)
    N.call("hibf_gpu_synth_ibf_queries", seed, bins, vpb, first, n, c.ctypes.data)
    np.testing.assert_array_equal(c, S.ibf_query_values(seed, bins, vpb, first, n))
    # half of the values are elements of a bin (the others uniform): check on a small workload by membership
    small = S.ibf_query_values(7, 8, 100, 0, 4000)
    members = np.concatenate([S.ibf_bin_values(7, 100, b) for b in range(8)])
    frac = np.isin(small, members).mean()
    assert 0.45 < frac < 0.55


@pytest.mark.gpu
def test_ibf_workload_device_generation(gpu_lib, oracle):
    """Device-generated queries equal the host ones; device-generated inserts set the bits the oracle sets."""
    import torch

    import hibf_gb300 as hg

    seed, bins, vpb = 3, 130, 700
    n = 50000
    d = torch.empty(n, dtype=torch.int64, device="cuda")
    N.call("hibf_gpu_synth_ibf_queries_d", seed, bins, vpb, 0, n, d.data_ptr(), None)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint64), S.ibf_query_values(seed, bins, vpb, 0, n))
    ibf = hg.interleaved_bloom_filter(hg.bin_count(bins), hg.bin_size(4096), hg.hash_function_count(3))
    N.call("hibf_gpu_synth_ibf_emplace", ibf._h, seed, vpb, 0, bins, None)
    O = oracle.ibf(bins, 4096, 3)
    for b in range(bins):
        O.emplace(S.ibf_bin_values(seed, vpb, b), b)
    np.testing.assert_array_equal(ibf.words(), O.words())
    q = S.ibf_query_values(seed, bins, vpb, 0, 3000)
    np.testing.assert_array_equal(ibf.counting_agent(2).bulk_count(q), O.bulk_count(q, 2, threads=4))
    np.testing.assert_array_equal(ibf.containment_agent().bulk_contains_words(q), O.bulk_contains(q, threads=4))
