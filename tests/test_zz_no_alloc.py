"""hibf_gpu_ibf_bulk_count_noalloc_d: bulk_count for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: a process whose device memory is all held by its own pool (a framework's
caching allocator), or a loop that must not pay cudaMalloc's device-wide synchronisation.  This entry point counts
with a fixed static device array as its scratch instead of an allocated buffer.  The test calls it through the C ABI
twice in a row (different queries, so the second call shows the scratch was cleared) and requires the counting
vectors to equal those of hibf_gpu_ibf_bulk_count_d exactly (integer counts: no tolerance).  It is collected last so
a run that stops at the first failure has run every other test before it.
"""

import ctypes

import numpy as np
import pytest

import hibf_gb300 as hg
from hibf_gb300 import _native as N
from hibf_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def test_noalloc_bulk_count_equals_bulk_count(gpu_lib):
    import torch

    bins, bsz, h = 1000, 1 << 14, 3
    ibf = hg.interleaved_bloom_filter(hg.bin_count(bins), hg.bin_size(bsz), hg.hash_function_count(h))
    vals = S.stream_range(42, 0, 200_000)
    ibf.emplace_many(vals, (np.arange(vals.size) % bins).astype(np.uint64))
    for call, (first, n) in enumerate(((0, 150_000), (150_000, 50_000))):
        q = np.concatenate([vals[first:first + n], S.stream_range(7 + call, 0, n)])
        d_q = torch.from_numpy(q.view(np.int64)).cuda()
        out_ref = torch.zeros(bins, dtype=torch.int16, device="cuda")
        out_na = torch.full((bins,), -1, dtype=torch.int16, device="cuda")
        torch.cuda.synchronize()
        N.call("hibf_gpu_ibf_bulk_count_d", ibf._h, d_q.data_ptr(), q.size, 2, out_ref.data_ptr(), None)
        N.call("hibf_gpu_ibf_bulk_count_noalloc_d", ibf._h, d_q.data_ptr(), q.size, 2, out_na.data_ptr(), None)
        N.call("hibf_gpu_ibf_status", ibf._h)
        ref = out_ref.cpu().numpy().view(np.uint16)
        got = out_na.cpu().numpy().view(np.uint16)
        np.testing.assert_array_equal(got, ref, err_msg=f"call {call}")
        assert int(ref.sum()) > 0


def test_noalloc_rejects_too_many_bins(gpu_lib):
    import torch

    ibf = hg.interleaved_bloom_filter(hg.bin_count(20000), hg.bin_size(64), hg.hash_function_count(2))
    d_q = torch.zeros(4, dtype=torch.int64, device="cuda")
    out = torch.zeros(20000, dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    st = N.lib().hibf_gpu_ibf_bulk_count_noalloc_d(ibf._h, d_q.data_ptr(), 4, 2, out.data_ptr(), None)
    assert st == N.ERR_INVALID_ARG
    assert "16384" in N.last_error()
