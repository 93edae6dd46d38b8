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


_TORCH_DT = {1: "int8", 2: "int16", 4: "int32", 8: "int64"}
_NP_DT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


@pytest.mark.parametrize("bins", [1000, 4096, 16384])
@pytest.mark.parametrize("width", [1, 2, 4, 8])
def test_noalloc_bulk_count_equals_bulk_count(gpu_lib, bins, width):
    """1,000 bins: per-warp counters in shared memory; 4,096: counters shared by the block; 16,384: the largest
    filter the static array holds, rows of 256 words (the path for rows wider than a warp), 64 KiB of dynamic shared
    memory.  The first call counts every stored value twice, so uint8 counts wrap."""
    import torch

    bsz, h = 1 << 14, 3
    ibf = hg.interleaved_bloom_filter(hg.bin_count(bins), hg.bin_size(bsz), hg.hash_function_count(h))
    vals = S.stream_range(42, 0, 200_000)
    ibf.emplace_many(vals, (np.arange(vals.size) % bins).astype(np.uint64))
    dt = getattr(torch, _TORCH_DT[width])
    for call, q in enumerate((np.concatenate([vals, vals[:100_000], S.stream_range(7, 0, 100_000)]),
                              np.concatenate([vals[150_000:], S.stream_range(8, 0, 50_000)]))):
        d_q = torch.from_numpy(q.view(np.int64)).cuda()
        out_ref = torch.zeros(bins, dtype=dt, device="cuda")
        out_na = torch.full((bins,), -1, dtype=dt, device="cuda")
        torch.cuda.synchronize()
        N.call("hibf_gpu_ibf_bulk_count_d", ibf._h, d_q.data_ptr(), q.size, width, out_ref.data_ptr(), None)
        N.call("hibf_gpu_ibf_bulk_count_noalloc_d", ibf._h, d_q.data_ptr(), q.size, width, out_na.data_ptr(), None)
        N.call("hibf_gpu_ibf_status", ibf._h)
        ref = out_ref.cpu().numpy().view(_NP_DT[width])
        got = out_na.cpu().numpy().view(_NP_DT[width])
        np.testing.assert_array_equal(got, ref, err_msg=f"call {call}")
        assert int(ref.astype(np.uint64).sum()) > 0
        if call == 0 and width == 1:
            # every bin holds >= 12 stored values and is hit by each of them at least once more than stored: compare
            # the wrapped uint8 counts with the exact 64-bit ones
            full = torch.zeros(bins, dtype=torch.int64, device="cuda")
            torch.cuda.synchronize()  # the zero fill runs on torch's stream, the count on the filter's
            N.call("hibf_gpu_ibf_bulk_count_d", ibf._h, d_q.data_ptr(), q.size, 8, full.data_ptr(), None)
            N.call("hibf_gpu_ibf_status", ibf._h)
            exact = full.cpu().numpy().view(np.uint64)
            np.testing.assert_array_equal(got.astype(np.uint64), exact % np.uint64(256))
            if bins == 1000:
                assert int(exact.min()) > 255  # 300 hits per bin at least: the uint8 counts wrapped


def test_noalloc_rejects_too_many_bins(gpu_lib):
    import torch

    ibf = hg.interleaved_bloom_filter(hg.bin_count(20000), hg.bin_size(64), hg.hash_function_count(2))
    d_q = torch.zeros(4, dtype=torch.int64, device="cuda")
    out = torch.zeros(20000, dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    st = N.lib().hibf_gpu_ibf_bulk_count_noalloc_d(ibf._h, d_q.data_ptr(), 4, 2, out.data_ptr(), None)
    assert st == N.ERR_INVALID_ARG
    assert "16384" in N.last_error()
