"""The chunking of streamed host batches (hibf_gpu_stream_plan, no device needed): chunks start only at queries whose
first value starts a 32-byte sector, so that no sector of the device copy holds values of two chunks (a sector cached
from an earlier chunk can then never hold values of a later one)."""

import numpy as np
import pytest

from hibf_gb300 import _native as N
from hibf_gb300.hibf import stream_plan


def _offsets(lens):
    qo = np.zeros(len(lens) + 1, np.uint64)
    np.cumsum(np.asarray(lens, np.uint64), out=qo[1:])
    return qo


def test_boundaries_start_sectors_and_cover_the_batch():
    rng = np.random.default_rng(1)
    lens = rng.integers(0, 1500, 40000) * 2 + 1  # odd lengths: about a quarter of the query starts are aligned
    qo = _offsets(lens)
    assert int(qo[-1]) * 8 >= 64 << 20
    b = stream_plan(qo)
    assert b[0] == 0 and b[-1] == qo.size - 1
    assert np.all(np.diff(b.astype(np.int64)) > 0)
    assert 3 <= b.size <= 65
    assert np.all(qo[b[1:-1]] % 4 == 0)
    # the chunks split the values evenly enough: none above three times the mean
    sizes = np.diff(qo[b].astype(np.int64))
    assert sizes.max() <= 3 * sizes.mean()


def test_small_batches_are_not_streamed():
    assert stream_plan(_offsets([100] * 1000)).size == 0
    assert stream_plan(_offsets([])).size == 0


def test_no_sector_aligned_query_start_means_one_copy():
    lens = [1] + [4] * 3_000_000  # every later query starts at 1 mod 4
    b = stream_plan(_offsets(lens))
    assert b.size <= 2


def test_aligned_queries_give_up_to_64_chunks():
    lens = [512] * 300_000  # 1.2 GiB of values: 64 chunks of 16 MiB or more
    b = stream_plan(_offsets(lens))
    assert b.size == 65


def test_decreasing_offsets_are_rejected():
    qo = _offsets([5] * 10)
    qo[3] = 1
    with pytest.raises(N.InvalidArgument):
        stream_plan(qo)
