"""bench.py's parity helper for bulk_count: the per-query digest of (user bin, count) pairs it forms from the device's
sparse results must be the oracle's (orc_hibf_query_batch) for the same dense count vectors."""

import numpy as np

import bench
from tests import golden_io as G


def test_count_digests_match_the_oracle(oracle):
    d = G.hibf_case("synth600")
    O = oracle.hibf(G.tables(d))
    qs = G.queries(d)[:120]
    v = np.concatenate(qs)
    qo = np.zeros(len(qs) + 1, np.uint64)
    np.cumsum([q.size for q in qs], out=qo[1:])
    thr = np.maximum(1, (np.diff(qo) * 3) // 10).astype(np.uint64)
    o = O.query_batch(v, qo, thr, thr, threads=2)
    offs, ids, cnts = [0], [], []
    for i in range(len(qs)):
        c = O.bulk_count(v[qo[i]:qo[i + 1]], int(thr[i]), 2)
        nz = np.nonzero(c)[0]
        ids += list(nz)
        cnts += list(c[nz])
        offs.append(len(ids))
    dg, nnz = bench.count_digests(np.array(offs, np.uint64), np.array(ids, np.uint64), np.array(cnts, np.uint16))
    assert nnz.sum() > 0
    np.testing.assert_array_equal(nnz, o["cnt_nnz"])
    np.testing.assert_array_equal(dg, o["cnt_digest"])
    # a changed count changes its query's digest
    cnts2 = np.array(cnts, np.uint16)
    cnts2[0] += 1
    dg2, _ = bench.count_digests(np.array(offs, np.uint64), np.array(ids, np.uint64), cnts2)
    assert (dg2 != dg).sum() == 1
