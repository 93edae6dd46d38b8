"""Replica sharding across ranks (multi-GPU serving by replicas): host logic on CPU, and a world_size-2 gloo run whose
ranks answer their shards with the C oracle and gather on rank 0, which must equal the reference's answers."""

import os
import socket

import numpy as np
import pytest

from hibf_gb300 import replicas as R
from tests import golden_io as G


def test_shard_ranges_cover_in_order():
    for n in (0, 1, 7, 100, 1001):
        for world in (1, 2, 3, 8):
            spans = [R.shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        R.shard_range(10, 2, 2)


def test_shard_and_merge_round_trip():
    rng = np.random.default_rng(3)
    lens = rng.integers(0, 9, 37)
    qo = np.zeros(38, np.uint64)
    np.cumsum(lens, out=qo[1:])
    v = rng.integers(0, 1 << 62, int(qo[-1]), dtype=np.uint64)
    thr = rng.integers(0, 5, 37).astype(np.uint64)
    # a fake answer per query (its first value, if any) so merging can be checked against the unsharded batch
    def answer(vv, oo):
        ro = np.zeros(oo.size, np.uint64)
        ids = []
        for i in range(oo.size - 1):
            if oo[i + 1] > oo[i]:
                ids.append(vv[oo[i]])
            ro[i + 1] = len(ids)
        return ro, np.array(ids, np.uint64)

    whole = answer(v, qo)
    for world in (1, 2, 5):
        parts = []
        for r in range(world):
            sv, so, st, first = R.shard_batch(v, qo, thr, r, world)
            np.testing.assert_array_equal(st, thr[first:first + so.size - 1])
            parts.append(answer(sv, so))
        mo, mi = R.merge_shards(parts)
        np.testing.assert_array_equal(mo, whole[0])
        np.testing.assert_array_equal(mi, whole[1])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    from oracle.bindings import Oracle, build_oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        build_oracle()
        d = G.hibf_case("synth600")
        O = Oracle().hibf(G.tables(d))
        v, qo, t, _ = R.shard_batch(d["q_values"], d["q_offsets"], d["mem_t"], rank, world)
        offs, ids = O.membership_batch(v, qo, t, threads=1)
        merged = R.gather_results(offs, ids)
        if rank == 0:
            np.savez(os.path.join(out_dir, "merged.npz"), offs=merged[0], ids=merged[1])
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_gather_equals_reference(tmp_path, oracle):
    import torch.multiprocessing as mp

    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    z = np.load(tmp_path / "merged.npz")
    d = G.hibf_case("synth600")
    exp = G.mem_lists(d, "mem_sorted")
    offs, ids = z["offs"], z["ids"]
    assert offs.size == len(exp) + 1
    for i, e in enumerate(exp):
        np.testing.assert_array_equal(ids[offs[i]:offs[i + 1]], e, err_msg=f"query {i}")
