"""Replicas across GPUs: every rank holds a full copy of the index and answers a contiguous shard of each query batch.

Queries are independent, so a batch splits by query with no exchange between ranks while it runs; each rank's
answer is a CSR block (result offsets, user bin ids) for its shard, and the blocks are concatenated in rank order.
The only communication is the host-side gather of finished results (any torch.distributed backend; gloo works without
a GPU).  One process per GPU, as torchrun launches them.
"""

from __future__ import annotations

import numpy as np


def shard_range(n_queries: int, rank: int, world: int) -> tuple[int, int]:
    """[first, last) queries of `rank`: contiguous, sizes differing by at most one, in rank order."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(n_queries, world)
    first = rank * base + min(rank, extra)
    return first, first + base + (1 if rank < extra else 0)


def shard_batch(values, query_offsets, thresholds, rank: int, world: int):
    """This rank's part of a CSR batch: (values, offsets rebased to 0, thresholds, first query index)."""
    qo = np.asarray(query_offsets, dtype=np.uint64)
    first, last = shard_range(qo.size - 1, rank, world)
    lo, hi = int(qo[first]), int(qo[last])
    v = np.asarray(values, dtype=np.uint64)[lo:hi]
    return v, qo[first:last + 1] - np.uint64(lo), np.asarray(thresholds, dtype=np.uint64)[first:last], first


def merge_shards(parts) -> tuple[np.ndarray, np.ndarray]:
    """Concatenates per-rank (offsets, ids) CSR blocks, in rank order, into the whole batch's."""
    offs = [np.zeros(1, np.uint64)]
    ids = []
    base = np.uint64(0)
    for o, i in parts:
        o = np.asarray(o, dtype=np.uint64)
        offs.append(o[1:] + base)
        ids.append(np.asarray(i, dtype=np.uint64))
        base = base + (o[-1] if o.size else np.uint64(0))
    return np.concatenate(offs), (np.concatenate(ids) if ids else np.zeros(0, np.uint64))


def gather_results(offsets, ids, group=None):
    """Gathers every rank's (offsets, ids) on rank 0 and merges them; other ranks get None."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    mine = (np.asarray(offsets, dtype=np.uint64), np.asarray(ids, dtype=np.uint64))
    got = [None] * world if rank == 0 else None
    dist.gather_object(mine, got, dst=0, group=group)
    return merge_shards(got) if rank == 0 else None


def answer_shard(agent, values, query_offsets, thresholds, rank: int, world: int, **kw):
    """Runs this rank's shard on its replica through `agent.query_batch` and returns (offsets, ids)."""
    v, qo, t, _ = shard_batch(values, query_offsets, thresholds, rank, world)
    offs, ids, _ = agent.query_batch(v, qo, t, **kw)
    return offs, ids
