"""Query-sharded search over replicas (one index replica per GPU / rank).

The reference's IndexBuilder::search answers the queries of a batch one
after another (an OpenMP loop over queries, src/builder.cpp:285); queries are
independent, so N replicas each answer a contiguous slice of the batch and
the results are concatenated in query order -- no collective on the data
path, only the gather of the answers and the sum of the counters.

SearchEntryRand draws one rand() per query in query order (the mt19937 seed
of its seeds), so a replica that starts at query `start` advances its rand
stream by `start` draws first: every query then gets the seeds it gets in a
one-replica run, and the concatenated ids equal the one-replica ids.
"""
from __future__ import annotations

import numpy as np


def query_slice(nq: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [start, end) of the nq queries for `rank` of `world`: the
    first nq % world ranks take one query more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    base, extra = divmod(nq, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def sharded_search(search, queries: np.ndarray, rank: int, world: int, skip_rand=None, gather=None):
    """Answers `queries` with `world` replicas, this process being `rank`.

    search(q) -> (ids [len(q), K] uint32, dist_count, hop_count) on this
    rank's replica; skip_rand(k) advances this replica's rand stream by k
    draws (SearchEntryRand: one per query) before the slice is searched;
    gather(obj) -> list of every rank's obj in rank order (e.g.
    torch.distributed.all_gather_object).  Returns (ids of all queries in
    query order, summed dist_count, summed hop_count); with world == 1 it is
    search(queries)."""
    start, end = query_slice(queries.shape[0], rank, world)
    if skip_rand is not None and start > 0:
        skip_rand(start)
    ids, dc, hc = search(queries[start:end])
    if world == 1:
        return ids, dc, hc
    if gather is None:
        raise ValueError("world > 1 needs a gather")
    parts = gather((start, np.ascontiguousarray(ids), int(dc), int(hc)))
    parts = sorted(parts, key=lambda p: p[0])
    out = np.concatenate([p[1] for p in parts], axis=0)
    return out, sum(p[2] for p in parts), sum(p[3] for p in parts)


def torch_gather(obj):
    """all_gather_object over the default process group."""
    import torch.distributed as dist
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out
