"""bench.py's multi-rank timing (torchrun, one replica per GPU, the search
sharded by query): the barrier around the timed region and the whole-job
rate -- all ranks' units over the slowest rank's step time -- checked with
two gloo ranks on the CPU."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(r, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=r, world_size=2)
    import bench
    rate, ms = bench.job_rate(1000, 2.0 + r)  # rank 1 is the slower one
    bench.rank_barrier()
    q.put((r, bench.world(), bench.rank(), rate, ms, bench.rank_reduce(r + 1, "sum"),
           bench.rank_reduce(5 - r, "max")))
    dist.destroy_process_group()


def test_job_rate_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rr, w, rk, rate, ms, s, m) in enumerate(out):
        assert (rr, w, rk) == (r, 2, r)
        assert ms == pytest.approx(3.0)                 # the slowest rank's step
        assert rate == pytest.approx(2000 / 3.0e-3)     # both ranks' queries
        assert s == 3 and m == 5


def test_single_process_is_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(500, 4.0) == (pytest.approx(125000.0), 4.0)


def test_query_slices_cover_the_batch():
    import sys
    sys.path.insert(0, ROOT)
    from weavess_gb300.replicas import query_slice
    for nq in (0, 1, 7, 10, 1000, 1001):
        for world in (1, 2, 3, 8):
            spans = [query_slice(nq, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == nq
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(e - s for s, e in spans) - min(e - s for s, e in spans) <= 1


def _shard_worker(r, port, q):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.update(RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=r, world_size=2)
    import oracle as O
    from weavess_gb300 import datasets as ds
    from weavess_gb300.replicas import sharded_search, torch_gather
    base, query = ds.int_mixture(3000, 32, 8, seed=5, n_query=101)
    rnd = O.Rand(1)
    g = O.nndescent(base, O.init_random(base, 10, rnd), 10, 16, 32, 4, 40, rnd)
    # each rank: its own replica of the index, its own rand stream from seed 3
    mine = O.Rand(3)
    ids, dc, hc = sharded_search(lambda qq: O.search(base, qq, g, 40, mine), query, r, 2,
                                 skip_rand=lambda k: mine.take(k), gather=torch_gather)
    q.put((r, ids, dc, hc))
    dist.destroy_process_group()


def test_sharded_search_over_two_gloo_ranks_equals_one_replica():
    """Two ranks each search a slice of the batch on their own replica (the
    oracle's route here), their rand streams advanced to the slice's first
    query; the gathered ids, in query order, and the summed counters equal
    one replica's search of the whole batch."""
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import torch.multiprocessing as mp
    import oracle as O
    from weavess_gb300 import datasets as ds
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_shard_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted((q.get(timeout=180) for _ in ps), key=lambda t: t[0])
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    base, query = ds.int_mixture(3000, 32, 8, seed=5, n_query=101)
    rnd = O.Rand(1)
    g = O.nndescent(base, O.init_random(base, 10, rnd), 10, 16, 32, 4, 40, rnd)
    want, wdc, whc = O.search(base, query, g, 40, O.Rand(3))
    for r, ids, dc, hc in out:
        assert np.array_equal(ids, want), r
        assert (dc, hc) == (wdc, whc)
