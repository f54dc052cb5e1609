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
