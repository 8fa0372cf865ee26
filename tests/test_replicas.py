"""Replicas on several GPUs, host side: two gloo ranks on CPU.

Each rank times its own replica; the job's rate is the units of all ranks over
the slowest rank's time.  A request stream is split round-robin, each rank
serves its share with its own scheduler, and the completed counts add up to
the whole stream with no request served twice."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from code_mge_gb300 import replicas as R


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, nranks, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=nranks)
    try:
        from code_mge_gb300 import serving as S
        res = {}
        assert R.world() == (rank, nranks)
        # timing: rank r took 1 + r seconds for 10 * (r + 1) units
        res["max"] = R.max_over_ranks(1.0 + rank)
        res["rate"] = R.whole_job_rate(10.0 * (rank + 1), 1.0 + rank)
        R.barrier()
        # a request stream split across the ranks
        reqs = S.poisson_requests(4.0, 3.0, sizes=(16, 24), tol=1e-3, max_cycles=60)
        for r in reqs:
            r.arrival = 0.0
        mine = R.shard(reqs)
        clock = iter(range(1 << 30))
        srv = S.Server(S.FakeBackend(rate=0.5, latency=1), reserve_bytes=0,
                       clock=lambda: 1e-3 * next(clock))
        for r in mine:
            srv.submit(r)
        done = srv.run(idle_sleep=0)
        res["total"] = len(reqs)
        res["mine"] = sorted(r.rid for r in done)
        res["completed_all"] = R.sum_over_ranks(len(done))
        out.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_and_serve_as_replicas():
    nranks = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, nranks, port, q)) for r in range(nranks)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(nranks))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(nranks):
        assert got[r]["max"] == 2.0
        assert got[r]["rate"] == pytest.approx((10.0 + 20.0) / 2.0)
        assert got[r]["completed_all"] == got[r]["total"]
    a, b = set(got[0]["mine"]), set(got[1]["mine"])
    assert not (a & b)
    assert len(a | b) == got[0]["total"]


def test_shard_is_round_robin_and_covers_everything():
    items = list(range(11))
    parts = [R.shard(items, r, 3) for r in range(3)]
    assert parts[0] == [0, 3, 6, 9] and parts[1] == [1, 4, 7, 10] and parts[2] == [2, 5, 8]
    assert sorted(sum(parts, [])) == items


def test_without_a_group_the_helpers_are_identities():
    assert R.world() == (0, 1)
    assert R.max_over_ranks(3.5) == 3.5
    assert R.whole_job_rate(12.0, 4.0) == 3.0
    assert R.shard([1, 2, 3]) == [1, 2, 3]
