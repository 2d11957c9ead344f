"""Replica runs over several ranks (plum_gb300/replicas.py, used by bench.py
under torchrun): two gloo ranks on CPU. Each rank's replica batch gets its
own seed, and the job's rate is the units of all ranks over the slowest
rank's step time, the same on every rank."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from plum_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r takes (r + 1) * 10 ms per step of 64 replicas x 256 steps
    rate, ms = replicas.job_rate(10.0 * (rank + 1), 64 * 256, world, dist, device="cpu")
    out.put((rank, replicas.replica_seed(rank), rate, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_share_the_slowest_step():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (r0, s0, v0, m0), (r1, s1, v1, m1) = got
    assert s0 != s1
    assert m0 == m1 == pytest.approx(20.0)
    assert v0 == v1 == pytest.approx(2 * 64 * 256 / 0.020)


def test_single_rank_rate():
    from plum_gb300 import replicas
    rate, ms = replicas.job_rate(50.0, 1000)
    assert ms == 50.0 and rate == pytest.approx(20000.0)
