"""Replica runs over several GPUs of one node: one process per GPU, each with
its own independent replica batch (the Monte Carlo chains do not shard: one
chain is sequential, so ranks exchange nothing on the data path). The only
collective is the timing one: the job's rate is the units all ranks
processed over the slowest rank's time.

Used by bench.py under torchrun (NCCL); the same functions run on CPU with
the gloo backend in the tests."""
from __future__ import annotations


def replica_seed(rank: int, base: int = 77) -> int:
    """Seed of a rank's replica batch: ranks draw disjoint streams (each
    replica of the batch then gets its own from the batch's seed)."""
    return 1000 * rank + base


def job_rate(step_ms: float, units_per_rank_step: float, world: int = 1, dist=None,
             device: str = "cuda"):
    """(units per second of the whole job, the slowest rank's step time in
    ms): step times are reduced with MAX over the ranks, so every rank
    returns the same numbers."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(step_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    return world * units_per_rank_step / (step_ms / 1e3), step_ms
