"""Sharding orbits across GPUs (one process per GPU).

Orbits are independent, so N ranks integrate N disjoint shards with no
exchange on the data path (weak scaling: every rank its own seeded shard).
Only three host-level reductions exist: the step (or gradient) count summed
over ranks, the step time maximised over ranks, and, for differentiation with
respect to potential parameters, the per-shard parameter gradients summed
(galax would differentiate one batched solve; here the batch is split and the
parameter cotangents add). All three go through ``torch.distributed`` on
whatever backend the process group uses (NCCL on GPUs, gloo on CPU).
"""

from __future__ import annotations

SEED_STRIDE = 1


def shard_seed(base_seed: int, rank: int) -> int:
    """Seed of a rank's shard: shards are disjoint draws of the same distribution."""
    return base_seed + SEED_STRIDE * rank


def aggregate(dist, local_units: float, local_ms: float, device="cpu") -> tuple[float, float]:
    """(units summed over ranks, time maximised over ranks); identity without a group."""
    if dist is None:
        return float(local_units), float(local_ms)
    import torch

    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u), float(t)


def sum_param_grads(dist, grad_params):
    """Sum per-shard parameter gradients (ncomp, 3) over ranks, in place."""
    if dist is None:
        return grad_params
    dist.all_reduce(grad_params, op=dist.ReduceOp.SUM)
    return grad_params
