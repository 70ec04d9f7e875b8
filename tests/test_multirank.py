"""The N > 1 path on CPU: two gloo ranks, each with its own seeded shard of the
batched uneven workload, integrated by the oracle (the GPU path shards the same
way). Checks that the aggregated step count and the summed parameter
gradients equal a single process doing both shards, and that the time is the
maximum over ranks."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from oracle import oracle as O


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard_work(rank: int, n: int):
    from galax_gb300 import shard
    from galax_gb300 import workloads as W

    b = W.uneven_ics(lambda x: O.gradient(O.milky_way(), x), n, seed=shard.shard_seed(1, rank), tmax=300.0,
                     smax=20)
    grids = [b.save_ts[b.save_offsets[i]:b.save_offsets[i + 1]] for i in range(n)]
    _, st, acc, _ = O.integrate(O.milky_way(), b.y0, b.t0, b.t1, grids,
                                O.solver_cfg(5, True, rtol=1e-8, atol=1e-10), nthreads=1)
    y0 = b.y0[:4]
    yT, *_ = O.integrate(O.milky_way(), y0, 0.0, 20.0, np.array([20.0]), O.solver_cfg(8, False, dt0=1.0))
    target = np.stack([s[-1] for s in yT]) + 0.01
    _, _, gp, _ = O.adjoint_fixed(O.milky_way(), y0, 0.0, 20.0, target, O.solver_cfg(8, False, dt0=1.0))
    return int(acc.sum()), gp


def _worker(rank, world, port, n, q):
    import torch
    import torch.distributed as dist

    from galax_gb300 import shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        steps, gp = _shard_work(rank, n)
        units, ms = shard.aggregate(dist, steps, 10.0 * (rank + 1))
        g = shard.sum_param_grads(dist, torch.as_tensor(gp))
        dist.barrier()
        if rank == 0:
            q.put((units, ms, g.numpy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_match_one_process():
    world, n = 2, 24
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        units, ms, g = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    ref = [_shard_work(r, n) for r in range(world)]
    assert units == sum(r[0] for r in ref)
    assert ms == pytest.approx(10.0 * world)
    np.testing.assert_allclose(g, ref[0][1] + ref[1][1], rtol=1e-12)


def test_aggregate_without_a_group_is_the_identity():
    from galax_gb300 import shard

    assert shard.aggregate(None, 7, 3.5) == (7.0, 3.5)
    assert shard.shard_seed(1, 0) == 1 and shard.shard_seed(1, 3) == 4
