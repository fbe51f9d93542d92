"""Multi-process host logic of bench.py on CPU (gloo, world size 2): the
max-over-ranks timing reduction and the per-rank sharding of the ragged
workload (each rank its own seeded systems, no data-path collective)."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from lineax_gb300 import workloads

        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 5.0], world, "cpu")
        n, k = workloads.ragged_spd_sizes(bench.SEED + rank, 64)
        q.put((rank, got, n[:8], k[:8]))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_sharding_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = {r: (g, n, k) for r, g, n, k in out}
    for r in range(world):
        assert res[r][0] == [2.0, 10.0, 5.0]
    # different seeded systems per rank (weak scaling: per-rank work is fixed)
    assert (res[0][1], res[0][2]) != (res[1][1], res[1][2])


def test_max_over_ranks_single_process_is_identity():
    import bench

    assert bench.max_over_ranks([3.0, 4.5], 1, "cpu") == [3.0, 4.5]


def _worker_solve(rank, world, port, q):
    """Each rank solves its own shard of the ragged workload (the oracle's
    Cholesky on the CPU stands in for the GPU kernel); the units and the worst
    backward error are combined with the same all-reduces the bench uses."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import numpy as np

        import bench
        from lineax_gb300 import workloads
        from oracle import dense

        count = 10
        wl = workloads.ragged_spd(bench.SEED + rank, count)
        worst, ao, bo = 0.0, 0, 0
        for n, k in zip(wl.n, wl.nrhs):
            a = wl.a[ao: ao + n * n].reshape(n, n)
            b = wl.b[bo: bo + n * k].reshape(k, n)
            x = dense.cholesky_linear_solve(a, b.T).T
            worst = max(worst, float(dense.backward_errors_exact(a, x, b).max()))
            ao += n * n
            bo += n * k
        units = torch.tensor([float(count)])
        dist.all_reduce(units, op=dist.ReduceOp.SUM)
        t = bench.max_over_ranks([0.5 + 0.25 * rank, worst], world, "cpu")
        first = float(np.asarray(wl.a[:16]).sum())
        q.put((rank, float(units.item()), t, first))
    finally:
        dist.destroy_process_group()


def test_sharded_solve_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_solve, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = {r: (u, t, f) for r, u, t, f in out}
    for r in range(world):
        units, (slowest, worst), _ = res[r]
        assert units == 10.0 * world          # every rank's systems counted once
        assert slowest == 0.75                # whole-job time = the slowest rank
        assert worst <= 1e-12                 # every shard solved to the bar
    assert res[0][2] != res[1][2]             # the shards hold different systems
