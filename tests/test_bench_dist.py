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
