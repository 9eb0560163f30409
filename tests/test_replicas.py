"""The multi-rank path of the bench and of batched sweeps (replicas only: one
process per GPU, no data exchange), as world_size-2 gloo process groups on
the CPU: the units shard without overlap or gap, every rank sees the
slowest rank's time and the summed work, and a sweep's instances split by
rank are exactly the single-process list."""

import socket
import time

import numpy as np
import pytest
import torch.multiprocessing as mp

from blademaster_gb300 import replicas


def test_shard_partitions_every_count():
    for count in (0, 1, 7, 256, 1001):
        for world in (1, 2, 3, 8):
            ranges = [replicas.shard(count, r, world) for r in range(world)]
            seen = [i for r in ranges for i in r]
            assert seen == list(range(count))
            sizes = [len(r) for r in ranges]
            assert max(sizes) - min(sizes) <= (1 if count else 0)
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    import os

    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    d, r, w, local = replicas.init("gloo")
    try:
        assert (r, w, local) == (rank, world, rank)
        replicas.barrier(d)
        slowest = replicas.max_over_ranks(d, 1.5 + rank)  # this rank's "time"
        total = replicas.sum_over_ranks(d, 100 * (rank + 1))  # this rank's "work"
        from blademaster_gb300.sweep import instances

        everything = instances(6, seed=0)
        mine = [everything[i] for i in replicas.shard(len(everything), rank, world)]
        spacings = replicas.sum_over_ranks(d, sum(i.config.grid_spacing for i in mine))
        results[rank] = (slowest, total, spacings, sum(i.config.grid_spacing for i in everything))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_total_and_shard_a_sweep():
    world, port = 2, _free_port()
    manager = mp.get_context("spawn").Manager()
    results = manager.dict()
    ctx = mp.start_processes(_rank_main, args=(world, port, results), nprocs=world, join=False, start_method="spawn")
    deadline = time.monotonic() + 120
    while not ctx.join(timeout=5):  # re-raises a rank's exception
        if time.monotonic() > deadline:
            for process in ctx.processes:  # only the two ranks this test started
                process.terminate()
            pytest.fail("the gloo ranks did not finish within 120 s")
    for rank in range(world):
        slowest, total, spacings, expected = results[rank]
        assert slowest == 2.5
        assert total == 300.0
        np.testing.assert_allclose(spacings, expected, rtol=1e-12)
