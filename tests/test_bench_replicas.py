"""Host logic of bench.py's N-GPU path (replicas: no data-path collective),
run as two gloo ranks on the CPU.

Under torchrun every rank solves its own copy of the workload; the job's
time is the slowest rank's (a MAX over ranks after a barrier) and its rate
the units of all ranks over that time.  The reference arm runs on rank 0
alone: the other ranks return without work."""
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port):
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        # each rank's own timings: rank r is slower on the first, faster on
        # the second; the job sees the slowest of each
        got = bench.ranks_max([1.0 + rank, 5.0 - rank], dist, "cpu")
        assert got == [float(world), 5.0], got
        bench.ranks_barrier(dist)
        # rate of the whole job: every rank did 10 steps within 2.0 s
        assert bench.replica_rate(world, 10, 2.0) == world * 5.0
        # the reference arm: only rank 0 works (args untouched elsewhere)
        if rank != 0:
            assert bench.run_reference(types.SimpleNamespace(), rank) is None
        bench.ranks_barrier(dist)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(2, _free_port()), nprocs=2, join=True,
                       start_method="spawn")


def test_single_process_values_pass_through():
    import bench
    assert bench.ranks_max([3.5, 1.25], None, "cpu") == [3.5, 1.25]
    bench.ranks_barrier(None)
    assert bench.replica_rate(1, 20, 0.5) == pytest.approx(40.0)
