"""bench.py's N > 1 path on CPU: two gloo ranks, each timing its own replica;
the job is timed by the slowest rank and counts the particles of all ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank          # rank 1 is the slow replica
    ms = bench.max_over_ranks(local_ms, world, "cpu")
    value = bench.replica_throughput(1000, 10, ms, world)
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_replica():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert res[0][1] == pytest.approx(2 * 1000 * 10 / 0.150)


def test_single_rank_is_identity():
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replica_throughput(4096000, 500, 379.0, 1) == pytest.approx(4096000 * 500 / 0.379)
