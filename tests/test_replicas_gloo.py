"""The multi-GPU form of the path on two CPU ranks (gloo): replicas need no data
collective, only a barrier, the maximum of the ranks' times and the whole-job rate;
sharding a batch of independent structures covers every structure exactly once."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from jse_gb300.replicas import barrier, max_over_ranks, shard, whole_job_rate  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        barrier(dist)
        t = max_over_ranks(1.0 + rank, dist)          # rank r took 1 + r seconds
        mine = shard(list(range(10)), rank, world)
        sizes = torch.tensor([len(mine)])
        dist.all_reduce(sizes)
        out[rank] = (t, whole_job_rate(1000, 5, world, t), mine, int(sizes[0]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_rate_and_shards():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    assert sorted(out.keys()) == [0, 1]
    for r in range(world):
        t, rate, mine, total = out[r]
        assert t == 2.0                                 # the slowest rank sets the time
        assert rate == pytest.approx(1000 * 5 * 2 / 2.0)
        assert total == 10
    assert sorted(out[0][2] + out[1][2]) == list(range(10))


def test_single_process_needs_no_group():
    assert max_over_ranks(3.5) == 3.5
    assert shard([1, 2, 3], 0, 1) == [1, 2, 3]
    with pytest.raises(ValueError):
        shard([1], 2, 2)
