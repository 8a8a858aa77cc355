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


def _shard_worker(rank, world, port, out):
    """Each rank evaluates its shard of a batch of independent structures (FP64 oracle) and
    the shards' energies and forces are gathered on every rank."""
    import numpy as np
    from jse_gb300 import workloads as W
    from oracle import model as OM, native as ON
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        structs = W.c4_structures(count=10, seed=13)
        pm = OM.load(W.model_for("c4"))
        ids = shard(list(range(len(structs))), rank, world)
        mine = {k: ON.compute(pm, structs[k].x, structs[k].types, structs[k].box_kind, structs[k].box)
                for k in ids}
        mine = {k: (v["energy"], np.asarray(v["forces"])) for k, v in mine.items()}
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        if rank == 0:
            out["all"] = {k: v for part in gathered for k, v in part.items()}
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_a_batch_like_one_rank():
    """Sharding a batch of independent structures over two ranks evaluates every structure
    once and gives exactly the single-process results (no data collective is involved)."""
    import numpy as np
    from jse_gb300 import workloads as W
    from oracle import model as OM, native as ON
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_shard_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    got = dict(out["all"])
    structs = W.c4_structures(count=10, seed=13)
    pm = OM.load(W.model_for("c4"))
    assert sorted(got) == list(range(len(structs)))
    for k, s in enumerate(structs):
        r = ON.compute(pm, s.x, s.types, s.box_kind, s.box)
        assert got[k][0] == r["energy"]
        assert np.array_equal(got[k][1], r["forces"])
