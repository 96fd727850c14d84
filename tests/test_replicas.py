"""The replica scale-out's host logic on CPU: world_size 2 over gloo."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _allreduce(values, op):
    t = torch.tensor(values, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return t.tolist()


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "kagomedsl.jl_gb300"))
    from kagomevmc import replicas

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, count = replicas.shard(2049, rank, world)
    seed = replicas.replica_seed(7, rank)
    ms, tot = replicas.reduce_run(10.0 + rank, {"accepted": 100 * (rank + 1), "walkers": count}, _allreduce)
    out[rank] = (first, count, seed, ms, tot["accepted"], tot["walkers"])
    dist.destroy_process_group()


def test_two_rank_reduction_and_sharding():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    r0, r1 = out[0], out[1]
    assert (r0[0], r0[1]) == (0, 1025) and (r1[0], r1[1]) == (1025, 1024)
    assert r0[2] != r1[2]
    for r in (r0, r1):
        assert r[3] == 11.0            # slowest rank's time
        assert r[4] == 300.0           # summed accepted moves
        assert r[5] == 2049.0          # every walker counted once


def test_single_process_passthrough():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "kagomedsl.jl_gb300"))
    from kagomevmc import replicas

    assert replicas.reduce_run(3.0, {"a": 2}) == (3.0, {"a": 2.0})
    assert replicas.shard(10, 0, 1) == (0, 10)
