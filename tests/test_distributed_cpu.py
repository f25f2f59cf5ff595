"""The N>1 plumbing of bench.py on CPU with the gloo backend, world size 2:
instance sharding is a partition, and the elapsed time reported is the max
over ranks (the contract's timing rule).  No GPU involved."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    import torch
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    mine = list(bench.shard(4096, rank, ws))
    gathered = [None] * ws
    dist.all_gather_object(gathered, mine)
    bench.barrier(ws)
    t = bench.max_over_ranks(1.0 + rank, ws)
    out[rank] = (gathered, t)
    dist.destroy_process_group()


def test_shards_and_max_over_ranks():
    ws = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_worker, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
    for r in range(ws):
        gathered, t = out[r]
        assert t == float(ws)  # max over ranks
        flat = sorted(i for part in gathered for i in part)
        assert flat == list(range(4096))
        assert abs(len(gathered[0]) - len(gathered[1])) <= 1


@pytest.mark.parametrize("n,ws", [(0, 2), (5, 3), (4096, 7), (3, 8)])
def test_shard_partition(n, ws):
    import bench
    parts = [list(bench.shard(n, r, ws)) for r in range(ws)]
    assert sorted(i for p in parts for i in p) == list(range(n))
    assert max(map(len, parts)) - min(map(len, parts)) <= 1
